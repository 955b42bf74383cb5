/* gbcomb -- GB300-native node-local sparse kernels for CombBLAS.
 *
 * C ABI of the shared library built from combblas_gb300/csrc (libgbcomb.so).
 * Plain pointers and sizes only.  Every entry point returns an int status
 * (GBC_OK = 0, negative on error; gbc_last_error() gives the message).
 *
 * Matrices are column-compressed with int64 indices, exactly the arrays the
 * reference keeps:
 *   DCSC (SpDCCols/Dcsc, dcsc.h:125-131): cp[nzc+1], jc[nzc] (ids of the
 *        nonempty columns, ascending), ir[nnz] (row ids, ascending within a
 *        column), numx[nnz];
 *   CSC  (SpCCols/Csc, csc.h:70-74): jc == NULL, cp has ncol+1 entries.
 * Inputs may live in host memory (copied to the device inside the call) or
 * device memory (GBC_DEVICE); results stay on the device and are copied out
 * with gbc_result_copy().
 */
#ifndef GBCOMB_H
#define GBCOMB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GBC_OK 0
#define GBC_EINVAL (-1)      /* bad argument or malformed matrix */
#define GBC_ENOMEM (-2)      /* device allocation failed */
#define GBC_ECUDA (-3)       /* CUDA runtime error */
#define GBC_EOVERFLOW (-4)   /* a size exceeds what the kernels index */
#define GBC_ETIMEOUT (-5)    /* a bounded device wait gave up */
#define GBC_EUNSUPPORTED (-6)

/* where a matrix's arrays live */
#define GBC_HOST 0
#define GBC_DEVICE 1

/* semirings (Semirings.h and the applications' own) */
#define GBC_SR_PLUSTIMES 0    /* PlusTimesSRing (Semirings.h:212-232) */
#define GBC_SR_MINPLUS 1      /* MinPlusSRing (Semirings.h:235-255) */
#define GBC_SR_SELECT2NDMIN 2 /* Select2ndMinSR (Applications/FastSV.h:25-44) */
#define GBC_SR_BOOL 3         /* PlusTimesSRing<bool,bool>: or / and */
#define GBC_SR_SELECT2ND 4    /* Select2ndSRing (Semirings.h:144-163): add keeps its second argument */
#define GBC_SR_SELECTMAX 5    /* SelectMaxSRing<bool,T> (Semirings.h:192-210): add = max */

/* value types */
#define GBC_F64 0
#define GBC_F32 1
#define GBC_I64 2
#define GBC_BOOL 3 /* 1 byte, 0 or 1 */

/* output row order inside a column */
#define GBC_SORTED 1   /* LocalHybridSpGEMM / LocalSpGEMMHash(sort=true) */
#define GBC_UNSORTED 0 /* LocalSpGEMMHash(sort=false); this library still sorts */

/* sizing mode of the SpGEMM */
#define GBC_SIZING_EXACT 0   /* symbolic pass + numeric pass (two-phase) */
#define GBC_SIZING_LEARNED 1 /* MLP-predicted capacities, overflow re-run exactly */

/* accumulation of PlusTimes fp64 products (gbc_context_set_fold) */
#define GBC_FOLD_EXACT 0   /* exact sum of the rounded products, rounded once (default) */
#define GBC_FOLD_ORDERED 1 /* left fold in B-entry order, the reference's hash path bit for bit */

typedef struct gbc_context gbc_context;
typedef struct gbc_result gbc_result;

typedef struct {
    int64_t nrow, ncol; /* global dimensions */
    int64_t nzc;        /* number of stored columns (== ncol for CSC) */
    int64_t nnz;
    const int64_t *cp;  /* [nzc+1] */
    const int64_t *jc;  /* [nzc] column ids, or NULL for CSC */
    const int64_t *ir;  /* [nnz] */
    const void *num;    /* [nnz] values, or NULL for an all-ones pattern */
    int where;          /* GBC_HOST or GBC_DEVICE */
} gbc_matrix;

typedef struct {
    int sizing;      /* GBC_SIZING_EXACT / GBC_SIZING_LEARNED */
    int sorted;      /* GBC_SORTED / GBC_UNSORTED */
    int keep_empty;  /* 1: one output column per stored column of B (SpTuples
                        view); 0: drop empty output columns (SpDCCols view) */
    int tile_rows;   /* rows of the block kernel's accumulator tile: 0 = 4096
                        up to 2^18 rows of A and 8192 above (4096 for PlusTimes
                        fp64 under the exact fold), or 4096 / 8192 / 16384
                        (at most 8192 under the exact fold) */
    int64_t tiny_limit;  /* columns with <= this many multiplications use the
                            smallest warp kernel (<= 256; -1 = default 256) */
    int64_t small_limit; /* ... <= this many the larger warp kernels (<= 4096;
                            -1 = default: 4096, or 1024 for PlusTimes fp64 under
                            the exact fold); above it the block kernel */
} gbc_spgemm_opts;

typedef struct {
    int64_t flops;          /* sum over columns of estimateFLOP */
    int64_t nnz;            /* nnz(C) */
    int64_t overflow_cols;  /* learned sizing: columns re-run exactly */
    int64_t alloc_entries;  /* entries allocated for C before trimming */
    double ms_total;        /* device time of the call (CUDA events) */
    double ms_symbolic;
    double ms_numeric;
    int64_t tile_visits_dense; /* exact-fold big columns: (column, row tile) visits through the
                                  dense accumulator (gbc_spgemm only; 0 otherwise) */
    int64_t tile_visits_range; /* ... and runs of light tiles summed through a sorted range */
} gbc_spgemm_stats;

/* ---------------------------------------------------------------- context */
int gbc_context_create(gbc_context **ctx, int device);
int gbc_context_destroy(gbc_context *ctx);
/* Use an existing cudaStream_t (passed as void*); NULL selects the
 * context's own stream. */
int gbc_context_set_stream(gbc_context *ctx, void *stream);
/* How PlusTimes fp64 products are summed into an output entry.  The
 * reference folds them as acc = add(product, acc) over the B column's entries
 * in order (mtSpGEMM.h:396-412).  GBC_FOLD_ORDERED reproduces that fold bit
 * for bit.  GBC_FOLD_EXACT (the default) adds the same rounded products
 * exactly and rounds the sum once to the nearest double: independent of any
 * order, identical on every run, and within the reference's own rounding
 * error of its result.  A column whose products span more than 61 binades,
 * or whose values include subnormal, infinite or NaN entries, keeps the
 * ordered fold. */
int gbc_context_set_fold(gbc_context *ctx, int fold);
int gbc_context_synchronize(gbc_context *ctx);
const char *gbc_last_error(void);
int gbc_version(void);
/* Number of CUDA kernels this library has launched in this process. */
int64_t gbc_launch_count(void);

/* ------------------------------------------------------------------ result */
/* A result is a device matrix owned by the library until gbc_result_free. */
int gbc_result_info(const gbc_result *r, int64_t *nrow, int64_t *ncol, int64_t *nzc, int64_t *nnz, int *valtype);
/* Copy out; cp[nzc+1], jc[nzc], ir[nnz], num[nnz].  Any pointer may be NULL.
 * `where` says whether the destination buffers are host or device memory. */
int gbc_result_copy(const gbc_result *r, int64_t *cp, int64_t *jc, int64_t *ir, void *num, int where);
/* Device pointers of the result arrays (valid until gbc_result_free). */
int gbc_result_device_ptrs(const gbc_result *r, const int64_t **cp, const int64_t **jc, const int64_t **ir,
                           const void **num);
int gbc_result_free(gbc_result *r);

/* ------------------------------------------------------------------ SpGEMM */
/* C = A * B over semiring `sr` with value type `vt` (A and B share it).
 * Replaces LocalHybridSpGEMM<SR,NTO>(const SpDCCols&, const SpDCCols&,
 * clearA, clearB, aux) (mtSpGEMM.h:213-217), its CSC overload
 * (mtSpGEMM.h:1148-1152), LocalSpGEMM (mtSpGEMM.h:74-78) and
 * LocalSpGEMMHash(..., sort) (mtSpGEMM.h:463-467): same product, rows
 * ascending within each output column. */
int gbc_spgemm(gbc_context *ctx, int sr, int vt, const gbc_matrix *A, const gbc_matrix *B,
               const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *stats);

/* Per-semiring, per-type instantiations of gbc_spgemm (int64 indices). */
int gbc_spgemm_plustimes_f64_i64(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B,
                                 const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *stats);
int gbc_spgemm_plustimes_f32_i64(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B,
                                 const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *stats);
int gbc_spgemm_plustimes_i64_i64(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B,
                                 const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *stats);
int gbc_spgemm_minplus_f64_i64(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B,
                               const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *stats);
int gbc_spgemm_minplus_i64_i64(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B,
                               const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *stats);
int gbc_spgemm_select2ndmin_i64_i64(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B,
                                    const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *stats);
int gbc_spgemm_bool_i64(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B, const gbc_spgemm_opts *opts,
                        gbc_result **C, gbc_spgemm_stats *stats);

/* Column-phased product for outputs larger than device memory: B's stored
 * columns are split into phases whose output holds at most max_phase_nnz
 * entries, as the phases of MemEfficientSpGEMM (ParFriends.h:553-556,
 * SpDCCols::ColSplit).  Each phase's C is produced in HBM and reduced to
 * checksums; the product itself is not returned.  sizing = GBC_SIZING_EXACT
 * cuts phases on the symbolic counts; GBC_SIZING_LEARNED cuts them on the
 * context's sizing model's capacities and recomputes overflowing columns
 * exactly, so nnz, row_checksum and content_hash are the same either way. */
typedef struct {
    int64_t flops;
    int64_t nnz;
    int64_t phases;
    int64_t max_phase_nnz;  /* largest phase, in output slots */
    int64_t row_checksum;   /* sum of row ids of all entries */
    double val_checksum;    /* sum of values (double; rounding depends on the phase cuts) */
    uint64_t content_hash;  /* wrap-around sum of a 64-bit mix of (column, row, value bits) */
    int64_t overflow_cols;  /* learned: columns recomputed exactly */
    int64_t alloc_nnz;      /* output slots allocated over all phases (= nnz when exact) */
    double ms_total;
    double ms_sizing;       /* exact: symbolic pass; learned: features + MLP + capacities */
    double ms_numeric;      /* sum over phases of the numeric kernels */
    double ms_rerun;        /* learned: exact recomputation of overflowing columns */
} gbc_phased_stats;

int gbc_spgemm_phased(gbc_context *ctx, int sr, int vt, const gbc_matrix *A, const gbc_matrix *B,
                      int64_t max_phase_nnz, int sizing, gbc_phased_stats *st);

/* Sparse matrix x dense vector, y <- y (+) A x over semiring `sr`:
 * replaces dcsc_gespmv / dcsc_gespmv_threaded (Friends.h:63-175), whose row
 * update is SR::axpy(a, x[col], y[row]).  A plan holds A row-major on the
 * device (built once by a stable device radix sort); x (ncol) and y (nrow)
 * are where-located arrays of the plan's value type.  Rows without entries
 * keep y.  Min-type, boolean and integer semirings give the reference's
 * result exactly; PlusTimes on floating values sums each row in a fixed
 * order (repeatable, within rounding of the reference's column order). */
typedef struct gbc_spmv_plan gbc_spmv_plan;
int gbc_spmv_plan_create(gbc_context *ctx, int vt, const gbc_matrix *A, gbc_spmv_plan **plan);
int gbc_spmv_plan_destroy(gbc_spmv_plan *plan);
int gbc_spmv(gbc_context *ctx, const gbc_spmv_plan *plan, int sr, const void *x, void *y, int where);

/* Sum of nlists matrices of one shape (nrow x ncol), entries with the same
 * (row, column) combined with the semiring's add in list order: replaces
 * MultiwayMerge<SR>(vector<SpTuples*>&, mdim, ndim, delarrs)
 * (MultiwayMerge.h:428-708), which merges the outputs of several SUMMA
 * stages or column phases.  The result has one column per column of the
 * shape (SpTuples view), rows ascending. */
int gbc_multiway_merge(gbc_context *ctx, int sr, int vt, int nlists, const gbc_matrix *lists, int64_t nrow,
                       int64_t ncol, gbc_result **C, gbc_spgemm_stats *stats);

/* Symbolic helpers: per stored column of B, flop = estimateFLOP
 * (mtSpGEMM.h:1057-1134) and nnz = estimateNNZ_Hash (mtSpGEMM.h:806-933).
 * Output arrays have B->nzc entries and live where `where` says. */
int gbc_spgemm_colstats(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B, int64_t *flop, int64_t *nnz,
                        int where);

/* ----------------------------------------------------------------- batches */
/* Many independent products C_p = A_p * B_p (uneven sizes) computed
 * together: every pass is one launch over the columns of all products, and
 * the symbolic + scan + numeric passes are captured once into a CUDA graph
 * that gbc_batch_run replays.  s1/s2 (-1: defaults 256/4096) are the flop
 * thresholds of the warp-kernel column classes, the knobs the autotuner
 * picks.  The batch owns copies of host inputs; device inputs must outlive
 * it.  No counterpart in the reference, which multiplies one pair at a time
 * (PSpGEMM, SpParMat.h:464). */
typedef struct gbc_batch gbc_batch;
int gbc_batch_create(gbc_context *ctx, int sr, int vt, int nprob, const gbc_matrix *A, const gbc_matrix *B,
                     int64_t s1, int64_t s2, gbc_batch **out);
int gbc_batch_run(gbc_batch *b, double *ms);
int gbc_batch_info(const gbc_batch *b, int p, int64_t *nzc, int64_t *nnz, int64_t *flops);
int gbc_batch_result(const gbc_batch *b, int p, int64_t *cp, int64_t *ir, void *num, int where);
int gbc_batch_destroy(gbc_batch *b);

/* -------------------------------------------------------- learned sizing */
/* The sizing model: a 6-32-32-1 MLP that predicts log2(1 + nnz) of each
 * output column from per-column features (no counterpart in the reference,
 * which always runs the exact symbolic pass estimateNNZ_Hash).  Trained and
 * evaluated by the library's own GPU kernels.  With GBC_SIZING_LEARNED the
 * predicted capacity replaces the symbolic pass; columns that overflow it are
 * recomputed exactly, so results are identical to GBC_SIZING_EXACT. */
typedef struct gbc_mlp gbc_mlp;
#define GBC_MLP_FEATURES 6
int gbc_mlp_create(gbc_context *ctx, uint64_t seed, gbc_mlp **m);
int gbc_mlp_destroy(gbc_mlp *m);
/* number of floats in the parameter block of gbc_mlp_get / gbc_mlp_set */
int gbc_mlp_num_params(void);
int gbc_mlp_get(gbc_mlp *m, float *params, float *margin);
int gbc_mlp_set(gbc_mlp *m, const float *params, float margin);
/* Full-batch Adam on (features [n x 6], targets log2(1 + nnz) [n]). */
int gbc_mlp_train(gbc_context *ctx, gbc_mlp *m, const float *feat, const float *target, int64_t n, int steps, float lr,
                  float *loss, int where);
/* grad[num params of the network + 1]: mean-squared-error gradient at the
 * current parameters, then the loss (checks the backward kernels). */
int gbc_mlp_gradient(gbc_context *ctx, gbc_mlp *m, const float *feat, const float *target, int64_t n, float *grad,
                     int where);
int gbc_mlp_predict(gbc_context *ctx, gbc_mlp *m, const float *feat, int64_t n, float *pred, int where);
/* Model used by GBC_SIZING_LEARNED on this context (NULL clears it). */
int gbc_context_set_mlp(gbc_context *ctx, gbc_mlp *m);
/* Per stored column of B: features [nzc x 6], flop, and (when nnz != NULL)
 * the exact nnz from the symbolic pass -- the model's training data. */
int gbc_spgemm_features(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B, float *feat, int64_t *flop,
                        int64_t *nnz, int where);

/* ------------------------------------------------------------------- MCL */
/* Prune and select of one MCL expansion step on a device fp32 result:
 * MCLPruneRecoverySelect with recoverNum == 0 (ParFriends.h:185-354) and
 * Kselect1 (SpParMat.cpp:1191-1300).  A column whose count of entries
 * > thr exceeds `select` keeps its entries >= the select-th largest value of
 * the whole column (ties kept); every other column keeps entries >= thr.
 * Entry order within a column is preserved.  *out is a new result. */
int gbc_mcl_prune_select_f32(gbc_context *ctx, const gbc_result *C, float thr, int64_t select, gbc_result **out);
/* One MCL expansion step as MemEfficientSpGEMM(A, A, phases=1, thr, select,
 * recoverNum=0, ..., computationKernel=1) runs it (ParFriends.h:452): C =
 * A*A over PlusTimes fp32, then the prune/select above.  sizing is
 * GBC_SIZING_EXACT or GBC_SIZING_LEARNED; stats describe the SpGEMM. */
int gbc_mcl_expand_f32(gbc_context *ctx, const gbc_matrix *A, float thr, int64_t select, int sizing, gbc_result **out,
                       gbc_spgemm_stats *stats);
/* The same two steps with recovery (recoverNum > 0, ParFriends.h:290-330):
 * a column left with fewer than recover_num entries > thr whose kept sum is
 * below recover_pct takes back its entries >= the recover_num-th largest
 * value (Kselect1 over the sparse column, SpParMat.cpp:1411-1690: the
 * column's smallest value when it holds fewer, FLT_MIN when empty).  Column
 * sums here are exact sums of the kept values rounded once to fp32, so they
 * do not depend on the entries' storage order.  recover_num == 0 gives the
 * calls above. */
int gbc_mcl_prune_select_recover_f32(gbc_context *ctx, const gbc_result *C, float thr, int64_t select,
                                     int64_t recover_num, float recover_pct, gbc_result **out);
int gbc_mcl_expand_recover_f32(gbc_context *ctx, const gbc_matrix *A, float thr, int64_t select, int64_t recover_num,
                               float recover_pct, int sizing, gbc_result **out, gbc_spgemm_stats *stats);
/* The MCL vector glue on a device fp32 result, in place (Applications/
 * MCL.cpp:389-449).  MakeColStochastic scales every column by 1 / (its sum),
 * FLT_MAX for a zero sum (safemultinv).  Inflate raises every value to
 * `power` (pow in double, rounded to fp32).  Chaos is the max over columns
 * of (column max - sum of squares) * nnz(column), at least 0; the column
 * sums are exact sums rounded once to fp32. */
int gbc_mcl_make_col_stochastic_f32(gbc_context *ctx, gbc_result *A);
int gbc_mcl_inflate_f32(gbc_context *ctx, gbc_result *A, double power);
int gbc_mcl_chaos_f32(gbc_context *ctx, const gbc_result *A, float *chaos);
/* The HipMCL iteration loop (MCL.cpp:526-626, one layer, one phase) on a
 * square fp32 matrix whose loops are already adjusted (AdjustLoops,
 * :463-473, is the caller's): MakeColStochastic; prune/select/recovery
 * once before the loop when nnz / n > max(select, recover_num); then, while
 * chaos > 0.0001: expansion with prune/select/recovery, MakeColStochastic,
 * Chaos, Inflate(inflation), MakeColStochastic.  max_iter > 0 caps the
 * iterations.  The matrix stays on the device between iterations; *out is
 * the converged matrix, *iterations and *chaos (either may be NULL) the
 * loop count and the last chaos. */
int gbc_mcl_iterate_f32(gbc_context *ctx, const gbc_matrix *A, double inflation, float thr, int64_t select,
                        int64_t recover_num, float recover_pct, int sizing, int64_t max_iter, gbc_result **out,
                        int64_t *iterations, float *chaos);

/* ------------------------------------------------------------ SpMSpV / BFS */
/* A square pattern matrix prepared once for repeated sparse-vector
 * multiplies and BFS (CSC, jc == NULL; values ignored). */
typedef struct gbc_graph gbc_graph;

typedef struct {
    int64_t iterations; /* level-loop iterations, as the reference's BFS loop counts them */
    int64_t reached;    /* vertices with a parent, plus the source */
    int64_t edges;      /* undirected edges of the reached vertices: sum(deg)/2 */
    double ms;          /* device time of the BFS */
    int64_t host_checks; /* host round trips inside the level loop: 0 when the
                            whole traversal ran as one graph (a while node) */
} gbc_bfs_stats;

int gbc_graph_create(gbc_context *ctx, const gbc_matrix *A, gbc_graph **g);
int gbc_graph_destroy(gbc_graph *g);
/* BFS direction policy: 0 (default) picks top-down or bottom-up per level
 * from the frontier and unreached edge counts; 1 always top-down (the
 * reference's SpMSpV formulation); 2 always bottom-up.  All three give the
 * same parents: a bottom-up step takes each vertex's first neighbour (rows
 * are ascending) in the frontier, which is the smallest one. */
int gbc_graph_set_policy(gbc_graph *g, int policy);

/* y = A x over SelectMinSR / Select2ndMinSR (add = min, multiply returns the
 * vector value): replaces SpMXSpV_Bucket<SR>(const Csc&, int32 mA, const
 * int32* indx, const IVT* numx, int32 veclen, vector<int32>& indy,
 * vector<OVT>& numy, PreAllocatedSPA&) (SpImpl.cpp:389-392, SpImpl.h:115-124).
 * indy/numy receive nnzy entries sorted by row; they must hold up to nrow
 * entries.  All four arrays live where `where` says. */
int gbc_spmspv_select2ndmin_i64(gbc_context *ctx, gbc_graph *g, const int32_t *indx, const int64_t *numx,
                                int32_t veclen, int32_t *indy, int64_t *numy, int32_t *nnzy, int where);

/* y = A x for any m x n matrix (CSC or DCSC, host or device) over the
 * semirings of the reference's SpMXSpV overload set (SpImpl.h:49-142).  The
 * plan copies A to the device once (for a numeric vt also row-major), so
 * repeated multiplies by one matrix move only the vectors.  sr:
 *   GBC_SR_SELECT2NDMIN  y(r) = min of the x values hitting r
 *                        (SpMXSpV_Bucket over SelectMinSR, SpImpl.cpp:389-699);
 *   GBC_SR_SELECT2ND     y(r) = the x value of the largest hitting column
 *                        (boolean SpMXSpV over Select2ndSRing, SpImpl.cpp:
 *                        167-328; TopDownBFS's path, BFSFriends.h:198-207);
 *   GBC_SR_SELECTMAX     y(r) = max of the hitting x values (SelectMaxSRing);
 *   GBC_SR_PLUSTIMES     y(r) = sum of A(r,c) * x(c), folded left in
 *                        ascending column order as SpMXSpV_Bucket's SPA does
 *                        (bit-exact); numeric plans only.
 * For the select semirings numx / numy are int64 and A's values are
 * ignored; for PlusTimes they have the plan's value type.  indx holds
 * distinct column ids (a repeated id is GBC_EINVAL).  indy / numy receive
 * nnzy entries sorted by row and must hold up to nrow entries; the vectors
 * live where `where` says. */
typedef struct gbc_spmspv_plan gbc_spmspv_plan;
int gbc_spmspv_plan_create(gbc_context *ctx, int vt, const gbc_matrix *A, gbc_spmspv_plan **plan);
int gbc_spmspv_plan_destroy(gbc_spmspv_plan *plan);
int gbc_spmspv_plan_info(const gbc_spmspv_plan *plan, int64_t *nrow, int64_t *ncol, int64_t *nnz);
int gbc_spmspv(gbc_context *ctx, gbc_spmspv_plan *plan, int sr, const int32_t *indx, const void *numx, int32_t veclen,
               int32_t *indy, void *numy, int32_t *nnzy, int where);

/* BFS from `source` by repeated SpMSpV with the per-level glue fused, as the
 * BFS_CSC loop of Applications/SpMSpV-IPDPS2017/SpMSpVBench.cpp:128-156:
 * parents[v] = smallest frontier neighbour that first reached v (-1 if
 * unreached; the source gets a parent only when a later level reaches it).
 * levels[v] = loop iteration (1-based) in which v first entered the fringe,
 * 0 for the source, -1 unreached.  Either output may be NULL. */
int gbc_bfs(gbc_context *ctx, gbc_graph *g, int64_t source, int64_t *parents, int64_t *levels, gbc_bfs_stats *st,
            int where);

/* Multi-source BFS: nroots BFS trees over the graph at once, the
 * Select2ndMin SpGEMM loop of the reference's multi-source traversals
 * (Applications/Ordering/MD.cpp:211-217 getReachesSPMM, BetwCent.cpp:185-186):
 * F_{l+1} = (A * F_l) masked by !visited, F's column r holding root r's
 * frontier with values equal to their row ids.  parents[r * n + v] (root-
 * major, int64) = the smallest frontier neighbour through which v was
 * reached from roots[r], roots[r] itself for the root (the reference's
 * visited matrix starts with the sources), -1 if unreached.  roots is a host
 * array; parents is where-located and holds nroots * n entries. */
typedef struct {
    int64_t levels;   /* loop iterations until every frontier was empty */
    int64_t reached;  /* reached (root, vertex) pairs, roots included */
    int64_t edges;    /* sum over roots of undirected edges of the reached vertices */
    double ms;        /* device time */
    int64_t host_checks; /* host round trips inside the level loop (0: one graph) */
} gbc_msbfs_stats;

int gbc_msbfs(gbc_context *ctx, gbc_graph *g, const int64_t *roots, int64_t nroots, int64_t *parents, int where,
              gbc_msbfs_stats *st);

/* Allocation-free form of gbc_spmspv_select2ndmin_i64, for callers that
 * cannot call cudaMalloc where they need the product: code running while
 * another component has reserved the device's free memory, latency-critical
 * paths that cannot take cudaMalloc's implicit device synchronisation, or
 * environments that forbid driver allocations after start-up.  It has no
 * counterpart in the reference.  Every array is caller-provided device
 * memory on the current device (A as CSC: cp[ncol+1], ir[nnz]; x: indx,
 * numx[veclen]; y: indy, numy with room for nrow entries); *nnzy (host) gets
 * the output count after the call synchronises `stream` (a cudaStream_t,
 * NULL for the default stream); every call waits for `stream` before it
 * returns.  Working storage is one fixed __device__ array of about 8.4 MB,
 * held until the process exits by every GPU on which it was used; nrow
 * above 1048576 is rejected with GBC_EOVERFLOW.  The CUDA runtime reserves
 * the array when it loads the library's device code on a device -- under
 * lazy module loading (the default) during the first call on that device --
 * so make one warm-up call per device at start-up (nrow = 0, veclen = 0),
 * while the 8.4 MB are still free.  All calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller.  Because
 * every call reads the output count back and synchronises `stream`, no call
 * can be captured into a CUDA graph: call it outside any stream capture. */
int gbc_spmspv_select2ndmin_noalloc(int64_t nrow, int64_t ncol, int64_t nnz, const int64_t *cp, const int64_t *ir,
                                    const int32_t *indx, const int64_t *numx, int32_t veclen, int32_t *indy,
                                    int64_t *numy, int32_t *nnzy, void *stream);

#ifdef __cplusplus
}
#endif
#endif
