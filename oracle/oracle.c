/* Oracle (test infrastructure only): a plain-C, OpenMP restatement of the
 * reference's node-local kernels, used by the tests as the checker of the
 * CUDA path and by the benchmark as the timed CPU baseline where the
 * reference itself was not compiled.  Product code never links it.
 *
 *   gbc_o_spgemm      LocalSpGEMMHash / LocalHybridSpGEMM hash path
 *                     (mtSpGEMM.h:463-656, 362-440): estimateFLOP
 *                     (mtSpGEMM.h:1318-1359), estimateNNZ_Hash
 *                     (mtSpGEMM.h:1363-1437), prefixsum (mtSpGEMM.h:23-70),
 *                     linear-probing table of size pow2 >= nnz (min 16,
 *                     hash key*107), sort by row (sort_less,
 *                     mtSpGEMM.h:206-210) or hash-slot order when unsorted.
 *                     Every column takes the hash path, so PlusTimes sums are
 *                     accumulated in B-entry order: val = add(mrhs, val).
 *   gbc_o_spgemm_exact  PlusTimes<double> with the library's exact fold
 *                     (sum of the same rounded products, rounded once).
 *   gbc_o_spmspv      SpMXSpV_Bucket (SpImpl.cpp:389-699): per-bucket row
 *                     split, SPA merge with the semiring add, sort of the
 *                     touched rows, output sorted by row.
 *   gbc_o_spmspv_sr   the other SpMXSpV semirings (Select2nd, SelectMax,
 *                     PlusTimes; SpImpl.cpp:167-328, 389-699)
 *   gbc_o_bfs         BFS_CSC level loop (SpMSpVBench.cpp:105-156) over
 *                     SelectMinSR (SpMSpVBench.cpp:79-100).
 *   gbc_o_mcl_select  MCLPruneRecoverySelect (recovery: gbc_o_mcl_select_recover)
 *                     (ParFriends.h:185-354) and Kselect1
 *                     (SpParMat.cpp:1191-1300): prune <= thr for the
 *                     statistics, select columns whose pruned nnz > k, kth =
 *                     k-th largest of the unpruned column, then remove < kth
 *                     there and < thr elsewhere (PruneColumn with std::less).
 *   gbc_o_mcl_colscale / gbc_o_mcl_chaos / gbc_o_mcl_inflate
 *                     MakeColStochastic, Chaos, Inflate (Applications/MCL.cpp:389-449)
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { SR_PT_F64 = 0, SR_PT_F32 = 1, SR_PT_I64 = 2, SR_MP_F64 = 3, SR_S2M_I64 = 4, SR_BOOL = 5, SR_MP_I64 = 6 };

static size_t sr_size(int sr)
{
    switch (sr) {
        case SR_PT_F32: return 4;
        case SR_BOOL: return 1;
        default: return 8;
    }
}

/* ---------------------------------------------------------------- result */
static int64_t *g_colptr = NULL, *g_rows = NULL;
static void *g_vals = NULL;
static int64_t g_ncol = 0, g_nnz = 0;
static size_t g_vsize = 8;

static void result_reset(int64_t ncol, int64_t nnz, size_t vsize)
{
    free(g_colptr);
    free(g_rows);
    free(g_vals);
    g_ncol = ncol;
    g_nnz = nnz;
    g_vsize = vsize;
    g_colptr = (int64_t *)calloc((size_t)ncol + 1, sizeof(int64_t));
    g_rows = (int64_t *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
    g_vals = malloc((size_t)(nnz > 0 ? nnz : 1) * vsize);
}

void gbc_o_result(int64_t *colptr, int64_t *rows, void *vals)
{
    if (colptr) memcpy(colptr, g_colptr, ((size_t)g_ncol + 1) * sizeof(int64_t));
    if (rows) memcpy(rows, g_rows, (size_t)g_nnz * sizeof(int64_t));
    if (vals) memcpy(vals, g_vals, (size_t)g_nnz * g_vsize);
}

int gbc_o_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int64_t gbc_o_mcl_select_recover(int64_t n, const int64_t *Ccp, const int64_t *Cri, const float *Cv, float thr,
                                 int64_t select, int64_t recover_num, float recover_pct);
void gbc_o_mcl_colscale(int64_t n, const int64_t *cp, float *v);
float gbc_o_mcl_chaos(int64_t n, const int64_t *cp, const float *v);
void gbc_o_mcl_inflate(int64_t nnz, float *v, double power);

/* ------------------------------------------------------- symbolic passes */
/* estimateFLOP, CSC form (mtSpGEMM.h:1318-1359). */
static void col_flops(int64_t n, const int64_t *Acp, const int64_t *Bcp, const int64_t *Bri, int64_t *flop)
{
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; ++j) {
        int64_t f = 0;
        for (int64_t p = Bcp[j]; p < Bcp[j + 1]; ++p) f += Acp[Bri[p] + 1] - Acp[Bri[p]];
        flop[j] = f;
    }
}

static int64_t pow2_at_least(int64_t x)
{
    int64_t s = 16; /* minHashTableSize */
    while (s < x) s <<= 1;
    return s;
}

/* estimateNNZ_Hash, CSC form (mtSpGEMM.h:1363-1437): table pow2 >= flop. */
static void col_nnz_hash(int64_t n, const int64_t *Acp, const int64_t *Ari, const int64_t *Bcp,
                         const int64_t *Bri, const int64_t *flop, int64_t *nnz)
{
#pragma omp parallel
    {
        int64_t cap = 0;
        int64_t *T = NULL;
#pragma omp for schedule(dynamic, 64)
        for (int64_t j = 0; j < n; ++j) {
            int64_t ht = pow2_at_least(flop[j]);
            if (ht > cap) {
                free(T);
                cap = ht;
                T = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
            }
            for (int64_t s = 0; s < ht; ++s) T[s] = -1;
            int64_t cnt = 0;
            for (int64_t p = Bcp[j]; p < Bcp[j + 1]; ++p) {
                int64_t c = Bri[p];
                for (int64_t q = Acp[c]; q < Acp[c + 1]; ++q) {
                    int64_t key = Ari[q];
                    int64_t h = (key * 107) & (ht - 1);
                    for (;;) {
                        if (T[h] == key) break;
                        if (T[h] == -1) {
                            T[h] = key;
                            ++cnt;
                            break;
                        }
                        h = (h + 1) & (ht - 1);
                    }
                }
            }
            nnz[j] = cnt;
        }
        free(T);
    }
}

/* ------------------------------------------------------- numeric passes */
/* Semiring operations (Semirings.h:212-255, FastSV.h:25-44). */
#define MUL_PT(a, b) ((a) * (b))
#define ADD_PT(a, b) ((a) + (b))
#define MUL_BOOL(a, b) ((uint8_t)((a) && (b)))
#define ADD_BOOL(a, b) ((uint8_t)((a) || (b)))
#define ADD_MIN(a, b) ((b) < (a) ? (b) : (a)) /* std::min */
#define MUL_S2(a, b) (b)
#define MUL_MPF64(a, b) (((a) == DBL_MAXV || (b) == DBL_MAXV) ? DBL_MAXV : (a) + (b))
#define MUL_MPI64(a, b) (((a) == INT64_MAX || (b) == INT64_MAX) ? INT64_MAX : (a) + (b))
static const double DBL_MAXV = 1.7976931348623157e308;

typedef struct {
    int64_t key;
    char val[8];
} slot_t;

static int cmp_slot(const void *x, const void *y)
{
    int64_t a = ((const slot_t *)x)->key, b = ((const slot_t *)y)->key;
    return (a > b) - (a < b);
}

/* One numeric routine per (value type, semiring): hash accumulate in the
 * order of mtSpGEMM.h:593-623, then sorted gather (:625-636) or slot-order
 * gather (:638-646). */
#define DEFINE_NUMERIC(NAME, T, MUL, ADD)                                                                      \
    static void NAME(int64_t n, const int64_t *Acp, const int64_t *Ari, const T *Av, const int64_t *Bcp,      \
                     const int64_t *Bri, const T *Bv, const int64_t *Ccp, int64_t *Cri, T *Cv, int sorted)    \
    {                                                                                                          \
        _Pragma("omp parallel")                                                                                \
        {                                                                                                      \
            int64_t cap = 0;                                                                                   \
            slot_t *H = NULL;                                                                                  \
            _Pragma("omp for schedule(dynamic, 64)") for (int64_t j = 0; j < n; ++j)                           \
            {                                                                                                  \
                int64_t nz = Ccp[j + 1] - Ccp[j];                                                              \
                int64_t ht = pow2_at_least(nz);                                                                \
                if (ht > cap) {                                                                                \
                    free(H);                                                                                   \
                    cap = ht;                                                                                  \
                    H = (slot_t *)malloc((size_t)cap * sizeof(slot_t));                                        \
                }                                                                                              \
                for (int64_t s = 0; s < ht; ++s) H[s].key = -1;                                                \
                for (int64_t p = Bcp[j]; p < Bcp[j + 1]; ++p) {                                                \
                    int64_t c = Bri[p];                                                                        \
                    T bval = Bv[p];                                                                            \
                    for (int64_t q = Acp[c]; q < Acp[c + 1]; ++q) {                                            \
                        T mrhs = MUL(Av[q], bval);                                                             \
                        int64_t key = Ari[q];                                                                  \
                        int64_t h = (key * 107) & (ht - 1);                                                    \
                        for (;;) {                                                                             \
                            T *sv = (T *)H[h].val;                                                             \
                            if (H[h].key == key) {                                                             \
                                *sv = ADD(mrhs, *sv);                                                          \
                                break;                                                                         \
                            }                                                                                  \
                            if (H[h].key == -1) {                                                              \
                                H[h].key = key;                                                                \
                                *sv = mrhs;                                                                    \
                                break;                                                                         \
                            }                                                                                  \
                            h = (h + 1) & (ht - 1);                                                            \
                        }                                                                                      \
                    }                                                                                          \
                }                                                                                              \
                int64_t idx = 0;                                                                               \
                for (int64_t s = 0; s < ht; ++s)                                                               \
                    if (H[s].key != -1) H[idx++] = H[s];                                                       \
                if (sorted) qsort(H, (size_t)idx, sizeof(slot_t), cmp_slot);                                   \
                int64_t o = Ccp[j];                                                                            \
                for (int64_t s = 0; s < idx; ++s, ++o) {                                                       \
                    Cri[o] = H[s].key;                                                                         \
                    Cv[o] = *(T *)H[s].val;                                                                    \
                }                                                                                              \
            }                                                                                                  \
            free(H);                                                                                           \
        }                                                                                                      \
    }

DEFINE_NUMERIC(num_pt_f64, double, MUL_PT, ADD_PT)
DEFINE_NUMERIC(num_pt_f32, float, MUL_PT, ADD_PT)
DEFINE_NUMERIC(num_pt_i64, int64_t, MUL_PT, ADD_PT)
DEFINE_NUMERIC(num_mp_f64, double, MUL_MPF64, ADD_MIN)
DEFINE_NUMERIC(num_s2m_i64, int64_t, MUL_S2, ADD_MIN)
DEFINE_NUMERIC(num_bool, uint8_t, MUL_BOOL, ADD_BOOL)
DEFINE_NUMERIC(num_mp_i64, int64_t, MUL_MPI64, ADD_MIN)

/* C = A * B over semiring `sr`, both CSC with int64 indices (B is m_B = k x n).
 * Returns nnz(C); the result is fetched with gbc_o_result.  flop_out /
 * nnz_out (optional, length n) receive the per-column symbolic counts. */
int64_t gbc_o_spgemm(int sr, int sorted, int64_t m, int64_t k, int64_t n, const int64_t *Acp, const int64_t *Ari,
                     const void *Av, const int64_t *Bcp, const int64_t *Bri, const void *Bv, int64_t *flop_out,
                     int64_t *nnz_out)
{
    (void)m;
    (void)k;
    int64_t *flop = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    int64_t *cnt = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    col_flops(n, Acp, Bcp, Bri, flop);
    col_nnz_hash(n, Acp, Ari, Bcp, Bri, flop, cnt);
    int64_t tot = 0;
    for (int64_t j = 0; j < n; ++j) tot += cnt[j];
    result_reset(n, tot, sr_size(sr));
    for (int64_t j = 0; j < n; ++j) g_colptr[j + 1] = g_colptr[j] + cnt[j];
    if (flop_out) memcpy(flop_out, flop, (size_t)n * sizeof(int64_t));
    if (nnz_out) memcpy(nnz_out, cnt, (size_t)n * sizeof(int64_t));
    free(flop);
    free(cnt);
    switch (sr) {
        case SR_PT_F64: num_pt_f64(n, Acp, Ari, Av, Bcp, Bri, Bv, g_colptr, g_rows, g_vals, sorted); break;
        case SR_PT_F32: num_pt_f32(n, Acp, Ari, Av, Bcp, Bri, Bv, g_colptr, g_rows, g_vals, sorted); break;
        case SR_PT_I64: num_pt_i64(n, Acp, Ari, Av, Bcp, Bri, Bv, g_colptr, g_rows, g_vals, sorted); break;
        case SR_MP_F64: num_mp_f64(n, Acp, Ari, Av, Bcp, Bri, Bv, g_colptr, g_rows, g_vals, sorted); break;
        case SR_S2M_I64: num_s2m_i64(n, Acp, Ari, Av, Bcp, Bri, Bv, g_colptr, g_rows, g_vals, sorted); break;
        case SR_BOOL: num_bool(n, Acp, Ari, Av, Bcp, Bri, Bv, g_colptr, g_rows, g_vals, sorted); break;
        case SR_MP_I64: num_mp_i64(n, Acp, Ari, Av, Bcp, Bri, Bv, g_colptr, g_rows, g_vals, sorted); break;
        default: return -1;
    }
    return tot;
}

/* ----------------------------------------------------------------- SpMSpV */
/* ------------------------------------------- exact PlusTimes fp64 fold */
/* The library's GBC_FOLD_EXACT semantics, restated on the host: every
 * product fl(a*b) is formed as the reference forms it, the products of one
 * output entry are added exactly (a signed 128-bit integer in units of
 * 2^(ebase-1075)), and the sum is rounded once to the nearest double, ties
 * to even.  A column takes this fold when its products are normal, finite
 * and span at most 61 binades, with the exact sum below 2^125 and the
 * rounded result finite (the window is bounded from each A column's
 * exponent range and each B value's exponent); other columns keep the hash
 * path's left fold.  Output rows are sorted. */
static void exp_range(int64_t ncol, const int64_t *Acp, const double *Av, int *amin, int *amax)
{
    _Pragma("omp parallel for schedule(static)")
    for (int64_t c = 0; c < ncol; ++c) {
        int lo = 32767, hi = -32768;
        for (int64_t q = Acp[c]; q < Acp[c + 1]; ++q) {
            uint64_t bits;
            memcpy(&bits, &Av[q], 8);
            if ((bits << 1) == 0) continue;
            int e = (int)((bits >> 52) & 0x7ff);
            if (e == 0) e = -64;
            if (e < lo) lo = e;
            if (e > hi) hi = e;
        }
        amin[c] = lo;
        amax[c] = hi;
    }
}

static int bit_length_i64(int64_t x)
{
    int b = 0;
    while (x > 0) {
        ++b;
        x >>= 1;
    }
    return b;
}

static double round_exact(__int128 M, int nonnegzero, int ebase)
{
    if (M == 0) return nonnegzero ? 0.0 : -0.0;
    const int neg = M < 0;
    unsigned __int128 u = neg ? (unsigned __int128)(-M) : (unsigned __int128)M;
    double d;
    if (u < ((unsigned __int128)1 << 53)) {
        d = ldexp((double)(uint64_t)u, ebase - 1075);
    } else {
        int top = 127;
        while (!((u >> top) & 1)) --top;
        int sh = top > 63 ? top - 63 : 0;
        uint64_t w = (uint64_t)(u >> sh);
        if (sh && (u & (((unsigned __int128)1 << sh) - 1))) w |= 1; /* sticky */
        d = ldexp((double)w, sh + ebase - 1075); /* (double)w rounds to nearest even */
    }
    return neg ? -d : d;
}

/* C = A*B over PlusTimes<double> with the exact fold; result as gbc_o_spgemm
 * (sorted rows).  Returns nnz(C). */
int64_t gbc_o_spgemm_exact(int64_t m, int64_t k, int64_t n, const int64_t *Acp, const int64_t *Ari,
                           const double *Av, const int64_t *Bcp, const int64_t *Bri, const double *Bv,
                           int64_t *flop_out, int64_t *nnz_out)
{
    const int64_t tot = gbc_o_spgemm(SR_PT_F64, 1, m, k, n, Acp, Ari, Av, Bcp, Bri, Bv, flop_out, nnz_out);
    int *amin = (int *)malloc((size_t)(k > 0 ? k : 1) * sizeof(int));
    int *amax = (int *)malloc((size_t)(k > 0 ? k : 1) * sizeof(int));
    exp_range(k, Acp, Av, amin, amax);
    double *Cv = (double *)g_vals;
    _Pragma("omp parallel")
    {
        int64_t cap = 0;
        __int128 *acc = NULL;
        unsigned char *nz = NULL;
        _Pragma("omp for schedule(dynamic, 64)") for (int64_t j = 0; j < n; ++j)
        {
            int ebase = 1 << 30, etop = -(1 << 30);
            for (int64_t p = Bcp[j]; p < Bcp[j + 1]; ++p) {
                const int64_t c = Bri[p];
                uint64_t bb;
                memcpy(&bb, &Bv[p], 8);
                if (amin[c] > amax[c] || (bb << 1) == 0) continue;
                int eb = (int)((bb >> 52) & 0x7ff);
                if (eb == 0) eb = -64;
                if (amin[c] + eb - 1023 < ebase) ebase = amin[c] + eb - 1023;
                if (amax[c] + eb - 1022 > etop) etop = amax[c] + eb - 1022;
            }
            const int lg = bit_length_i64(Bcp[j + 1] - Bcp[j]);
            if (ebase > etop) {
                ebase = 1;
            } else if (!(ebase >= 1 && etop <= 2046 - lg - 2 && etop - ebase <= 61 && etop - ebase + 53 + lg <= 125)) {
                continue; /* keeps the hash path's left fold */
            }
            const int64_t c0 = g_colptr[j], c1 = g_colptr[j + 1];
            if (c1 - c0 > cap) {
                free(acc);
                free(nz);
                cap = c1 - c0;
                acc = (__int128 *)malloc((size_t)cap * sizeof(__int128));
                nz = (unsigned char *)malloc((size_t)cap);
            }
            memset(acc, 0, (size_t)(c1 - c0) * sizeof(__int128));
            memset(nz, 0, (size_t)(c1 - c0));
            for (int64_t p = Bcp[j]; p < Bcp[j + 1]; ++p) {
                const int64_t c = Bri[p];
                const double b = Bv[p];
                for (int64_t q = Acp[c]; q < Acp[c + 1]; ++q) {
                    const double prod = Av[q] * b;
                    int64_t lo = c0, hi = c1;
                    while (lo < hi) {
                        const int64_t mid = (lo + hi) >> 1;
                        if (g_rows[mid] < Ari[q])
                            lo = mid + 1;
                        else
                            hi = mid;
                    }
                    const int64_t o = lo - c0;
                    uint64_t bits;
                    memcpy(&bits, &prod, 8);
                    if (bits != (1ull << 63)) nz[o] = 1;
                    const int e = (int)((bits >> 52) & 0x7ff);
                    if (e == 0) continue; /* zero: admitted columns have no subnormal products */
                    const __int128 mag = (__int128)((bits & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << (e - ebase);
                    acc[o] += (bits >> 63) ? -mag : mag;
                }
            }
            for (int64_t o = c0; o < c1; ++o) Cv[o] = round_exact(acc[o - c0], nz[o - c0], ebase);
        }
        free(acc);
        free(nz);
    }
    free(amin);
    free(amax);
    return tot;
}

static int cmp_i32(const void *x, const void *y)
{
    int32_t a = *(const int32_t *)x, b = *(const int32_t *)y;
    return (a > b) - (a < b);
}

/* y = A x over SelectMinSR (pattern A, int64 x values): SpMXSpV_Bucket
 * (SpImpl.cpp:389-699).  The frontier is split evenly over `buckets` row
 * splits; each split's entries are merged into a dense SPA with min, its
 * touched rows sorted; splits are concatenated in row order.  Result: row
 * ids in g_rows, values (int64) in g_vals; returns nnz(y). */
int64_t gbc_o_spmspv(int64_t m, const int64_t *Acp, const int64_t *Ari, const int32_t *indx, const int64_t *numx,
                     int32_t veclen, int buckets)
{
    if (buckets < 1) buckets = 1;
    int32_t rowPerSplit = (int32_t)(m / buckets);
    /* scatter every (row, value) into its row split -- count, then fill */
    int64_t *bcnt = (int64_t *)calloc((size_t)buckets + 1, sizeof(int64_t));
    for (int32_t i = 0; i < veclen; ++i) {
        int64_t c = indx[i];
        for (int64_t p = Acp[c]; p < Acp[c + 1]; ++p) {
            int64_t r = Ari[p];
            int64_t s = rowPerSplit ? r / rowPerSplit : buckets - 1;
            if (s > buckets - 1) s = buckets - 1;
            bcnt[s + 1]++;
        }
    }
    for (int b = 0; b < buckets; ++b) bcnt[b + 1] += bcnt[b];
    int64_t tot = bcnt[buckets];
    int32_t *brow = (int32_t *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(int32_t));
    int64_t *bval = (int64_t *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(int64_t));
    int64_t *fill = (int64_t *)malloc((size_t)buckets * sizeof(int64_t));
    memcpy(fill, bcnt, (size_t)buckets * sizeof(int64_t));
    for (int32_t i = 0; i < veclen; ++i) {
        int64_t c = indx[i];
        for (int64_t p = Acp[c]; p < Acp[c + 1]; ++p) {
            int64_t r = Ari[p];
            int64_t s = rowPerSplit ? r / rowPerSplit : buckets - 1;
            if (s > buckets - 1) s = buckets - 1;
            brow[fill[s]] = (int32_t)r;
            bval[fill[s]++] = numx[i]; /* multiply returns the vector value */
        }
    }
    free(fill);
    int64_t *spa = (int64_t *)malloc((size_t)(m > 0 ? m : 1) * sizeof(int64_t));
    uint8_t *seen = (uint8_t *)calloc((size_t)(m > 0 ? m : 1), 1);
    int32_t *nz = (int32_t *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(int32_t));
    int64_t *nzcnt = (int64_t *)calloc((size_t)buckets, sizeof(int64_t));
#pragma omp parallel for schedule(dynamic, 1)
    for (int b = 0; b < buckets; ++b) {
        int64_t o = bcnt[b];
        for (int64_t i = bcnt[b]; i < bcnt[b + 1]; ++i) {
            int32_t r = brow[i];
            if (!seen[r]) {
                seen[r] = 1;
                spa[r] = bval[i];
                nz[o++] = r;
            } else {
                spa[r] = ADD_MIN(spa[r], bval[i]);
            }
        }
        nzcnt[b] = o - bcnt[b];
        qsort(nz + bcnt[b], (size_t)nzcnt[b], sizeof(int32_t), cmp_i32);
    }
    int64_t ny = 0;
    for (int b = 0; b < buckets; ++b) ny += nzcnt[b];
    result_reset(0, ny, 8);
    int64_t o = 0;
    for (int b = 0; b < buckets; ++b)
        for (int64_t i = 0; i < nzcnt[b]; ++i, ++o) {
            int32_t r = nz[bcnt[b] + i];
            g_rows[o] = r;
            ((int64_t *)g_vals)[o] = spa[r];
        }
    free(brow);
    free(bval);
    free(spa);
    free(seen);
    free(nz);
    free(nzcnt);
    free(bcnt);
    return ny;
}

/* y = A x over the other SpMXSpV semirings (SpImpl.h:49-142).  Every
 * variant visits the vector's columns in the vector's (ascending) order and,
 * per row, stores the first product and folds later ones in with the add
 * (the SPA of SpMXSpV_Bucket, SpImpl.cpp:389-699, and of the boolean loops,
 * SpImpl.cpp:167-328); rows come out ascending.  sx: 0 SelectMin (add min,
 * multiply returns x), 1 Select2nd (add keeps the second argument), 2
 * SelectMax (add max), 3 PlusTimes (multiply A*x, add +).  Values: int64 for
 * 0-2; for 3 vt 0 double, 1 float, 2 int64 (matrix and vector alike).
 * Returns nnz(y); rows and values in the result buffers. */
int64_t gbc_o_spmspv_sr(int sx, int vt, int64_t m, const int64_t *Acp, const int64_t *Ari, const void *Av,
                        const int32_t *indx, const void *numx, int32_t veclen)
{
    const size_t vs = sx == 3 && vt == 1 ? 4 : 8;
    char *spa = (char *)malloc((size_t)(m > 0 ? m : 1) * vs);
    uint8_t *seen = (uint8_t *)calloc((size_t)(m > 0 ? m : 1), 1);
    int32_t *nz = (int32_t *)malloc((size_t)(m > 0 ? m : 1) * sizeof(int32_t));
    int64_t ny = 0;
    for (int32_t f = 0; f < veclen; ++f) {
        const int64_t c = indx[f];
        for (int64_t p = Acp[c]; p < Acp[c + 1]; ++p) {
            const int64_t r = Ari[p];
            const int first = !seen[r];
            if (first) {
                seen[r] = 1;
                nz[ny++] = (int32_t)r;
            }
            if (sx == 3 && vt == 0) {
                const double v = ((const double *)Av)[p] * ((const double *)numx)[f];
                double *y = (double *)spa + r;
                *y = first ? v : *y + v;
            } else if (sx == 3 && vt == 1) {
                const float v = ((const float *)Av)[p] * ((const float *)numx)[f];
                float *y = (float *)spa + r;
                *y = first ? v : *y + v;
            } else {
                const int64_t v = sx == 3 ? ((const int64_t *)Av)[p] * ((const int64_t *)numx)[f]
                                          : ((const int64_t *)numx)[f];
                int64_t *y = (int64_t *)spa + r;
                if (first)
                    *y = v;
                else if (sx == 0)
                    *y = v < *y ? v : *y;
                else if (sx == 1)
                    *y = v;
                else if (sx == 2)
                    *y = v > *y ? v : *y;
                else
                    *y = *y + v;
            }
        }
    }
    qsort(nz, (size_t)ny, sizeof(int32_t), cmp_i32);
    result_reset(0, ny, vs);
    for (int64_t i = 0; i < ny; ++i) {
        g_rows[i] = nz[i];
        memcpy((char *)g_vals + i * vs, spa + (size_t)nz[i] * vs, vs);
    }
    free(spa);
    free(seen);
    free(nz);
    return ny;
}

/* BFS from `source` as the BFS_CSC loop (SpMSpVBench.cpp:128-156):
 *   fringe = {source: source}
 *   while fringe nonempty:
 *     fringe.setNumToInd(); fringe = A*fringe over SelectMin;
 *     fringe = EWiseMult(fringe, parents, exclude=true, -1); parents.Set(fringe)
 * The source itself receives a parent only when a later level reaches it.
 * levels[v] = loop iteration (1-based) in which v first entered the fringe,
 * levels[source] = 0, -1 unreached.  Returns the number of iterations. */
int gbc_o_bfs(int64_t n, const int64_t *Acp, const int64_t *Ari, int64_t source, int64_t *parents, int64_t *levels)
{
    for (int64_t i = 0; i < n; ++i) {
        parents[i] = -1;
        if (levels) levels[i] = -1;
    }
    if (levels) levels[source] = 0;
    int64_t *fr = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int64_t *nfr = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int64_t *cand = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) cand[i] = INT64_MAX;
    int64_t nf = 1;
    fr[0] = source;
    int it = 0;
    while (nf > 0) {
        /* y(r) = min over frontier columns c with A(r,c) of c */
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < nf; ++i) {
            int64_t c = fr[i];
            for (int64_t p = Acp[c]; p < Acp[c + 1]; ++p) {
                int64_t r = Ari[p];
                if (parents[r] != -1) continue; /* EWiseMult exclude: dropped anyway */
                int64_t cur = __atomic_load_n(&cand[r], __ATOMIC_RELAXED);
                while (c < cur && !__atomic_compare_exchange_n(&cand[r], &cur, c, 0, __ATOMIC_RELAXED,
                                                               __ATOMIC_RELAXED)) {
                }
            }
        }
        /* gather the new fringe in row order (the SpMSpV output is sorted) */
        int64_t k = 0;
        for (int64_t i = 0; i < nf; ++i) {
            int64_t c = fr[i];
            for (int64_t p = Acp[c]; p < Acp[c + 1]; ++p) {
                int64_t r = Ari[p];
                if (cand[r] != INT64_MAX && parents[r] == -1) {
                    parents[r] = cand[r];
                    nfr[k++] = r;
                }
            }
        }
        ++it;
        for (int64_t i = 0; i < k; ++i) {
            cand[nfr[i]] = INT64_MAX;
            if (levels && levels[nfr[i]] < 0) levels[nfr[i]] = it;
        }
        int64_t *t = fr;
        fr = nfr;
        nfr = t;
        nf = k;
    }
    free(fr);
    free(nfr);
    free(cand);
    return it;
}

/* ------------------------------------------------------------ MCL select */
static int cmp_f32_desc(const void *x, const void *y)
{
    float a = *(const float *)x, b = *(const float *)y;
    return (a < b) - (a > b);
}

/* Column sum of the fp32 values of [b, e) that pass keep(v) (mode 0: v > thr,
 * mode 1: !(v < thr)): the exact sum of their parts
 * (with 2^emax the largest value's exponent among them, every part below
 * 2^(emax - 72) is truncated),
 * rounded to double and then to float -- independent of the column's
 * storage order (the library's definition of the MCL column sums). */
static float mcl_colsum(const float *v, int64_t b, int64_t e, float thr, int mode)
{
    int emax = -1000;
    for (int64_t p = b; p < e; ++p) {
        const float x = mode == 2 ? (float)((double)v[p] * v[p]) : v[p];
        if (mode == 0 ? !(x > thr) : mode == 1 ? (x < thr) : 0) continue;
        uint32_t u;
        memcpy(&u, &x, 4);
        if ((u << 1) == 0) continue;
        int ex = (int)((u >> 23) & 0xff);
        if (ex == 0) ex = 1;
        if (ex > emax) emax = ex;
    }
    if (emax == -1000) return 0.0f;
    const int unit = emax - 150 - 72; /* value of the accumulator's lowest bit: 2^unit */
    __int128 acc = 0;
    for (int64_t p = b; p < e; ++p) {
        const float x = mode == 2 ? (float)((double)v[p] * v[p]) : v[p];
        if (mode == 0 ? !(x > thr) : mode == 1 ? (x < thr) : 0) continue;
        uint32_t u;
        memcpy(&u, &x, 4);
        int ex = (int)((u >> 23) & 0xff);
        uint32_t m = u & 0x7fffff;
        if (ex) m |= 0x800000; else ex = 1;
        const int sh = ex - 150 - unit; /* m * 2^(ex - 150) = (m << sh) * 2^unit */
        __int128 t = sh >= 0 ? ((__int128)m << sh) : (__int128)(m >> (-sh < 32 ? -sh : 31));
        acc += (u >> 31) ? -t : t;
    }
    return (float)round_exact(acc, 1, unit + 1075);
}

/* Kselect1 with a sparse column list (SpParMat.cpp:1411-1690): the k-th
 * largest value of the column, its smallest value when it holds fewer than
 * k entries, numeric_limits<float>::min() when it is empty. */
static float mcl_kth(const float *v, int64_t b, int64_t e, int64_t k, float **buf, int64_t *cap)
{
    if (e == b) return 1.17549435e-38f;
    if (e - b > *cap) {
        free(*buf);
        *cap = e - b;
        *buf = (float *)malloc((size_t)*cap * sizeof(float));
    }
    memcpy(*buf, v + b, (size_t)(e - b) * sizeof(float));
    qsort(*buf, (size_t)(e - b), sizeof(float), cmp_f32_desc);
    return e - b >= k ? (*buf)[k - 1] : (*buf)[e - b - 1];
}

/* Prune + select + recovery of one MCL expansion step
 * (MCLPruneRecoverySelect, ParFriends.h:185-354).  Per column of C (fp32
 * CSC, rows in any order; the output keeps the within-column order):
 *   nnzP, sumP of the entries with val > thr (the "val <= thr" prune);
 *   recovered when recover_num > 0, nnzP < recover_num, nnz > nnzP and
 *     sumP < recover_pct: cut = Kselect(recover_num) of the whole column;
 *   else selected when select > 0 and nnzP > select: cut = Kselect(select),
 *     and, when recover_num > 0, the selection is recovered if the entries
 *     it keeps (val >= cut) number fewer than recover_num and sum below
 *     recover_pct: cut = Kselect(recover_num);
 *   else cut = thr;
 * then PruneColumn(std::less) drops val < cut.  Column sums: mcl_colsum.
 * Returns nnz of the result. */
int64_t gbc_o_mcl_select_recover(int64_t n, const int64_t *Ccp, const int64_t *Cri, const float *Cv, float thr,
                                 int64_t select, int64_t recover_num, float recover_pct)
{
    float *cut = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
    int64_t *keep = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
#pragma omp parallel
    {
        float *buf = NULL;
        int64_t cap = 0;
#pragma omp for schedule(dynamic, 64)
        for (int64_t j = 0; j < n; ++j) {
            const int64_t b = Ccp[j], e = Ccp[j + 1];
            int64_t npruned = 0; /* entries surviving "val <= thr" pruning */
            for (int64_t p = b; p < e; ++p) npruned += !(Cv[p] <= thr);
            float c = thr; /* pruneCols default: hardThreshold */
            const int recover = recover_num > 0 && npruned < recover_num && (e - b) > npruned &&
                                mcl_colsum(Cv, b, e, thr, 0) < recover_pct;
            if (recover) {
                c = mcl_kth(Cv, b, e, recover_num, &buf, &cap);
            } else if (select > 0 && npruned > select) {
                c = mcl_kth(Cv, b, e, select, &buf, &cap);
                if (recover_num > 0) {
                    int64_t n1 = 0;
                    for (int64_t p = b; p < e; ++p) n1 += !(Cv[p] < c);
                    if (n1 < recover_num && mcl_colsum(Cv, b, e, c, 1) < recover_pct)
                        c = mcl_kth(Cv, b, e, recover_num, &buf, &cap);
                }
            }
            cut[j] = c;
            int64_t kcount = 0; /* PruneColumn(std::less): drop val < cut */
            for (int64_t p = b; p < e; ++p) kcount += !(Cv[p] < c);
            keep[j] = kcount;
        }
        free(buf);
    }
    int64_t tot = 0;
    for (int64_t j = 0; j < n; ++j) tot += keep[j];
    result_reset(n, tot, 4);
    for (int64_t j = 0; j < n; ++j) g_colptr[j + 1] = g_colptr[j] + keep[j];
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n; ++j) {
        int64_t o = g_colptr[j];
        for (int64_t p = Ccp[j]; p < Ccp[j + 1]; ++p)
            if (!(Cv[p] < cut[j])) {
                g_rows[o] = Cri[p];
                ((float *)g_vals)[o++] = Cv[p];
            }
    }
    free(cut);
    free(keep);
    return tot;
}

/* recoverNum = 0 (the expansion step of MemEfficientSpGEMM without recovery). */
int64_t gbc_o_mcl_select(int64_t n, const int64_t *Ccp, const int64_t *Cri, const float *Cv, float thr,
                         int64_t select)
{
    return gbc_o_mcl_select_recover(n, Ccp, Cri, Cv, thr, select, 0, 0.0f);
}

/* MakeColStochastic (Applications/MCL.cpp:389-394) in place: every column
 * scaled by 1 / (its sum), FLT_MAX for a zero sum (safemultinv,
 * Operations.h:103-110).  The sum is mcl_colsum over all values. */
void gbc_o_mcl_colscale(int64_t n, const int64_t *cp, float *v)
{
    _Pragma("omp parallel for schedule(dynamic, 256)")
    for (int64_t j = 0; j < n; ++j) {
        const float sum = mcl_colsum(v, cp[j], cp[j + 1], -3.4028235e38f, 1);
        const float inv = sum == 0.0f ? 3.4028235e38f : 1.0f / sum;
        for (int64_t p = cp[j]; p < cp[j + 1]; ++p) v[p] = v[p] * inv;
    }
}

/* Chaos (MCL.cpp:407-421): max over columns of (column max - sum of
 * squares) * nnz(column); both maxima start from 0 (the entries are
 * non-negative).  Each square is rounded to float, as static_cast<float> of
 * pow(val, 2) is; the sum of squares is mcl_colsum's exact sum. */
float gbc_o_mcl_chaos(int64_t n, const int64_t *cp, const float *v)
{
    float best = 0.0f;
    for (int64_t j = 0; j < n; ++j) {
        float mx = 0.0f;
        for (int64_t p = cp[j]; p < cp[j + 1]; ++p) mx = v[p] > mx ? v[p] : mx;
        const float sq = mcl_colsum(v, cp[j], cp[j + 1], 0.0f, 2);
        const float c = (mx - sq) * (float)(cp[j + 1] - cp[j]);
        best = c > best ? c : best;
    }
    return best;
}

/* Inflate (MCL.cpp:446-450) in place: pow(val, power) in double, stored as
 * float. */
void gbc_o_mcl_inflate(int64_t nnz, float *v, double power)
{
    for (int64_t p = 0; p < nnz; ++p) v[p] = (float)pow((double)v[p], power);
}
