// Test infrastructure (oracle only): a ctypes-callable harness around the
// reference's own, unmodified header templates, compiled from the reference
// sources in place against the single-rank MPI stand-in in oracle/mpistub.
// Nothing here is product code; the tests and the CPU baseline leg of the
// benchmark are its only users.
//
// Entry points mirror the reference calls they wrap:
//   ref_spgemm           -> LocalHybridSpGEMM (mtSpGEMM.h:213), LocalSpGEMM
//                           (mtSpGEMM.h:74), LocalSpGEMMHash (mtSpGEMM.h:463),
//                           CSC LocalHybridSpGEMM (mtSpGEMM.h:1148),
//                           PSpGEMM on a 1x1 grid (SpParMat.h:464)
//   ref_colstats         -> estimateFLOP (mtSpGEMM.h:1057),
//                           estimateNNZ_Hash (mtSpGEMM.h:806)
//   ref_spmspv_bucket    -> SpMXSpV_Bucket (SpImpl.cpp:389)
//   ref_spmspv_sr        -> boolean SpMXSpV over Select2ndSRing with the
//                           optbuf outputs (SpImpl.cpp:222-272, TopDownBFS's
//                           path), SpMXSpV_Bucket over SelectMaxSRing and
//                           PlusTimesSRing (SpImpl.cpp:389-699)
//   ref_bfs_selectmin    -> the BFS_CSC level loop of
//                           Applications/SpMSpV-IPDPS2017/SpMSpVBench.cpp:105-156
//   ref_mcl_expand       -> MemEfficientSpGEMM + MCLPruneRecoverySelect
//                           (ParFriends.h:452,185)
//   ref_mcl_iterate      -> the HipMCL loop of Applications/MCL.cpp:526-626
//                           (one layer), over MemEfficientSpGEMM and the
//                           reference's SpParMat Reduce / DimApply / Apply
//   ref_multiway_merge   -> MultiwayMerge (MultiwayMerge.h:428)
//   ref_spmv             -> dcsc_gespmv (Friends.h:63)
#include "CombBLAS/CombBLAS.h"
#include "CombBLAS/mtSpGEMM.h"

#include <chrono>
#include <cstring>
#include <memory>
#include <vector>

using namespace combblas;

int cblas_splits = 1;
double cblas_alltoalltime, cblas_allgathertime, cblas_localspmvtime, cblas_mergeconttime, cblas_transvectime;
double mcl_Abcasttime, mcl_Bbcasttime, mcl_localspgemmtime, mcl_multiwaymergetime, mcl_kselecttime,
    mcl_prunecolumntime, mcl_symbolictime;
double mcl3d_conversiontime, mcl3d_symbolictime, mcl3d_Abcasttime, mcl3d_Bbcasttime, mcl3d_SUMMAtime,
    mcl3d_localspgemmtime, mcl3d_SUMMAmergetime, mcl3d_reductiontime, mcl3d_3dmergetime, mcl3d_kselecttime;

// Same meaning as SelectMinSR in Applications/SpMSpV-IPDPS2017/SpMSpVBench.cpp:79-100:
// add = min, multiply returns the vector value, identity -1.
struct HarnessSelectMinSR {
    typedef int64_t T_promote;
    static T_promote id() { return -1; }
    static bool returnedSAID() { return false; }
    static T_promote add(const T_promote &a, const T_promote &b) { return std::min(a, b); }
    static T_promote multiply(const bool &, const T_promote &x) { return x; }
    static void axpy(bool, const T_promote &x, T_promote &y) { y = std::min(y, x); }
};

// Same meaning as Applications/FastSV.h:25-44 (Select2ndMinSR).
template <typename T1, typename T2>
struct HarnessSelect2ndMinSR {
    typedef typename promote_trait<T1, T2>::T_promote T_promote;
    static T_promote id() { return std::numeric_limits<T_promote>::max(); }
    static bool returnedSAID() { return false; }
    static MPI_Op mpi_op() { return MPI_MIN; }
    static T_promote add(const T_promote &a, const T_promote &b) { return std::min(a, b); }
    static T_promote multiply(const T1 &, const T2 &b) { return static_cast<T_promote>(b); }
    static void axpy(const T1 a, const T2 &x, T_promote &y) { y = add(y, multiply(a, x)); }
};

namespace {

struct Result {
    std::vector<int64_t> rows, cols;
    std::vector<char> vals;  // raw bytes, element size given by the semiring
    double seconds = 0.0;
};
Result g_res;

template <typename NT>
std::vector<std::tuple<int64_t, int64_t, NT>> csc_to_tuples(int64_t n, const int64_t *cp, const int64_t *ri,
                                                             const void *vals)
{
    std::vector<std::tuple<int64_t, int64_t, NT>> t;
    t.reserve(cp[n]);
    const NT *v = static_cast<const NT *>(vals);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t p = cp[j]; p < cp[j + 1]; ++p) t.emplace_back(ri[p], j, v ? v[p] : NT(1));
    return t;
}

template <typename NT>
SpDCCols<int64_t, NT> *make_dcsc(int64_t m, int64_t n, const int64_t *cp, const int64_t *ri, const void *vals)
{
    auto t = csc_to_tuples<NT>(n, cp, ri, vals);
    auto *arr = new std::tuple<int64_t, int64_t, NT>[t.size()];
    std::copy(t.begin(), t.end(), arr);
    SpTuples<int64_t, NT> tup((int64_t)t.size(), m, n, arr, /*sorted=*/true, /*isOpNew=*/false);
    return new SpDCCols<int64_t, NT>(tup, false);
}

template <typename NT>
SpCCols<int64_t, NT> *make_csc(int64_t m, int64_t n, const int64_t *cp, const int64_t *ri, const void *vals)
{
    auto t = csc_to_tuples<NT>(n, cp, ri, vals);
    auto *arr = new std::tuple<int64_t, int64_t, NT>[t.size()];
    std::copy(t.begin(), t.end(), arr);
    SpTuples<int64_t, NT> tup((int64_t)t.size(), m, n, arr, true, false);
    return new SpCCols<int64_t, NT>(tup, false);
}

template <typename NT>
void store_tuples(SpTuples<int64_t, NT> *C)
{
    int64_t nnz = C->getnnz();
    g_res.rows.resize(nnz);
    g_res.cols.resize(nnz);
    g_res.vals.resize(nnz * sizeof(NT));
    NT *v = reinterpret_cast<NT *>(g_res.vals.data());
    for (int64_t i = 0; i < nnz; ++i) {
        g_res.rows[i] = C->rowindex(i);
        g_res.cols[i] = C->colindex(i);
        v[i] = C->numvalue(i);
    }
}

template <typename NT>
void store_dcsc(const SpDCCols<int64_t, NT> &C)
{
    int64_t nnz = C.getnnz();
    g_res.rows.resize(nnz);
    g_res.cols.resize(nnz);
    g_res.vals.resize(nnz * sizeof(NT));
    NT *v = reinterpret_cast<NT *>(g_res.vals.data());
    if (nnz == 0) return;
    Dcsc<int64_t, NT> *d = C.GetDCSC();
    int64_t q = 0;
    for (int64_t i = 0; i < d->nzc; ++i)
        for (int64_t p = d->cp[i]; p < d->cp[i + 1]; ++p, ++q) {
            g_res.rows[q] = d->ir[p];
            g_res.cols[q] = d->jc[i];
            v[q] = d->numx[p];
        }
}

double now() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

template <typename SR, typename NT>
int64_t run_spgemm(int variant, int64_t m, int64_t k, int64_t n, const int64_t *Acp, const int64_t *Ari,
                   const void *Av, const int64_t *Bcp, const int64_t *Bri, const void *Bv, int reps)
{
    if (variant == 4) {  // CSC overload
        std::unique_ptr<SpCCols<int64_t, NT>> A(make_csc<NT>(m, k, Acp, Ari, Av));
        std::unique_ptr<SpCCols<int64_t, NT>> B(make_csc<NT>(k, n, Bcp, Bri, Bv));
        SpTuples<int64_t, NT> *C = nullptr;
        double best = 1e300;
        for (int r = 0; r < reps; ++r) {
            delete C;
            double t0 = now();
            C = LocalHybridSpGEMM<SR, NT>(*A, *B, false, false);
            best = std::min(best, now() - t0);
        }
        g_res.seconds = best;
        store_tuples(C);
        int64_t nnz = C->getnnz();
        delete C;
        return nnz;
    }
    std::unique_ptr<SpDCCols<int64_t, NT>> A(make_dcsc<NT>(m, k, Acp, Ari, Av));
    std::unique_ptr<SpDCCols<int64_t, NT>> B(make_dcsc<NT>(k, n, Bcp, Bri, Bv));
    if (variant == 5) {  // PSpGEMM on a 1x1 grid: Mult_AnXBn_Synch + SpTuples->DCSC
        auto grid = std::make_shared<CommGrid>(MPI_COMM_WORLD, 1, 1);
        typedef SpParMat<int64_t, NT, SpDCCols<int64_t, NT>> PM;
        PM PA(new SpDCCols<int64_t, NT>(*A), grid);
        PM PB(new SpDCCols<int64_t, NT>(*B), grid);
        double best = 1e300;
        PM PC(grid);
        for (int r = 0; r < reps; ++r) {
            double t0 = now();
            PC = PSpGEMM<SR>(PA, PB);
            best = std::min(best, now() - t0);
        }
        g_res.seconds = best;
        store_dcsc(PC.seq());
        return PC.seq().getnnz();
    }
    SpTuples<int64_t, NT> *C = nullptr;
    double best = 1e300;
    for (int r = 0; r < reps; ++r) {
        delete C;
        double t0 = now();
        switch (variant) {
            case 0: C = LocalHybridSpGEMM<SR, NT>(*A, *B, false, false); break;
            case 1: C = LocalSpGEMM<SR, NT>(*A, *B, false, false); break;
            case 2: C = LocalSpGEMMHash<SR, NT>(*A, *B, false, false, true); break;
            case 3: C = LocalSpGEMMHash<SR, NT>(*A, *B, false, false, false); break;
            default: return -1;
        }
        best = std::min(best, now() - t0);
    }
    g_res.seconds = best;
    store_tuples(C);
    int64_t nnz = C->getnnz();
    delete C;
    return nnz;
}

template <typename SR, typename NT>
int64_t run_merge(int nlists, int64_t m, int64_t n, const int64_t *const *cps, const int64_t *const *ris,
                  const void *const *vals)
{
    std::vector<SpTuples<int64_t, NT> *> lists;
    for (int k = 0; k < nlists; ++k) {
        auto t = csc_to_tuples<NT>(n, cps[k], ris[k], vals[k]);
        auto *arr = new std::tuple<int64_t, int64_t, NT>[t.size()];
        std::copy(t.begin(), t.end(), arr);
        lists.push_back(new SpTuples<int64_t, NT>((int64_t)t.size(), m, n, arr, true, false));
    }
    double t0 = now();
    SpTuples<int64_t, NT> *C = MultiwayMerge<SR>(lists, m, n, false);
    g_res.seconds = now() - t0;
    store_tuples(C);
    const int64_t nnz = C->getnnz();
    if (nlists != 1 || C != lists[0]) delete C;
    for (auto *L : lists) delete L;
    return nnz;
}

template <typename SR, typename NT>
int run_spmv(int64_t m, int64_t n, const int64_t *cp, const int64_t *ri, const void *v, const void *x, void *y)
{
    std::unique_ptr<SpDCCols<int64_t, NT>> A(make_dcsc<NT>(m, n, cp, ri, v));
    double t0 = now();
    dcsc_gespmv<SR>(*A, static_cast<const NT *>(x), static_cast<NT *>(y));
    g_res.seconds = now() - t0;
    return 0;
}

}  // namespace

template <typename SR, typename NT, typename VT>
static int64_t spmspv_bucket(int64_t m, int64_t n, const int64_t *Acp, const int64_t *Ari, const void *Av,
                             const int32_t *indx, const VT *numx, int32_t veclen)
{
    std::unique_ptr<SpCCols<int64_t, NT>> A(make_csc<NT>(m, n, Acp, Ari, Av));
    PreAllocatedSPA<VT> SPA(*A, 32);
    std::vector<int32_t> indy;
    std::vector<VT> numy;
    double t0 = now();
    SpMXSpV_Bucket<SR>(*A->GetCSC(), (int32_t)m, indx, numx, veclen, indy, numy, SPA);
    g_res.seconds = now() - t0;
    g_res.rows.assign(indy.begin(), indy.end());
    g_res.cols.clear();
    g_res.vals.resize(numy.size() * sizeof(VT));
    std::memcpy(g_res.vals.data(), numy.data(), numy.size() * sizeof(VT));
    return (int64_t)indy.size();
}

extern "C" {

// Semiring codes: 0 PlusTimes<double>, 1 PlusTimes<float>, 2 PlusTimes<int64>,
// 3 MinPlus<double>, 4 Select2ndMin<int64>, 5 PlusTimes<bool> (or/and),
// 6 MinPlus<int64>.
// Variant codes: 0 LocalHybridSpGEMM (DCSC), 1 LocalSpGEMM (heap),
// 2 LocalSpGEMMHash sorted, 3 LocalSpGEMMHash unsorted, 4 CSC
// LocalHybridSpGEMM, 5 PSpGEMM on a 1x1 grid.
int64_t ref_spgemm(int variant, int sr, int64_t m, int64_t k, int64_t n, const int64_t *Acp, const int64_t *Ari,
                   const void *Av, const int64_t *Bcp, const int64_t *Bri, const void *Bv, int reps)
{
    if (reps < 1) reps = 1;
    switch (sr) {
        case 0: return run_spgemm<PlusTimesSRing<double, double>, double>(variant, m, k, n, Acp, Ari, Av, Bcp, Bri, Bv, reps);
        case 1: return run_spgemm<PlusTimesSRing<float, float>, float>(variant, m, k, n, Acp, Ari, Av, Bcp, Bri, Bv, reps);
        case 2: return run_spgemm<PlusTimesSRing<int64_t, int64_t>, int64_t>(variant, m, k, n, Acp, Ari, Av, Bcp, Bri, Bv, reps);
        case 3: return run_spgemm<MinPlusSRing<double, double>, double>(variant, m, k, n, Acp, Ari, Av, Bcp, Bri, Bv, reps);
        case 4: return run_spgemm<HarnessSelect2ndMinSR<int64_t, int64_t>, int64_t>(variant, m, k, n, Acp, Ari, Av, Bcp, Bri, Bv, reps);
        case 5: return run_spgemm<PlusTimesSRing<bool, bool>, bool>(variant, m, k, n, Acp, Ari, Av, Bcp, Bri, Bv, reps);
        case 6: return run_spgemm<MinPlusSRing<int64_t, int64_t>, int64_t>(variant, m, k, n, Acp, Ari, Av, Bcp, Bri, Bv, reps);
        default: return -1;
    }
}

// MultiwayMerge<SR> (MultiwayMerge.h:428) of nlists CSC matrices of one
// shape; result (column-major tuples) in g_res.
int64_t ref_multiway_merge(int sr, int nlists, int64_t m, int64_t n, const int64_t *const *cps,
                           const int64_t *const *ris, const void *const *vals)
{
    switch (sr) {
        case 0: return run_merge<PlusTimesSRing<double, double>, double>(nlists, m, n, cps, ris, vals);
        case 1: return run_merge<PlusTimesSRing<float, float>, float>(nlists, m, n, cps, ris, vals);
        case 2: return run_merge<PlusTimesSRing<int64_t, int64_t>, int64_t>(nlists, m, n, cps, ris, vals);
        case 3: return run_merge<MinPlusSRing<double, double>, double>(nlists, m, n, cps, ris, vals);
        case 4: return run_merge<HarnessSelect2ndMinSR<int64_t, int64_t>, int64_t>(nlists, m, n, cps, ris, vals);
        case 5: return run_merge<PlusTimesSRing<bool, bool>, bool>(nlists, m, n, cps, ris, vals);
        case 6: return run_merge<MinPlusSRing<int64_t, int64_t>, int64_t>(nlists, m, n, cps, ris, vals);
        default: return -1;
    }
}

// dcsc_gespmv<SR> (Friends.h:63): y <- y (+) A x in place.
int ref_spmv(int sr, int64_t m, int64_t n, const int64_t *cp, const int64_t *ri, const void *v, const void *x,
             void *y)
{
    switch (sr) {
        case 0: return run_spmv<PlusTimesSRing<double, double>, double>(m, n, cp, ri, v, x, y);
        case 1: return run_spmv<PlusTimesSRing<float, float>, float>(m, n, cp, ri, v, x, y);
        case 2: return run_spmv<PlusTimesSRing<int64_t, int64_t>, int64_t>(m, n, cp, ri, v, x, y);
        case 3: return run_spmv<MinPlusSRing<double, double>, double>(m, n, cp, ri, v, x, y);
        case 4: return run_spmv<HarnessSelect2ndMinSR<int64_t, int64_t>, int64_t>(m, n, cp, ri, v, x, y);
        case 5: return run_spmv<PlusTimesSRing<bool, bool>, bool>(m, n, cp, ri, v, x, y);
        case 6: return run_spmv<MinPlusSRing<int64_t, int64_t>, int64_t>(m, n, cp, ri, v, x, y);
        default: return -1;
    }
}

void ref_result_copy(int64_t *rows, int64_t *cols, void *vals)
{
    if (rows) std::memcpy(rows, g_res.rows.data(), g_res.rows.size() * sizeof(int64_t));
    if (cols) std::memcpy(cols, g_res.cols.data(), g_res.cols.size() * sizeof(int64_t));
    if (vals) std::memcpy(vals, g_res.vals.data(), g_res.vals.size());
}

double ref_result_seconds() { return g_res.seconds; }

int64_t ref_result_nnz() { return (int64_t)g_res.rows.size(); }

// which = 0: estimateFLOP per nonempty column of B; 1: estimateNNZ_Hash.
// Pattern-only (values ignored).  Returns nzc(B).
int64_t ref_colstats(int which, int64_t m, int64_t k, int64_t n, const int64_t *Acp, const int64_t *Ari,
                     const int64_t *Bcp, const int64_t *Bri, int64_t *out)
{
    std::unique_ptr<SpDCCols<int64_t, double>> A(make_dcsc<double>(m, k, Acp, Ari, nullptr));
    std::unique_ptr<SpDCCols<int64_t, double>> B(make_dcsc<double>(k, n, Bcp, Bri, nullptr));
    if (A->isZero() || B->isZero()) return 0;
    int64_t nzc = B->GetDCSC()->nzc;
    int64_t *flop = estimateFLOP(*A, *B);
    if (which == 0) {
        std::memcpy(out, flop, nzc * sizeof(int64_t));
    } else {
        int64_t *nnz = estimateNNZ_Hash(*A, *B, flop);
        std::memcpy(out, nnz, nzc * sizeof(int64_t));
        delete[] nnz;
    }
    delete[] flop;
    return nzc;
}

// y = A x over SelectMinSR with the CSC bucket algorithm.  x: int32 indices,
// int64 values.  Result in g_res.rows (row ids) and g_res.vals (int64).
int64_t ref_spmspv_bucket(int64_t m, int64_t n, const int64_t *Acp, const int64_t *Ari, const int32_t *indx,
                          const int64_t *numx, int32_t veclen, int buckets)
{
    std::unique_ptr<SpCCols<int64_t, bool>> A(make_csc<bool>(m, n, Acp, Ari, nullptr));
    PreAllocatedSPA<int64_t> SPA(*A, buckets);
    std::vector<int32_t> indy;
    std::vector<int64_t> numy;
    double t0 = now();
    SpMXSpV_Bucket<HarnessSelectMinSR>(*A->GetCSC(), (int32_t)m, indx, numx, veclen, indy, numy, SPA);
    g_res.seconds = now() - t0;
    g_res.rows.assign(indy.begin(), indy.end());
    g_res.cols.clear();
    g_res.vals.resize(numy.size() * sizeof(int64_t));
    std::memcpy(g_res.vals.data(), numy.data(), numy.size() * sizeof(int64_t));
    return (int64_t)indy.size();
}

// y = A x over the other SpMXSpV semirings: sx 1 Select2ndSRing<bool,int64,
// int64> through the boolean DCSC SpMXSpV with the optbuf outputs and one
// receiver (what TopDownBFS's LocalSpMV calls, BFSFriends.h:198-207); sx 2
// SelectMaxSRing<bool,int64> and sx 3 PlusTimesSRing (vt 0 double, 1 float,
// 2 int64) through SpMXSpV_Bucket.  Result in g_res.rows / g_res.vals.
int64_t ref_spmspv_sr(int sx, int vt, int64_t m, int64_t n, const int64_t *Acp, const int64_t *Ari, const void *Av,
                      const int32_t *indx, const void *numx, int32_t veclen)
{
    if (sx == 1) {
        std::unique_ptr<SpDCCols<int64_t, bool>> A(make_dcsc<bool>(m, n, Acp, Ari, nullptr));
        std::vector<int32_t> indy(m > 0 ? m : 1);
        std::vector<int64_t> numy(m > 0 ? m : 1);
        int cnts[1] = {0}, dspls[1] = {0};
        double t0 = now();
        if (A->getnnz() > 0 && veclen > 0)
            SpMXSpV<Select2ndSRing<bool, int64_t, int64_t>>(*A->GetDCSC(), (int32_t)m, indx,
                                                             static_cast<const int64_t *>(numx), veclen, indy.data(),
                                                             numy.data(), cnts, dspls, 1);
        g_res.seconds = now() - t0;
        g_res.rows.assign(indy.begin(), indy.begin() + cnts[0]);
        g_res.cols.clear();
        g_res.vals.resize(cnts[0] * sizeof(int64_t));
        std::memcpy(g_res.vals.data(), numy.data(), cnts[0] * sizeof(int64_t));
        return cnts[0];
    }
    if (sx == 2)
        return spmspv_bucket<SelectMaxSRing<bool, int64_t>, bool, int64_t>(m, n, Acp, Ari, nullptr, indx,
                                                                           static_cast<const int64_t *>(numx), veclen);
    if (sx == 3 && vt == 0)
        return spmspv_bucket<PlusTimesSRing<double, double>, double, double>(m, n, Acp, Ari, Av, indx,
                                                                            static_cast<const double *>(numx), veclen);
    if (sx == 3 && vt == 1)
        return spmspv_bucket<PlusTimesSRing<float, float>, float, float>(m, n, Acp, Ari, Av, indx,
                                                                        static_cast<const float *>(numx), veclen);
    if (sx == 3 && vt == 2)
        return spmspv_bucket<PlusTimesSRing<int64_t, int64_t>, int64_t, int64_t>(
            m, n, Acp, Ari, Av, indx, static_cast<const int64_t *>(numx), veclen);
    return -1;
}

// BFS from `source` over the symmetric pattern A, as the BFS_CSC loop of
// SpMSpVBench.cpp:105-156: fringe.setNumToInd(); SpMV<SelectMinSR>;
// EWiseMult(fringe, parents, exclude=true, -1); parents.Set(fringe).
// parents_out[n] receives the parent array (-1 = unreached); returns the
// number of level iterations.  levels_out[n] (optional) receives the loop
// iteration (1-based) at which each vertex first received a parent (0 for
// the source itself if it never receives one, -1 if unreached).
int ref_bfs_selectmin(int64_t n, const int64_t *Acp, const int64_t *Ari, int64_t source, int64_t *parents_out,
                      int64_t *levels_out)
{
    auto grid = std::make_shared<CommGrid>(MPI_COMM_WORLD, 1, 1);
    typedef SpParMat<int64_t, bool, SpCCols<int64_t, bool>> ParCSC;
    ParCSC A(make_csc<bool>(n, n, Acp, Ari, nullptr), grid);
    int nthreads = 1;
#ifdef THREADED
#pragma omp parallel
    {
        nthreads = omp_get_num_threads();
    }
#endif
    PreAllocatedSPA<int64_t> SPA(A.seq(), nthreads * 4);
    FullyDistVec<int64_t, int64_t> parents(grid, n, (int64_t)-1);
    FullyDistSpVec<int64_t, int64_t> fringe(grid, n);
    std::vector<int64_t> level(n, -1);
    if (levels_out) level[source] = 0;
    double t0 = now();
    fringe.SetElement(source, source);
    int iterations = 0;
    while (fringe.getnnz() > 0) {
        fringe.setNumToInd();
        SpMV<HarnessSelectMinSR>(A, fringe, fringe, false, SPA);
        fringe = EWiseMult(fringe, parents, true, (int64_t)-1);
        parents.Set(fringe);
        iterations++;
        if (levels_out) {
            const std::vector<int64_t> &ind = fringe.GetLocalInd();
            for (int64_t v : ind)
                if (level[v] < 0) level[v] = iterations;
        }
    }
    g_res.seconds = now() - t0;
    for (int64_t i = 0; i < n; ++i) parents_out[i] = parents.GetElement(i);
    if (levels_out) std::memcpy(levels_out, level.data(), n * sizeof(int64_t));
    return iterations;
}

// MCL expansion on a 1x1 grid as MCL.cpp:573 calls it with one phase:
// MemEfficientSpGEMM<PlusTimesSRing<float,float>>(A, A, phases=1,
// hardThreshold, selectNum, recoverNum, recoverPct, kselectVersion=1,
// computationKernel=1, perProcessMemory).  Result in g_res (DCSC order).
int64_t ref_mcl_expand(int64_t n, const int64_t *Acp, const int64_t *Ari, const float *Av, float thr,
                       int64_t select, int64_t recover_num, float recover_pct)
{
    auto grid = std::make_shared<CommGrid>(MPI_COMM_WORLD, 1, 1);
    typedef SpParMat<int64_t, float, SpDCCols<int64_t, float>> PM;
    PM A(make_dcsc<float>(n, n, Acp, Ari, Av), grid);
    PM B(A);
    double t0 = now();
    PM C = MemEfficientSpGEMM<PlusTimesSRing<float, float>, float, SpDCCols<int64_t, float>>(
        A, B, 1, thr, select, recover_num, recover_pct, 1, 1, (int64_t)0);
    g_res.seconds = now() - t0;
    store_dcsc(C.seq());
    return C.seq().getnnz();
}

// MakeColStochastic, Chaos and Inflate as Applications/MCL.cpp:389-449
// writes them (that file holds a main() and cannot be included): the
// reference's own SpParMat::Reduce, DimApply and Apply do the arithmetic.
typedef SpParMat<int64_t, float, SpDCCols<int64_t, float>> MclMat;

static void mcl_make_col_stochastic(MclMat &A)
{
    FullyDistVec<int64_t, float> colsums = A.Reduce(Column, std::plus<float>(), 0.0);
    colsums.Apply(safemultinv<float>());
    A.DimApply(Column, colsums, std::multiplies<float>());
}

static float mcl_chaos(MclMat &A)
{
    FullyDistVec<int64_t, float> colssqs = A.Reduce(Column, std::plus<float>(), 0.0, [](float val) { return pow(val, 2); });
    FullyDistVec<int64_t, float> colmaxs = A.Reduce(Column, maximum<float>(), 0.0);
    colmaxs -= colssqs;
    FullyDistVec<int64_t, float> nnzPerColumn = A.Reduce(Column, std::plus<float>(), 0.0, [](float val) { return 1.0; });
    colmaxs.EWiseApply(nnzPerColumn, std::multiplies<float>());
    return colmaxs.Reduce(maximum<float>(), 0.0);
}

static void mcl_inflate(MclMat &A, double power)
{
    A.Apply([power](float val) { return pow(val, power); });
}

// The HipMCL loop from the loop-adjusted matrix on (MCL.cpp:526-626 with
// layers == 1, phases == 1, kselectVersion 1, computationKernel 1).  mode 0
// runs the loop (at most max_iter iterations when max_iter > 0) and returns
// the iteration count, the last chaos in *chaos; mode 1 applies only
// MakeColStochastic, mode 2 only Inflate(inflation), mode 3 only Chaos (into
// *chaos).  The matrix ends in g_res (DCSC order).
int64_t ref_mcl_iterate(int64_t n, const int64_t *Acp, const int64_t *Ari, const float *Av, double inflation,
                        float thr, int64_t select, int64_t recover_num, float recover_pct, int64_t max_iter, int mode,
                        float *chaos_out)
{
    auto grid = std::make_shared<CommGrid>(MPI_COMM_WORLD, 1, 1);
    MclMat A(make_dcsc<float>(n, n, Acp, Ari, Av), grid);
    int64_t it = 0;
    double t0 = now();
    if (mode == 1) {
        mcl_make_col_stochastic(A);
    } else if (mode == 2) {
        mcl_inflate(A, inflation);
    } else if (mode == 3) {
        *chaos_out = mcl_chaos(A);
    } else {
        mcl_make_col_stochastic(A);
        const int64_t nnz = A.getnnz(), nv = A.getnrow();
        if (nnz / nv > std::max(select, recover_num))
            MCLPruneRecoverySelect(A, thr, select, recover_num, recover_pct, 1);
        float chaos = 1;
        while (chaos > 0.0001 && (max_iter <= 0 || it < max_iter)) {
            A = MemEfficientSpGEMM<PlusTimesSRing<float, float>, float, SpDCCols<int64_t, float>>(
                A, A, 1, thr, select, recover_num, recover_pct, 1, 1, (int64_t)0);
            mcl_make_col_stochastic(A);
            chaos = mcl_chaos(A);
            mcl_inflate(A, inflation);
            mcl_make_col_stochastic(A);
            ++it;
        }
        *chaos_out = chaos;
    }
    g_res.seconds = now() - t0;
    store_dcsc(A.seq());
    return it;
}

int ref_num_threads()
{
    int nthreads = 1;
#ifdef THREADED
#pragma omp parallel
    {
        nthreads = omp_get_num_threads();
    }
#endif
    return nthreads;
}

}  // extern "C"
