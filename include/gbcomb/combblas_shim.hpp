/* Drop-in GPU forms of CombBLAS's node-local multiplies.
 *
 * Include this header after the CombBLAS headers (it names
 * combblas::SpDCCols, SpCCols, SpTuples, Csc, PreAllocatedSPA and the stock
 * semirings) and call gbcomb::X where the reference calls combblas::X:
 *
 *   gbcomb::LocalHybridSpGEMM<SR, NTO>(A, B, clearA, clearB)   mtSpGEMM.h:213-217
 *   gbcomb::LocalSpGEMM<SR, NTO>(A, B, clearA, clearB)         mtSpGEMM.h:74-78
 *   gbcomb::LocalSpGEMMHash<SR, NTO>(A, B, clearA, clearB, sort) mtSpGEMM.h:463-467
 *   gbcomb::LocalHybridSpGEMM<SR, NTO>(SpCCols A, SpCCols B, ...)  mtSpGEMM.h:1142-1152
 *   gbcomb::SpMXSpV<SR>(Csc, mA, indx, numx, veclen, indy, numy, SPA)  SpImpl.h:115-124
 *   gbcomb::SpMXSpV<SR>(Dcsc, mA, indx, numx, veclen, indy, numy, SPA)  SpImpl.h:49-56
 *   gbcomb::SpMXSpV<SR>(Dcsc, mA, indx, numx, veclen, indy*, numy*, cnts, dspls, p_c)  SpImpl.h:59-65
 *   gbcomb::SpMXSpV_ForThreading<SR>(Dcsc or Csc piece, ..., offset[, SPA buffers])  SpImpl.h:68-82, 126-142
 *   gbcomb::MultiwayMerge<SR>(ArrSpTups, mdim, ndim, delarrs)  MultiwayMerge.h:428-708
 *   gbcomb::dcsc_gespmv<SR>(A, x, y)                           Friends.h:63-77
 *
 * Same arguments, same ownership (inputs borrowed; clearA / clearB delete
 * them; the returned SpTuples owns a tuple array from ::operator new with
 * isOpNew = true; an empty operand gives new SpTuples(0, m, n); SpMXSpV
 * appends to indy / numy), same results.  A call runs on the GPU when its
 * (semiring, index, value) combination is registered in gbcomb::semiring_of
 * and the index type is int64_t; every other combination falls through to
 * the reference template unchanged.  A nonzero status from the C ABI is
 * reported on stderr and thrown as std::runtime_error (the reference's
 * local kernels have no error path; its distributed layer aborts).
 *
 * Stock semirings registered here: PlusTimesSRing<double,double>,
 * <float,float>, <int64_t,int64_t>; MinPlusSRing<double,double>,
 * <int64_t,int64_t>.  Application-defined semirings (Select2ndMinSR of
 * FastSV.h / CC.h, SelectMinSR of SpMSpVBench.cpp, boolean or-and) are
 * registered by the application with GBCOMB_REGISTER_SEMIRING.
 */
#pragma once

#include <cstdint>
#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "../gbcomb.h"

namespace gbcomb {

// (semiring, value type) codes of the C ABI for a CombBLAS semiring type;
// sr < 0: not registered (the reference template runs).
template <class SR>
struct semiring_of {
    static constexpr int sr = -1;
    static constexpr int vt = -1;
};

template <int VT>
struct value_c;
template <>
struct value_c<GBC_F64> {
    typedef double type;
};
template <>
struct value_c<GBC_F32> {
    typedef float type;
};
template <>
struct value_c<GBC_I64> {
    typedef int64_t type;
};
template <>
struct value_c<GBC_BOOL> {
    typedef bool type;
};

}  // namespace gbcomb

#define GBCOMB_REGISTER_SEMIRING(SRTYPE, SR_CODE, VT_CODE) \
    namespace gbcomb {                                     \
    template <>                                            \
    struct semiring_of<SRTYPE> {                           \
        static constexpr int sr = (SR_CODE);               \
        static constexpr int vt = (VT_CODE);               \
    };                                                     \
    }

// SRTYPE must be a single token or parenthesis-free name: use a typedef for
// a template with several arguments, e.g.
//   typedef combblas::Select2ndMinSR<int64_t, int64_t> S2M;
//   GBCOMB_REGISTER_SEMIRING(S2M, GBC_SR_SELECT2NDMIN, GBC_I64)

namespace gbcomb {

#define GBCOMB_STOCK(T1, T2, SRT, SR_CODE, VT_CODE) \
    template <>                                      \
    struct semiring_of<combblas::SRT<T1, T2>> {      \
        static constexpr int sr = (SR_CODE);         \
        static constexpr int vt = (VT_CODE);         \
    };
GBCOMB_STOCK(double, double, PlusTimesSRing, GBC_SR_PLUSTIMES, GBC_F64)
GBCOMB_STOCK(float, float, PlusTimesSRing, GBC_SR_PLUSTIMES, GBC_F32)
GBCOMB_STOCK(int64_t, int64_t, PlusTimesSRing, GBC_SR_PLUSTIMES, GBC_I64)
GBCOMB_STOCK(double, double, MinPlusSRing, GBC_SR_MINPLUS, GBC_F64)
GBCOMB_STOCK(int64_t, int64_t, MinPlusSRing, GBC_SR_MINPLUS, GBC_I64)
#undef GBCOMB_STOCK

namespace detail {

inline void check(int rc, const char *what)
{
    if (rc != GBC_OK) {
        std::string msg = std::string(what) + ": " + gbc_last_error();
        std::fprintf(stderr, "gbcomb: %s\n", msg.c_str());
        throw std::runtime_error(msg);
    }
}

// One library context per process (device 0 unless gbcomb::set_device ran
// first); the reference calls its local kernels from a single thread.
inline gbc_context *&context_slot()
{
    static gbc_context *ctx = nullptr;
    return ctx;
}

inline int &device_slot()
{
    static int dev = 0;
    return dev;
}

inline gbc_context *context()
{
    gbc_context *&c = context_slot();
    if (!c) check(gbc_context_create(&c, device_slot()), "gbc_context_create");
    return c;
}

// Offload test: registered semiring, int64 indices, every value type equal
// to the semiring's.
template <class SR, class NTO, class IT, class NT1, class NT2>
constexpr bool offloaded()
{
    if constexpr (semiring_of<SR>::sr < 0) {
        return false;
    } else {
        typedef typename value_c<semiring_of<SR>::vt>::type V;
        return std::is_same<IT, int64_t>::value && std::is_same<NT1, V>::value && std::is_same<NT2, V>::value &&
               std::is_same<NTO, V>::value;
    }
}

// Host views of the reference's storage as C-ABI descriptors (no copies).
// Dcsc (Dcsc.h): cp[nzc+1] pointers of the nzc nonempty columns jc[nzc],
// ir / numx the entries.  Csc (csc.h): jc[n+1] holds the column pointers.
// values = false leaves num null (pattern operands).
template <class IT, class NT>
gbc_matrix view_dcsc(const combblas::Dcsc<IT, NT> *d, int64_t nrow, int64_t ncol, bool values = true)
{
    gbc_matrix g{};
    g.nrow = nrow;
    g.ncol = ncol;
    g.nzc = d ? d->nzc : 0;
    g.nnz = d ? d->nz : 0;
    g.cp = d ? d->cp : nullptr;
    g.jc = d ? d->jc : nullptr;
    g.ir = d ? d->ir : nullptr;
    g.num = d && values ? static_cast<const void *>(d->numx) : nullptr;
    g.where = GBC_HOST;
    return g;
}

template <class IT, class NT>
gbc_matrix view_csc(const combblas::Csc<IT, NT> *c, int64_t nrow, int64_t ncol, bool values = true)
{
    gbc_matrix g{};
    g.nrow = nrow;
    g.ncol = ncol;
    g.nzc = ncol;
    g.nnz = c ? c->nz : 0;
    g.cp = c ? c->jc : nullptr;  // Csc::jc holds the column pointers
    g.jc = nullptr;
    g.ir = c ? c->ir : nullptr;
    g.num = c && values ? static_cast<const void *>(c->num) : nullptr;
    g.where = GBC_HOST;
    return g;
}

template <class IT, class NT>
gbc_matrix view(const combblas::SpDCCols<IT, NT> &M)
{
    return view_dcsc(M.GetDCSC(), M.getnrow(), M.getncol());
}

template <class IT, class NT>
gbc_matrix view(const combblas::SpCCols<IT, NT> &M)
{
    return view_csc(M.GetCSC(), M.getnrow(), M.getncol());
}

// A result's arrays (cp[nzc+1], jc[nzc] column ids, ir, num) as the
// reference's tuple array: (row, col, value) in column-major order, rows
// ascending within a column.  opnew: storage from ::operator new (the
// SpTuples then takes isOpNew = true, as mtSpGEMM.h's products do), else
// from new[] (MultiwayMerge.h's result).
template <class IT, class NT>
std::tuple<IT, IT, NT> *tuples_of(int64_t nzc, const int64_t *cp, const int64_t *jc, const int64_t *ir, const NT *num,
                                  bool opnew)
{
    typedef std::tuple<IT, IT, NT> T;
    const int64_t nnz = cp[nzc];
    T *tuples = opnew ? static_cast<T *>(::operator new(sizeof(T) * (nnz > 0 ? nnz : 1)))
                      : new T[nnz > 0 ? nnz : 1];
    for (int64_t k = 0; k < nzc; ++k)
        for (int64_t p = cp[k]; p < cp[k + 1]; ++p) {
            if (opnew)
                new (tuples + p) T((IT)ir[p], (IT)jc[k], num[p]);
            else
                tuples[p] = T((IT)ir[p], (IT)jc[k], num[p]);
        }
    return tuples;
}

// A column-sorted SpTuples as a host CSC (arrays owned by the struct).
template <class NT>
struct TupleCsc {
    std::vector<int64_t> cp, ir;
    std::unique_ptr<NT[]> num;  // NT may be bool: no std::vector
    gbc_matrix g{};
};

template <class IT, class NT>
void csc_of_tuples(const combblas::SpTuples<IT, NT> &T, IT mdim, IT ndim, TupleCsc<NT> &out)
{
    const int64_t nnz = T.getnnz();
    out.cp.assign(ndim + 1, 0);
    out.ir.resize(nnz);
    out.num.reset(new NT[nnz > 0 ? nnz : 1]);
    for (int64_t p = 0; p < nnz; ++p) {
        ++out.cp[T.colindex(p) + 1];
        out.ir[p] = T.rowindex(p);
        out.num[p] = T.numvalue(p);
    }
    for (IT j = 0; j < ndim; ++j) out.cp[j + 1] += out.cp[j];
    gbc_matrix &g = out.g;
    g = gbc_matrix{};
    g.nrow = mdim;
    g.ncol = ndim;
    g.nzc = ndim;
    g.nnz = nnz;
    g.cp = out.cp.data();
    g.jc = nullptr;
    g.ir = nnz ? out.ir.data() : nullptr;
    g.num = nnz ? static_cast<const void *>(out.num.get()) : nullptr;
    g.where = GBC_HOST;
}

// Rows of y = A x (ascending, global) split among p_c receivers as the
// optbuf SpMXSpV does (SpImpl.cpp:222-272): owner = min(row / (mA / p_c),
// p_c - 1); each receiver's rows ascending and local to its offset;
// cnts[p] entries land at indy / numy + dspls[p].
template <class OVT>
void split_rows(const std::vector<int32_t> &r, const std::vector<OVT> &v, int32_t mA, int32_t *indy, OVT *numy,
                int *cnts, const int *dspls, int p_c)
{
    const int32_t perproc = p_c > 0 ? mA / p_c : mA;
    for (int p = 0; p < p_c; ++p) cnts[p] = 0;
    size_t k = 0;
    for (int p = 0; p < p_c; ++p) {
        const int32_t offset = perproc * p;
        while (k < r.size() && (p == p_c - 1 || perproc == 0 || r[k] / perproc <= p)) {
            indy[dspls[p] + cnts[p]] = r[k] - offset;
            numy[dspls[p] + cnts[p]] = v[k];
            ++cnts[p];
            ++k;
        }
    }
}

// Run the product and wrap it as the reference does (tuples_of).
template <class SR, class NTO, class IT>
combblas::SpTuples<IT, NTO> *multiply(const gbc_matrix &A, const gbc_matrix &B, int sorted)
{
    gbc_spgemm_opts opt{GBC_SIZING_EXACT, sorted, 1, 0, -1, -1};
    gbc_result *C = nullptr;
    check(gbc_spgemm(context(), semiring_of<SR>::sr, semiring_of<SR>::vt, &A, &B, &opt, &C, nullptr), "gbc_spgemm");
    int64_t nrow = 0, ncol = 0, nzc = 0, nnz = 0;
    int vt = 0;
    gbc_result_info(C, &nrow, &ncol, &nzc, &nnz, &vt);
    std::vector<int64_t> cp(nzc + 1), jc(nzc), ir(nnz);
    std::unique_ptr<NTO[]> num(new NTO[nnz > 0 ? nnz : 1]);  // NTO may be bool: no std::vector
    int rc = gbc_result_copy(C, cp.data(), nzc ? jc.data() : nullptr, nnz ? ir.data() : nullptr,
                             nnz ? static_cast<void *>(num.get()) : nullptr, GBC_HOST);
    gbc_result_free(C);
    check(rc, "gbc_result_copy");
    return new combblas::SpTuples<IT, NTO>(nnz, (IT)A.nrow, (IT)B.ncol,
                                           tuples_of<IT, NTO>(nzc, cp.data(), jc.data(), ir.data(), num.get(), true),
                                           true, true);
}

template <class SR, class NTO, class M1, class M2>
auto run(const M1 &A, const M2 &B, bool clearA, bool clearB, int sorted)
{
    typedef decltype(A.getnrow()) IT;
    const IT m = A.getnrow(), n = B.getncol();
    combblas::SpTuples<IT, NTO> *out;
    if (A.isZero() || B.isZero())
        out = new combblas::SpTuples<IT, NTO>(0, m, n);
    else
        out = multiply<SR, NTO, IT>(view(A), view(B), sorted);
    if (clearA) delete const_cast<M1 *>(&A);
    if (clearB) delete const_cast<M2 *>(&B);
    return out;
}

}  // namespace detail

inline void set_device(int device) { detail::device_slot() = device; }

// PlusTimes fp64 accumulation of the offloaded products: GBC_FOLD_EXACT (the
// library default: exact sum of the rounded products, rounded once) or
// GBC_FOLD_ORDERED (the reference's hash-path fold, mtSpGEMM.h:396-412, bit
// for bit).
inline void set_fold(int fold) { detail::check(gbc_context_set_fold(detail::context(), fold), "gbc_context_set_fold"); }

template <class SR, class NTO, class IT, class NT1, class NT2>
combblas::SpTuples<IT, NTO> *LocalHybridSpGEMM(const combblas::SpDCCols<IT, NT1> &A,
                                               const combblas::SpDCCols<IT, NT2> &B, bool clearA, bool clearB,
                                               IT *aux = nullptr)
{
    if constexpr (detail::offloaded<SR, NTO, IT, NT1, NT2>())
        return detail::run<SR, NTO>(A, B, clearA, clearB, GBC_SORTED);
    else
        return combblas::LocalHybridSpGEMM<SR, NTO>(A, B, clearA, clearB, aux);
}

template <class SR, class NTO, class IT, class NT1, class NT2>
combblas::SpTuples<IT, NTO> *LocalSpGEMM(const combblas::SpDCCols<IT, NT1> &A, const combblas::SpDCCols<IT, NT2> &B,
                                         bool clearA, bool clearB)
{
    if constexpr (detail::offloaded<SR, NTO, IT, NT1, NT2>())
        return detail::run<SR, NTO>(A, B, clearA, clearB, GBC_SORTED);
    else
        return combblas::LocalSpGEMM<SR, NTO>(A, B, clearA, clearB);
}

// sort = false asks for the reference's unsorted hash output; the GPU path
// returns rows ascending either way (a valid unsorted order), and the
// SpTuples is flagged sorted as the reference flags it.
template <class SR, class NTO, class IT, class NT1, class NT2>
combblas::SpTuples<IT, NTO> *LocalSpGEMMHash(const combblas::SpDCCols<IT, NT1> &A,
                                             const combblas::SpDCCols<IT, NT2> &B, bool clearA, bool clearB,
                                             bool sort = true)
{
    if constexpr (detail::offloaded<SR, NTO, IT, NT1, NT2>())
        return detail::run<SR, NTO>(A, B, clearA, clearB, GBC_SORTED);
    else
        return combblas::LocalSpGEMMHash<SR, NTO>(A, B, clearA, clearB, sort);
}

template <class SR, class NTO, class IT, class NT1, class NT2>
combblas::SpTuples<IT, NTO> *LocalHybridSpGEMM(const combblas::SpCCols<IT, NT1> &A,
                                               const combblas::SpCCols<IT, NT2> &B, bool clearA, bool clearB)
{
    if constexpr (detail::offloaded<SR, NTO, IT, NT1, NT2>())
        return detail::run<SR, NTO>(A, B, clearA, clearB, GBC_SORTED);
    else
        return combblas::LocalHybridSpGEMM<SR, NTO>(A, B, clearA, clearB);
}

// Sum of column-sorted SpTuples of one shape, equal (row, col) combined by
// SR::add in list order.  One or no list, or a shape mismatch, behave as the
// reference (copy, empty result, message and an empty 0 x 0 result); the
// result's tuple array comes from new[] (isOpNew = false) as the
// reference's; delarrs deletes the inputs.  With three or more lists the
// reference combines equal keys in its heap's order, so PlusTimes sums of
// floating values can differ in the last bit.
template <class SR, class IT, class NT>
combblas::SpTuples<IT, NT> *MultiwayMerge(std::vector<combblas::SpTuples<IT, NT> *> &ArrSpTups, IT mdim = 0,
                                          IT ndim = 0, bool delarrs = false)
{
    constexpr bool gpu = detail::offloaded<SR, NT, IT, NT, NT>();
    const int nlists = (int)ArrSpTups.size();
    if constexpr (!gpu) {
        return combblas::MultiwayMerge<SR>(ArrSpTups, mdim, ndim, delarrs);
    } else {
        if (nlists <= 1) return combblas::MultiwayMerge<SR>(ArrSpTups, mdim, ndim, delarrs);
        for (int k = 0; k < nlists; ++k)
            if (mdim != ArrSpTups[k]->getnrow() || ndim != ArrSpTups[k]->getncol()) {
                std::fprintf(stderr, "Dimensions of SpTuples do not match on multiwayMerge()\n");
                return new combblas::SpTuples<IT, NT>(0, 0, 0);
            }
        // each list as a host CSC (tuples are column sorted)
        std::vector<detail::TupleCsc<NT>> lists(nlists);
        std::vector<gbc_matrix> mats(nlists);
        for (int k = 0; k < nlists; ++k) {
            detail::csc_of_tuples(*ArrSpTups[k], mdim, ndim, lists[k]);
            mats[k] = lists[k].g;
        }
        gbc_result *C = nullptr;
        detail::check(gbc_multiway_merge(detail::context(), semiring_of<SR>::sr, semiring_of<SR>::vt, nlists,
                                         mats.data(), mdim, ndim, &C, nullptr),
                      "gbc_multiway_merge");
        int64_t nrow = 0, ncol = 0, nzc = 0, nnz = 0;
        int vt = 0;
        gbc_result_info(C, &nrow, &ncol, &nzc, &nnz, &vt);
        std::vector<int64_t> cp(nzc + 1), jc(nzc), ir(nnz);
        std::unique_ptr<NT[]> num(new NT[nnz > 0 ? nnz : 1]);
        const int rc = gbc_result_copy(C, cp.data(), nzc ? jc.data() : nullptr, nnz ? ir.data() : nullptr,
                                       nnz ? static_cast<void *>(num.get()) : nullptr, GBC_HOST);
        gbc_result_free(C);
        detail::check(rc, "gbc_result_copy");
        auto *tuples = detail::tuples_of<IT, NT>(nzc, cp.data(), jc.data(), ir.data(), num.get(), false);
        if (delarrs)
            for (int k = 0; k < nlists; ++k) delete ArrSpTups[k];
        return new combblas::SpTuples<IT, NT>(nnz, mdim, ndim, tuples, true, false);
    }
}

// ------------------------------------------------------------------ SpMSpV
// Semiring code for the sparse-vector multiplies: the stock boolean
// Select2ndSRing (TopDownBFS, BFSFriends.h:198-207) and SelectMaxSRing, or a
// registered Select2ndMin / PlusTimes semiring.
template <class SR>
struct spmspv_of {
    static constexpr int sr = semiring_of<SR>::sr == GBC_SR_SELECT2NDMIN || semiring_of<SR>::sr == GBC_SR_PLUSTIMES
                                  ? semiring_of<SR>::sr
                                  : -1;
};
template <class T1, class T2>
struct spmspv_of<combblas::Select2ndSRing<bool, T1, T2>> {
    static constexpr int sr = GBC_SR_SELECT2ND;
};
template <class T2>
struct spmspv_of<combblas::SelectMaxSRing<bool, T2>> {
    static constexpr int sr = GBC_SR_SELECTMAX;
};

namespace detail {

// Device copies of the matrices multiplied so far, one gbc_spmspv_plan per
// matrix, keyed by the addresses and sizes of its arrays and a strided
// sample of their contents: a BFS that multiplies one matrix level after
// level copies it to the device once.
struct PlanKey {
    const void *cp, *ir, *num;
    int64_t m, n, nz, sample;
    int vt;
    bool operator<(const PlanKey &o) const
    {
        return std::tie(cp, ir, num, m, n, nz, sample, vt) < std::tie(o.cp, o.ir, o.num, o.m, o.n, o.nz, o.sample, o.vt);
    }
};

inline std::map<PlanKey, gbc_spmspv_plan *> &plan_cache()
{
    static std::map<PlanKey, gbc_spmspv_plan *> cache;
    return cache;
}

inline long long &plan_builds()
{
    static long long n = 0;
    return n;
}

inline int64_t sample_of(const int64_t *cp, int64_t ncp, const int64_t *ir, int64_t nz)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](uint64_t v) { h = (h ^ v) * 1099511628211ull; };
    for (int64_t k = 0; k < 64 && ncp > 0; ++k) mix((uint64_t)cp[(ncp - 1) * k / 63]);
    for (int64_t k = 0; k < 64 && nz > 0; ++k) mix((uint64_t)ir[(nz - 1) * k / 63]);
    return (int64_t)h;
}

inline std::map<PlanKey, gbc_spmv_plan *> &spmv_plan_cache()
{
    static std::map<PlanKey, gbc_spmv_plan *> cache;
    return cache;
}

inline gbc_spmv_plan *spmv_plan(const gbc_matrix &g, int vt)
{
    const PlanKey key{g.cp, g.ir, g.num, g.nrow, g.ncol, g.nnz, sample_of(g.cp, g.nzc + 1, g.ir, g.nnz), vt};
    auto it = spmv_plan_cache().find(key);
    if (it != spmv_plan_cache().end()) return it->second;
    gbc_spmv_plan *p = nullptr;
    check(gbc_spmv_plan_create(context(), vt, &g, &p), "gbc_spmv_plan_create");
    ++plan_builds();
    spmv_plan_cache()[key] = p;
    return p;
}

inline gbc_spmspv_plan *spmspv_plan(const gbc_matrix &g, int vt)
{
    const PlanKey key{g.cp, g.ir, g.num, g.nrow, g.ncol, g.nnz, sample_of(g.cp, g.nzc + 1, g.ir, g.nnz), vt};
    auto it = plan_cache().find(key);
    if (it != plan_cache().end()) return it->second;
    gbc_spmspv_plan *p = nullptr;
    check(gbc_spmspv_plan_create(context(), vt, &g, &p), "gbc_spmspv_plan_create");
    ++plan_builds();
    plan_cache()[key] = p;
    return p;
}

template <class SR, class NUM, class IVT, class OVT>
constexpr int spmspv_vt()
{
    constexpr int sr = spmspv_of<SR>::sr;
    if constexpr (sr == GBC_SR_SELECT2NDMIN || sr == GBC_SR_SELECT2ND || sr == GBC_SR_SELECTMAX) {
        return std::is_integral<IVT>::value && std::is_integral<OVT>::value && sizeof(IVT) <= 8 && sizeof(OVT) <= 8
                   ? GBC_BOOL
                   : -1;
    } else if constexpr (sr == GBC_SR_PLUSTIMES) {
        constexpr int vt = semiring_of<SR>::vt;
        if constexpr (vt == GBC_F64 || vt == GBC_F32 || vt == GBC_I64) {
            typedef typename value_c<vt>::type V;
            return std::is_same<NUM, V>::value && std::is_same<IVT, V>::value && std::is_same<OVT, V>::value ? vt
                                                                                                              : -1;
        } else {
            return -1;
        }
    } else {
        return -1;
    }
}

// Calls into the library from the SpMSpV drop-ins are serialised: the
// reference calls SpMXSpV_ForThreading from an OpenMP loop over row pieces,
// and the process has one device context and one plan cache.
inline std::mutex &call_mutex()
{
    static std::mutex m;
    return m;
}

// y = A x on the GPU into (row, value) arrays sorted by row; x entries whose
// column is not below g.ncol hit nothing and are dropped first.
template <class SR, class IVT, class OVT>
void spmspv_run(const gbc_matrix &g, int vt, const int32_t *indx, const IVT *numx, int32_t veclen,
                std::vector<int32_t> &rows, std::vector<OVT> &vals)
{
    std::lock_guard<std::mutex> lock(call_mutex());
    constexpr int sr = spmspv_of<SR>::sr;
    typedef typename std::conditional<sr == GBC_SR_PLUSTIMES, IVT, int64_t>::type XV;
    typedef typename std::conditional<sr == GBC_SR_PLUSTIMES, OVT, int64_t>::type YV;
    std::vector<int32_t> xi;
    std::vector<XV> xv;
    xi.reserve(veclen);
    xv.reserve(veclen);
    for (int32_t k = 0; k < veclen; ++k)
        if (indx[k] >= 0 && indx[k] < g.ncol) {
            xi.push_back(indx[k]);
            xv.push_back(static_cast<XV>(numx[k]));
        }
    gbc_spmspv_plan *p = spmspv_plan(g, vt);
    rows.resize(g.nrow > 0 ? g.nrow : 1);
    std::vector<YV> yv(g.nrow > 0 ? g.nrow : 1);
    int32_t ny = 0;
    check(gbc_spmspv(context(), p, sr, xi.data(), xv.data(), (int32_t)xi.size(), rows.data(), yv.data(), &ny,
                     GBC_HOST),
          "gbc_spmspv");
    rows.resize(ny);
    vals.resize(ny);
    for (int32_t k = 0; k < ny; ++k) vals[k] = static_cast<OVT>(yv[k]);
}

// A row piece's entries (rows ascending, local to the piece) as the
// threaded SpMSpV returns them: each row plus the piece's offset; replacing
// indy / numy (the boolean SPA version, SpImpl.cpp:311-317) or appended to
// them (the heap version, SpImpl.cpp:362-384, whose callers pass them empty).
template <class OVT>
void shift_rows(const std::vector<int32_t> &r, const std::vector<OVT> &v, int32_t offset, std::vector<int32_t> &indy,
                std::vector<OVT> &numy, bool append)
{
    if (!append) {
        indy.clear();
        numy.clear();
    }
    indy.reserve(indy.size() + r.size());
    numy.reserve(numy.size() + r.size());
    for (size_t k = 0; k < r.size(); ++k) {
        indy.push_back(r[k] + offset);
        numy.push_back(v[k]);
    }
}

// Value code of a threaded SpMSpV over a Dcsc piece: the reference computes
// it only for boolean matrices (SpImpl.cpp:276-324; other value types print
// "not yet supported"), folding x values in column order like the optbuf
// version.
template <class SR, class NUM, class IVT, class OVT>
constexpr int threaded_dcsc_vt()
{
    return std::is_same<NUM, bool>::value ? spmspv_vt<SR, NUM, IVT, OVT>() : -1;
}

// ... for the heap versions (the threaded Csc one, SpImpl.cpp:345-386, and
// the Dcsc one with vector outputs, SpImpl.cpp:56-157 and 166-209), which
// combine equal rows in heap order: only semirings whose add does not depend
// on order are offloaded (Select2ndMin, SelectMax, integer PlusTimes).
template <class SR, class NUM, class IVT, class OVT>
constexpr int heap_vt()
{
    constexpr int vt = spmspv_vt<SR, NUM, IVT, OVT>();
    constexpr int sr = spmspv_of<SR>::sr;
    return vt >= 0 && (sr == GBC_SR_SELECT2NDMIN || sr == GBC_SR_SELECTMAX || (sr == GBC_SR_PLUSTIMES && vt == GBC_I64))
               ? vt
               : -1;
}

}  // namespace detail

// Drop the device copies of every matrix multiplied so far (call after
// changing a matrix in place).
inline void forget_matrices()
{
    std::lock_guard<std::mutex> lock(detail::call_mutex());
    for (auto &e : detail::plan_cache()) gbc_spmspv_plan_destroy(e.second);
    detail::plan_cache().clear();
    for (auto &e : detail::spmv_plan_cache()) gbc_spmv_plan_destroy(e.second);
    detail::spmv_plan_cache().clear();
}

// y <- y (+) A x with dense vectors (Friends.h:63-77): the row-major plan of
// A is built on the first product with A and kept (forget_matrices drops it).
template <class SR, class IU, class NU, class RHS, class LHS>
void dcsc_gespmv(const combblas::SpDCCols<IU, NU> &A, const RHS *x, LHS *y)
{
    if constexpr (!detail::offloaded<SR, NU, IU, RHS, LHS>()) {
        combblas::dcsc_gespmv<SR>(A, x, y);
    } else {
        if (A.isZero()) return;
        const gbc_matrix g = detail::view(A);
        std::lock_guard<std::mutex> lock(detail::call_mutex());
        gbc_spmv_plan *p = detail::spmv_plan(g, semiring_of<SR>::vt);
        detail::check(gbc_spmv(detail::context(), p, semiring_of<SR>::sr, x, y, GBC_HOST), "gbc_spmv");
    }
}

// y = A x (SpImpl.h:115-124, the PreAllocatedSPA overload that reaches
// SpMXSpV_Bucket): appended to indy / numy sorted by row.  Offloaded for
// Select2ndMin (registered), boolean Select2nd and SelectMax (integer
// vectors; A's values ignored) and PlusTimes (registered value type
// throughout), with int64 indices; any m x n matrix.
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV(const combblas::Csc<IT, NUM> &Acsc, int32_t mA, const int32_t *indx, const IVT *numx, int32_t veclen,
             std::vector<int32_t> &indy, std::vector<OVT> &numy, combblas::PreAllocatedSPA<OVT> &SPA)
{
    constexpr int vt = detail::spmspv_vt<SR, NUM, IVT, OVT>();
    if constexpr (vt < 0 || !std::is_same<IT, int64_t>::value) {
        combblas::SpMXSpV<SR>(Acsc, mA, indx, numx, veclen, indy, numy, SPA);
    } else {
        const gbc_matrix g = detail::view_csc(&Acsc, mA, Acsc.n, vt != GBC_BOOL);
        std::vector<int32_t> r;
        std::vector<OVT> v;
        detail::spmspv_run<SR>(g, vt, indx, numx, veclen, r, v);
        indy.insert(indy.end(), r.begin(), r.end());
        numy.insert(numy.end(), v.begin(), v.end());
    }
}

// y = A x over a Dcsc with vector outputs (SpImpl.h:49-56, the heap merge of
// SpImpl.cpp:56-157 and, for boolean matrices, 166-209; the call of
// Friends.h's local SpMV on a SpDCCols): appended to indy / numy sorted by
// row.  Offloaded where the heap's combination order does not show (heap_vt),
// with int64 indices.
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV(const combblas::Dcsc<IT, NUM> &Adcsc, int32_t mA, const int32_t *indx, const IVT *numx, int32_t veclen,
             std::vector<int32_t> &indy, std::vector<OVT> &numy, combblas::PreAllocatedSPA<OVT> &SPA)
{
    constexpr int vt = detail::heap_vt<SR, NUM, IVT, OVT>();
    if constexpr (vt < 0 || !std::is_same<IT, int64_t>::value) {
        combblas::SpMXSpV<SR>(Adcsc, mA, indx, numx, veclen, indy, numy, SPA);
    } else {
        const gbc_matrix g =
            detail::view_dcsc(&Adcsc, mA, Adcsc.nzc > 0 ? Adcsc.jc[Adcsc.nzc - 1] + 1 : 0, vt != GBC_BOOL);
        std::vector<int32_t> r;
        std::vector<OVT> v;
        if (g.nnz > 0) detail::spmspv_run<SR>(g, vt, indx, numx, veclen, r, v);
        detail::shift_rows(r, v, 0, indy, numy, true);
    }
}

// y = A x with the optbuf outputs (SpImpl.h:59-65 -> SpImpl.cpp:222-272, the
// call of BFSFriends.h:207): entries split among p_c receivers by row
// (owner = min(row / (mA / p_c), p_c - 1)), each receiver's rows ascending
// and local to its offset; cnts[p] entries land at indy/numy + dspls[p].
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV(const combblas::Dcsc<IT, NUM> &Adcsc, int32_t mA, const int32_t *indx, const IVT *numx, int32_t veclen,
             int32_t *indy, OVT *numy, int *cnts, int *dspls, int p_c)
{
    constexpr int vt = detail::spmspv_vt<SR, NUM, IVT, OVT>();
    if constexpr (vt < 0 || !std::is_same<IT, int64_t>::value) {
        combblas::SpMXSpV<SR>(Adcsc, mA, indx, numx, veclen, indy, numy, cnts, dspls, p_c);
    } else {
        // a Dcsc does not store its column count: its last nonempty column bounds it
        const gbc_matrix g =
            detail::view_dcsc(&Adcsc, mA, Adcsc.nzc > 0 ? Adcsc.jc[Adcsc.nzc - 1] + 1 : 0, vt != GBC_BOOL);
        std::vector<int32_t> r;
        std::vector<OVT> v;
        if (g.nnz > 0) detail::spmspv_run<SR>(g, vt, indx, numx, veclen, r, v);
        detail::split_rows(r, v, mA, indy, numy, cnts, dspls, p_c);
    }
}

// y = A x over one row piece of a RowSplit matrix (SpImpl.h:68-82, called
// per piece from an OpenMP loop by Friends.h:203-218 and BFSFriends.h:75-82):
// indy / numy are replaced by the piece's entries, rows ascending, each row
// plus `offset`.  Offloaded for boolean pieces under Select2nd, SelectMax and
// a registered Select2ndMin, with int64 indices; concurrent calls are
// serialised.  The overload with the caller's SPA buffers (localy, isthere,
// nzinds) gives the same result and leaves the buffers as they were: the
// device keeps its own working storage (the reference's result equals it
// when the buffers start cleared).
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV_ForThreading(const combblas::Dcsc<IT, NUM> &Adcsc, int32_t mA, const int32_t *indx, const IVT *numx,
                          int32_t veclen, std::vector<int32_t> &indy, std::vector<OVT> &numy, int32_t offset)
{
    constexpr int vt = detail::threaded_dcsc_vt<SR, NUM, IVT, OVT>();
    if constexpr (vt < 0 || !std::is_same<IT, int64_t>::value) {
        combblas::SpMXSpV_ForThreading<SR>(Adcsc, mA, indx, numx, veclen, indy, numy, offset);
    } else {
        const gbc_matrix g =
            detail::view_dcsc(&Adcsc, mA, Adcsc.nzc > 0 ? Adcsc.jc[Adcsc.nzc - 1] + 1 : 0, false);
        std::vector<int32_t> r;
        std::vector<OVT> v;
        if (g.nnz > 0) detail::spmspv_run<SR>(g, vt, indx, numx, veclen, r, v);
        detail::shift_rows(r, v, offset, indy, numy, false);
    }
}

template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV_ForThreading(const combblas::Dcsc<IT, NUM> &Adcsc, int32_t mA, const int32_t *indx, const IVT *numx,
                          int32_t veclen, std::vector<int32_t> &indy, std::vector<OVT> &numy, int32_t offset,
                          std::vector<OVT> &localy, combblas::BitMap &isthere, std::vector<uint32_t> &nzinds)
{
    constexpr int vt = detail::threaded_dcsc_vt<SR, NUM, IVT, OVT>();
    if constexpr (vt < 0 || !std::is_same<IT, int64_t>::value)
        combblas::SpMXSpV_ForThreading<SR>(Adcsc, mA, indx, numx, veclen, indy, numy, offset, localy, isthere,
                                           nzinds);
    else
        gbcomb::SpMXSpV_ForThreading<SR>(Adcsc, mA, indx, numx, veclen, indy, numy, offset);
}

// The same over a Csc piece (SpImpl.h:126-142, the heap version): x values
// multiplied into A's, the piece's entries appended to indy / numy with rows
// plus `offset`.  Offloaded where the heap's combination order does not show
// (heap_vt).
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV_ForThreading(const combblas::Csc<IT, NUM> &Acsc, int32_t mA, const int32_t *indx, const IVT *numx,
                          int32_t veclen, std::vector<int32_t> &indy, std::vector<OVT> &numy, int32_t offset)
{
    constexpr int vt = detail::heap_vt<SR, NUM, IVT, OVT>();
    if constexpr (vt < 0 || !std::is_same<IT, int64_t>::value) {
        combblas::SpMXSpV_ForThreading<SR>(Acsc, mA, indx, numx, veclen, indy, numy, offset);
    } else {
        const gbc_matrix g = detail::view_csc(&Acsc, mA, Acsc.n, vt != GBC_BOOL);
        std::vector<int32_t> r;
        std::vector<OVT> v;
        detail::spmspv_run<SR>(g, vt, indx, numx, veclen, r, v);
        detail::shift_rows(r, v, offset, indy, numy, true);
    }
}

template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV_ForThreading(const combblas::Csc<IT, NUM> &Acsc, int32_t mA, const int32_t *indx, const IVT *numx,
                          int32_t veclen, std::vector<int32_t> &indy, std::vector<OVT> &numy, int32_t offset,
                          std::vector<OVT> &localy, combblas::BitMap &isthere, std::vector<uint32_t> &nzinds)
{
    constexpr int vt = detail::heap_vt<SR, NUM, IVT, OVT>();
    if constexpr (vt < 0 || !std::is_same<IT, int64_t>::value)
        combblas::SpMXSpV_ForThreading<SR>(Acsc, mA, indx, numx, veclen, indy, numy, offset, localy, isthere,
                                           nzinds);
    else
        gbcomb::SpMXSpV_ForThreading<SR>(Acsc, mA, indx, numx, veclen, indy, numy, offset);
}

}  // namespace gbcomb
