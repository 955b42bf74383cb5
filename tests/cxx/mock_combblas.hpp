// Stand-ins with the member names of the CombBLAS types that
// include/gbcomb/combblas_shim.hpp touches (SpDCCols/Dcsc, SpCCols/Csc,
// SpTuples, PreAllocatedSPA, the stock semirings) and plain CPU versions of
// the four multiplies the shim falls back to, so the shim can be compiled
// and run where the reference sources are not present.  Test code only.
#pragma once
#include <algorithm>
#include <cstdint>
#include <map>
#include <tuple>
#include <vector>

namespace combblas {

template <class T1, class T2>
struct PlusTimesSRing {
    typedef T1 T_promote;
    static T1 add(const T1 &a, const T1 &b) { return a + b; }
    static T1 multiply(const T1 &a, const T2 &b) { return a * b; }
};
template <class T1, class T2>
struct MinPlusSRing {
    typedef T1 T_promote;
    static T1 add(const T1 &a, const T1 &b) { return std::min(a, b); }
    static T1 multiply(const T1 &a, const T2 &b) { return a + b; }
};

template <class T1, class T2, class OUT>
struct Select2ndSRing {
    static OUT add(const OUT &, const OUT &b) { return b; }
    static OUT multiply(const T1 &, const T2 &b) { return static_cast<OUT>(b); }
};
template <class T1, class T2>
struct SelectMaxSRing {
    typedef T2 T_promote;
    static T2 add(const T2 &a, const T2 &b) { return std::max(a, b); }
    static T2 multiply(const T1 &, const T2 &b) { return b; }
};

template <class IT, class NT>
struct Dcsc {
    IT *cp = nullptr, *jc = nullptr, *ir = nullptr;
    NT *numx = nullptr;
    IT nz = 0, nzc = 0;
};

template <class IT, class NT>
class SpDCCols {
  public:
    SpDCCols(IT m, IT n, std::vector<IT> cp, std::vector<IT> jc, std::vector<IT> ir, std::vector<NT> v)
        : m_(m), n_(n), cp_(cp), jc_(jc), ir_(ir), v_(v)
    {
        d_.cp = cp_.data();
        d_.jc = jc_.data();
        d_.ir = ir_.data();
        d_.numx = v_.data();
        d_.nz = (IT)ir_.size();
        d_.nzc = (IT)jc_.size();
    }
    IT getnrow() const { return m_; }
    IT getncol() const { return n_; }
    IT getnnz() const { return d_.nz; }
    bool isZero() const { return d_.nz == 0; }
    Dcsc<IT, NT> *GetDCSC() const { return const_cast<Dcsc<IT, NT> *>(&d_); }
    static int deleted;
    ~SpDCCols() { ++deleted; }

  private:
    IT m_, n_;
    std::vector<IT> cp_, jc_, ir_;
    std::vector<NT> v_;
    Dcsc<IT, NT> d_;
};
template <class IT, class NT>
int SpDCCols<IT, NT>::deleted = 0;

template <class IT, class NT>
struct Csc {
    IT *jc = nullptr, *ir = nullptr;
    NT *num = nullptr;
    IT n = 0, nz = 0;
};

template <class IT, class NT>
class SpCCols {
  public:
    SpCCols(IT m, IT n, std::vector<IT> cp, std::vector<IT> ir, std::vector<NT> v) : m_(m), n_(n), cp_(cp), ir_(ir), v_(v)
    {
        c_.jc = cp_.data();
        c_.ir = ir_.data();
        c_.num = v_.data();
        c_.n = n;
        c_.nz = (IT)ir_.size();
    }
    IT getnrow() const { return m_; }
    IT getncol() const { return n_; }
    bool isZero() const { return c_.nz == 0; }
    Csc<IT, NT> *GetCSC() const { return const_cast<Csc<IT, NT> *>(&c_); }

  private:
    IT m_, n_;
    std::vector<IT> cp_, ir_;
    std::vector<NT> v_;
    Csc<IT, NT> c_;
};

template <class IT, class NT>
class SpTuples {
  public:
    SpTuples(int64_t size, IT m, IT n) : nnz(size), m_(m), n_(n) {}
    SpTuples(int64_t size, IT m, IT n, std::tuple<IT, IT, NT> *t, bool sorted = false, bool isOpNew = false)
        : nnz(size), m_(m), n_(n), tuples(t), sorted_(sorted), opnew_(isOpNew)
    {
    }
    ~SpTuples()
    {
        if (tuples && opnew_) ::operator delete(tuples);
        else delete[] tuples;
    }
    int64_t getnnz() const { return nnz; }
    IT rowindex(int64_t i) const { return std::get<0>(tuples[i]); }
    IT colindex(int64_t i) const { return std::get<1>(tuples[i]); }
    NT numvalue(int64_t i) const { return std::get<2>(tuples[i]); }
    IT getnrow() const { return m_; }
    IT getncol() const { return n_; }
    int64_t nnz;
    IT m_, n_;
    std::tuple<IT, IT, NT> *tuples = nullptr;
    bool sorted_ = false, opnew_ = false;
};

template <class OVT>
struct PreAllocatedSPA {};

struct BitMap {
    std::vector<bool> bits;
    explicit BitMap(uint64_t n = 0) : bits(n) {}
    void set_bit(uint64_t i) { bits[i] = true; }
    bool get_bit(uint64_t i) const { return bits[i]; }
};

// CPU product over column j of B in k order: acc = add(mrhs, acc), first
// contribution stored as is; rows ascending.
template <class SR, class NTO, class IT, class NT1, class NT2, class MA, class MB>
SpTuples<IT, NTO> *cpu_multiply(IT m, IT n, const MA &acol, const MB &bcol)
{
    std::vector<std::tuple<IT, IT, NTO>> out;
    for (IT j = 0; j < n; ++j) {
        std::map<IT, NTO> acc;
        for (auto &kb : bcol(j))
            for (auto &ra : acol(kb.first)) {
                const NTO v = SR::multiply(ra.second, kb.second);
                auto it = acc.find(ra.first);
                if (it == acc.end()) acc[ra.first] = v;
                else it->second = SR::add(v, it->second);
            }
        for (auto &e : acc) out.emplace_back(e.first, j, e.second);
    }
    auto *t = static_cast<std::tuple<IT, IT, NTO> *>(::operator new(sizeof(std::tuple<IT, IT, NTO>) * (out.size() + 1)));
    std::copy(out.begin(), out.end(), t);
    return new SpTuples<IT, NTO>((int64_t)out.size(), m, n, t, true, true);
}

template <class IT, class NT>
std::vector<std::pair<IT, NT>> dcsc_col(const SpDCCols<IT, NT> &M, IT j)
{
    std::vector<std::pair<IT, NT>> r;
    const Dcsc<IT, NT> *d = M.GetDCSC();
    for (IT q = 0; q < d->nzc; ++q)
        if (d->jc[q] == j)
            for (IT p = d->cp[q]; p < d->cp[q + 1]; ++p) r.emplace_back(d->ir[p], d->numx[p]);
    return r;
}

// the reference templates the shim falls back to (here: the CPU product,
// marked so a test can tell which path ran)
inline int &fallback_calls()
{
    static int c = 0;
    return c;
}

template <class SR, class NTO, class IT, class NT1, class NT2>
SpTuples<IT, NTO> *LocalHybridSpGEMM(const SpDCCols<IT, NT1> &A, const SpDCCols<IT, NT2> &B, bool, bool,
                                     IT * = nullptr)
{
    ++fallback_calls();
    return cpu_multiply<SR, NTO, IT, NT1, NT2>(A.getnrow(), B.getncol(), [&](IT k) { return dcsc_col(A, k); },
                                               [&](IT j) { return dcsc_col(B, j); });
}
template <class SR, class NTO, class IT, class NT1, class NT2>
SpTuples<IT, NTO> *LocalSpGEMM(const SpDCCols<IT, NT1> &A, const SpDCCols<IT, NT2> &B, bool c1, bool c2)
{
    return LocalHybridSpGEMM<SR, NTO>(A, B, c1, c2);
}
template <class SR, class NTO, class IT, class NT1, class NT2>
SpTuples<IT, NTO> *LocalSpGEMMHash(const SpDCCols<IT, NT1> &A, const SpDCCols<IT, NT2> &B, bool c1, bool c2,
                                   bool = true)
{
    return LocalHybridSpGEMM<SR, NTO>(A, B, c1, c2);
}
template <class SR, class NTO, class IT, class NT1, class NT2>
SpTuples<IT, NTO> *LocalHybridSpGEMM(const SpCCols<IT, NT1> &, const SpCCols<IT, NT2> &, bool, bool)
{
    ++fallback_calls();
    return nullptr;
}
// y <- y (+) A x, columns in order (the reference's dcsc_gespmv)
template <class SR, class IU, class NU, class RHS, class LHS>
void dcsc_gespmv(const SpDCCols<IU, NU> &A, const RHS *x, LHS *y)
{
    ++fallback_calls();
    const Dcsc<IU, NU> *d = A.GetDCSC();
    for (IU q = 0; q < d->nzc; ++q)
        for (IU p = d->cp[q]; p < d->cp[q + 1]; ++p)
            y[d->ir[p]] = SR::add(y[d->ir[p]], SR::multiply(d->numx[p], x[d->jc[q]]));
}

// column-sorted merge with equal keys combined in list order
template <class SR, class IT, class NT>
SpTuples<IT, NT> *MultiwayMerge(std::vector<SpTuples<IT, NT> *> &L, IT mdim = 0, IT ndim = 0, bool delarrs = false)
{
    ++fallback_calls();
    std::map<std::pair<IT, IT>, NT> acc;  // (col, row)
    for (auto *T : L)
        for (int64_t p = 0; p < T->getnnz(); ++p) {
            const auto key = std::make_pair(T->colindex(p), T->rowindex(p));
            auto it = acc.find(key);
            if (it == acc.end()) acc[key] = T->numvalue(p);
            else it->second = SR::add(it->second, T->numvalue(p));
        }
    auto *t = new std::tuple<IT, IT, NT>[acc.size() + 1];
    int64_t q = 0;
    for (auto &e : acc) t[q++] = std::tuple<IT, IT, NT>(e.first.second, e.first.first, e.second);
    if (delarrs)
        for (auto *T : L) delete T;
    return new SpTuples<IT, NT>(q, mdim, ndim, t, true, false);
}

template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV(const Csc<IT, NUM> &, int32_t, const int32_t *, const IVT *, int32_t, std::vector<int32_t> &,
             std::vector<OVT> &, PreAllocatedSPA<OVT> &)
{
    ++fallback_calls();
}
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV(const Dcsc<IT, NUM> &, int32_t, const int32_t *, const IVT *, int32_t, int32_t *, OVT *, int *, int *,
             int)
{
    ++fallback_calls();
}
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV(const Dcsc<IT, NUM> &, int32_t, const int32_t *, const IVT *, int32_t, std::vector<int32_t> &,
             std::vector<OVT> &, PreAllocatedSPA<OVT> &)
{
    ++fallback_calls();
}

// the threaded SpMSpV over a row piece: SPA in column order for Dcsc (rows
// ascending, plus offset, replacing the outputs); x multiplied in and
// appended for Csc (a map stands in for the reference's heap)
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV_ForThreading(const Dcsc<IT, NUM> &d, int32_t, const int32_t *indx, const IVT *numx, int32_t veclen,
                          std::vector<int32_t> &indy, std::vector<OVT> &numy, int32_t offset)
{
    ++fallback_calls();
    std::map<int32_t, OVT> y;
    for (IT q = 0; q < d.nzc; ++q)
        for (int32_t k = 0; k < veclen; ++k)
            if (indx[k] == d.jc[q])
                for (IT p = d.cp[q]; p < d.cp[q + 1]; ++p) {
                    auto it = y.find((int32_t)d.ir[p]);
                    if (it == y.end()) y[(int32_t)d.ir[p]] = static_cast<OVT>(numx[k]);
                    else it->second = SR::add(it->second, static_cast<OVT>(numx[k]));
                }
    indy.clear();
    numy.clear();
    for (auto &e : y) {
        indy.push_back(e.first + offset);
        numy.push_back(e.second);
    }
}
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV_ForThreading(const Dcsc<IT, NUM> &d, int32_t mA, const int32_t *indx, const IVT *numx, int32_t veclen,
                          std::vector<int32_t> &indy, std::vector<OVT> &numy, int32_t offset, std::vector<OVT> &,
                          BitMap &, std::vector<uint32_t> &)
{
    SpMXSpV_ForThreading<SR>(d, mA, indx, numx, veclen, indy, numy, offset);
}
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV_ForThreading(const Csc<IT, NUM> &c, int32_t, const int32_t *indx, const IVT *numx, int32_t veclen,
                          std::vector<int32_t> &indy, std::vector<OVT> &numy, int32_t offset)
{
    ++fallback_calls();
    std::map<int32_t, OVT> y;
    for (int32_t k = 0; k < veclen; ++k)
        for (IT p = c.jc[indx[k]]; p < c.jc[indx[k] + 1]; ++p) {
            const OVT v = SR::multiply(c.num[p], numx[k]);
            auto it = y.find((int32_t)c.ir[p]);
            if (it == y.end()) y[(int32_t)c.ir[p]] = v;
            else it->second = SR::add(it->second, v);
        }
    for (auto &e : y) {
        indy.push_back(e.first + offset);
        numy.push_back(e.second);
    }
}
template <class SR, class IT, class NUM, class IVT, class OVT>
void SpMXSpV_ForThreading(const Csc<IT, NUM> &c, int32_t mA, const int32_t *indx, const IVT *numx, int32_t veclen,
                          std::vector<int32_t> &indy, std::vector<OVT> &numy, int32_t offset, std::vector<OVT> &,
                          BitMap &, std::vector<uint32_t> &)
{
    SpMXSpV_ForThreading<SR>(c, mA, indx, numx, veclen, indy, numy, offset);
}

}  // namespace combblas
