// Runs the host-side layout code of include/gbcomb/combblas_shim.hpp against
// the reference's own types and algorithms, on the CPU (no GPU call):
//  * detail::view / view_dcsc / view_csc describe SpDCCols, SpCCols, Dcsc and
//    Csc objects built by the reference's constructors (SpDCCols.h:60,
//    SpCCols.h:50) with the entries the reference's own column iterators
//    visit;
//  * detail::tuples_of builds tuple arrays that the reference's SpTuples and
//    SpDCCols constructors turn back into the same matrix (operator new and
//    new[] storage, as the products and MultiwayMerge return them);
//  * detail::csc_of_tuples reads a column-sorted SpTuples into the CSC the
//    merge sends to the device;
//  * detail::split_rows, applied to the reference's heap SpMXSpV output
//    (SpImpl.cpp:166-209), gives the reference's optbuf output
//    (SpImpl.cpp:222-272): counts, receiver-local rows and values;
//    detail::shift_rows gives its threaded outputs over a row piece
//    (SpImpl.cpp:276-324, 345-386).
// A layout mismatch between the shim and the reference's classes fails here.
// Prints "layout-ok" and exits 0 when every check passes.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <tuple>
#include <vector>

#include "CombBLAS/CombBLAS.h"
#include "gbcomb/combblas_shim.hpp"

using namespace combblas;

namespace {

int g_fail = 0;

void check(bool ok, const char *what)
{
    if (!ok) {
        std::printf("FAIL %s\n", what);
        ++g_fail;
    }
}

template <class NT>
using Triples = std::vector<std::tuple<int64_t, int64_t, NT>>;  // (row, col, value), column-major

// seeded entries of an m x n matrix; every seventh column left empty (a
// DCSC then has fewer nonempty columns than columns)
template <class NT>
Triples<NT> random_entries(int64_t m, int64_t n, int64_t count, uint64_t seed)
{
    uint64_t s = seed;
    auto next = [&s]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return s >> 17;
    };
    Triples<NT> t;
    for (int64_t k = 0; k < count; ++k) {
        const int64_t c = (int64_t)(next() % (uint64_t)n);
        if (c % 7 == 3) continue;
        const int64_t r = (int64_t)(next() % (uint64_t)m);
        t.emplace_back(r, c, (NT)(1 + (int64_t)(next() % 1000)) / (NT)8);
    }
    std::sort(t.begin(), t.end(), [](const auto &a, const auto &b) {
        return std::get<1>(a) != std::get<1>(b) ? std::get<1>(a) < std::get<1>(b) : std::get<0>(a) < std::get<0>(b);
    });
    t.erase(std::unique(t.begin(), t.end(),
                        [](const auto &a, const auto &b) {
                            return std::get<0>(a) == std::get<0>(b) && std::get<1>(a) == std::get<1>(b);
                        }),
            t.end());
    return t;
}

// the reference's SpTuples over a new[] copy of the entries (it takes ownership)
template <class NT>
SpTuples<int64_t, NT> *sptuples(const Triples<NT> &t, int64_t m, int64_t n, bool shuffled)
{
    auto *arr = new std::tuple<int64_t, int64_t, NT>[t.empty() ? 1 : t.size()];
    for (size_t k = 0; k < t.size(); ++k) arr[k] = t[shuffled ? t.size() - 1 - k : k];
    // unsorted input: the constructor sorts it by column (SpTuples.cpp:52-60)
    return new SpTuples<int64_t, NT>((int64_t)t.size(), m, n, arr, !shuffled, false);
}

// the entries a C-ABI descriptor describes
template <class NT>
Triples<NT> triples_of_view(const gbc_matrix &g)
{
    Triples<NT> t;
    const NT *num = static_cast<const NT *>(g.num);
    for (int64_t k = 0; k < g.nzc; ++k) {
        const int64_t col = g.jc ? g.jc[k] : k;
        for (int64_t p = g.cp[k]; p < g.cp[k + 1]; ++p) t.emplace_back(g.ir[p], col, num ? num[p] : (NT)1);
    }
    return t;
}

// the entries the reference's own column iterators visit
template <class M, class NT>
Triples<NT> triples_of_iterators(M &A)
{
    Triples<NT> t;
    for (auto c = A.begcol(); c != A.endcol(); ++c)
        for (auto z = A.begnz(c); z != A.endnz(c); ++z) t.emplace_back(z.rowid(), c.colid(), z.value());
    return t;
}

// order-independent semiring for the SpMXSpV comparison: the heap and the
// optbuf versions add in different orders
struct MinSR {
    static int64_t id() { return std::numeric_limits<int64_t>::max(); }
    static bool returnedSAID() { return false; }
    static MPI_Op mpi_op() { return MPI_MIN; }
    static int64_t add(const int64_t &a, const int64_t &b) { return std::min(a, b); }
    static int64_t multiply(const bool &, const int64_t &b) { return b; }
    static void axpy(bool a, const int64_t &x, int64_t &y) { y = add(y, multiply(a, x)); }
};

void test_matrices()
{
    const int64_t m = 300, n = 257;
    const Triples<double> ref = random_entries<double>(m, n, 2400, 7);
    SpTuples<int64_t, double> *T = sptuples(ref, m, n, true);
    check(T->getnnz() == (int64_t)ref.size(), "SpTuples nnz");

    SpDCCols<int64_t, double> A(*T, false);
    check(triples_of_iterators<SpDCCols<int64_t, double>, double>(A) == ref, "SpDCCols holds the entries");
    const gbc_matrix ga = gbcomb::detail::view(A);
    check(ga.nrow == m && ga.ncol == n && ga.nnz == (int64_t)ref.size(), "view(SpDCCols) sizes");
    check(ga.nzc < n && ga.jc != nullptr, "view(SpDCCols) is a DCSC (empty columns skipped)");
    check(triples_of_view<double>(ga) == ref, "view(SpDCCols) entries");
    const gbc_matrix gd = gbcomb::detail::view_dcsc(A.GetDCSC(), m, n);
    check(triples_of_view<double>(gd) == ref, "view_dcsc entries");
    const gbc_matrix gp = gbcomb::detail::view_dcsc(A.GetDCSC(), m, n, false);
    check(gp.num == nullptr && gp.nnz == ga.nnz, "view_dcsc pattern");

    SpCCols<int64_t, double> Ac(*T, false);
    check(triples_of_iterators<SpCCols<int64_t, double>, double>(Ac) == ref, "SpCCols holds the entries");
    const gbc_matrix gc = gbcomb::detail::view(Ac);
    check(gc.nzc == n && gc.jc == nullptr, "view(SpCCols) is a CSC");
    check(triples_of_view<double>(gc) == ref, "view(SpCCols) entries");
    check(triples_of_view<double>(gbcomb::detail::view_csc(Ac.GetCSC(), m, n)) == ref, "view_csc entries");

    // tuples_of: the DCSC arrays back into SpTuples, both storage kinds
    for (int opnew = 0; opnew < 2; ++opnew) {
        auto *tup = gbcomb::detail::tuples_of<int64_t, double>(ga.nzc, ga.cp, ga.jc, ga.ir,
                                                               static_cast<const double *>(ga.num), opnew != 0);
        SpTuples<int64_t, double> S((int64_t)ref.size(), m, n, tup, true, opnew != 0);
        bool same = S.getnnz() == (int64_t)ref.size();
        for (int64_t p = 0; same && p < S.getnnz(); ++p)
            same = S.rowindex(p) == std::get<0>(ref[p]) && S.colindex(p) == std::get<1>(ref[p]) &&
                   S.numvalue(p) == std::get<2>(ref[p]);
        check(same, opnew ? "tuples_of (operator new) order and entries" : "tuples_of (new[]) order and entries");
        SpDCCols<int64_t, double> B(S, false);
        check(triples_of_view<double>(gbcomb::detail::view(B)) == ref, "tuples_of round trip through SpDCCols");
    }
    // the CSC form of a result: column ids 0..n-1
    {
        std::vector<int64_t> iota(n);
        for (int64_t j = 0; j < n; ++j) iota[j] = j;
        auto *tup = gbcomb::detail::tuples_of<int64_t, double>(n, gc.cp, iota.data(), gc.ir,
                                                               static_cast<const double *>(gc.num), true);
        SpTuples<int64_t, double> S((int64_t)ref.size(), m, n, tup, true, true);
        SpDCCols<int64_t, double> B(S, false);
        check(triples_of_view<double>(gbcomb::detail::view(B)) == ref, "tuples_of of a CSC result");
    }

    // csc_of_tuples: the merge's input conversion
    gbcomb::detail::TupleCsc<double> tc;
    gbcomb::detail::csc_of_tuples<int64_t, double>(*T, m, n, tc);
    check(tc.g.nzc == n && tc.g.nrow == m && tc.g.ncol == n, "csc_of_tuples sizes");
    check(triples_of_view<double>(tc.g) == ref, "csc_of_tuples entries");
    delete T;

    // empty operands
    SpTuples<int64_t, double> E(0, m, n);
    gbcomb::detail::TupleCsc<double> te;
    gbcomb::detail::csc_of_tuples<int64_t, double>(E, m, n, te);
    check(te.g.nnz == 0 && te.g.ir == nullptr && te.cp.size() == (size_t)n + 1 && te.cp[n] == 0, "csc_of_tuples empty");
}

void test_split_rows()
{
    const int64_t m = 1000;
    Triples<bool> pat;
    for (const auto &e : random_entries<double>(m, m, 9000, 11)) pat.emplace_back(std::get<0>(e), std::get<1>(e), true);
    SpTuples<int64_t, bool> *T = sptuples(pat, m, m, false);
    SpDCCols<int64_t, bool> A(*T, false);
    delete T;
    const Dcsc<int64_t, bool> &d = *A.GetDCSC();
    // a sparse vector: ascending columns, values its own index + 1
    std::vector<int32_t> indx;
    std::vector<int64_t> numx;
    for (int32_t c = 0; c < (int32_t)m; c += 3) {
        indx.push_back(c);
        numx.push_back(((int64_t)c * 7919) % 1009 + 1);
    }
    const int32_t veclen = (int32_t)indx.size(), mA = (int32_t)m;
    typedef SpImpl<MinSR, int64_t, bool, int64_t, int64_t> Impl;
    std::vector<int32_t> heap_rows;
    std::vector<int64_t> heap_vals;
    Impl::SpMXSpV(d, mA, indx.data(), numx.data(), veclen, heap_rows, heap_vals);
    check(!heap_rows.empty(), "reference SpMXSpV found entries");
    for (int p_c : {1, 3, 4, 7, 16}) {
        std::vector<int> dspls(p_c), cr(p_c), cs(p_c);
        for (int p = 0; p < p_c; ++p) dspls[p] = p * mA;
        std::vector<int32_t> ir(p_c * mA, -1), is(p_c * mA, -1);
        std::vector<int64_t> vr(p_c * mA, -1), vs(p_c * mA, -1);
        Impl::SpMXSpV(d, mA, indx.data(), numx.data(), veclen, ir.data(), vr.data(), cr.data(), dspls.data(), p_c);
        gbcomb::detail::split_rows(heap_rows, heap_vals, mA, is.data(), vs.data(), cs.data(), dspls.data(), p_c);
        bool same = cr == cs;
        for (int p = 0; same && p < p_c; ++p)
            for (int k = 0; same && k < cr[p]; ++k)
                same = ir[dspls[p] + k] == is[dspls[p] + k] && vr[dspls[p] + k] == vs[dspls[p] + k];
        char what[64];
        std::snprintf(what, sizeof(what), "split_rows against the optbuf SpMXSpV, p_c = %d", p_c);
        check(same, what);
    }
    // shift_rows against the threaded versions over a row piece: the boolean
    // SPA one (outputs replaced) and the Csc heap one (outputs appended)
    const int32_t off = 4096;
    std::vector<int32_t> ty{9, 9, 9}, sy;
    std::vector<int64_t> tv{1, 1, 1}, sv;
    Impl::SpMXSpV_ForThreading(d, mA, indx.data(), numx.data(), veclen, ty, tv, off);
    sy = {5};
    sv = {6};
    gbcomb::detail::shift_rows(heap_rows, heap_vals, off, sy, sv, false);
    check(ty == sy && tv == sv, "shift_rows against the boolean threaded SpMXSpV");
    SpTuples<int64_t, bool> *T2 = sptuples(pat, m, m, false);
    SpCCols<int64_t, bool> Ac(*T2, false);
    delete T2;
    std::vector<int32_t> hy, gy;
    std::vector<int64_t> hv, gv;
    combblas::SpMXSpV_ForThreading<MinSR>(*Ac.GetCSC(), mA, indx.data(), numx.data(), veclen, hy, hv, off);
    gbcomb::detail::shift_rows(heap_rows, heap_vals, off, gy, gv, true);
    check(!hy.empty() && hy == gy && hv == gv, "shift_rows against the Csc heap threaded SpMXSpV");
}

}  // namespace

int main()
{
    test_matrices();
    test_split_rows();
    if (g_fail) {
        std::printf("%d layout check(s) failed\n", g_fail);
        return 1;
    }
    std::printf("layout-ok\n");
    return 0;
}
