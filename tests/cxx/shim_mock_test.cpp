// Runs include/gbcomb/combblas_shim.hpp against the stand-in types of
// mock_combblas.hpp: GPU results must equal the CPU product bit for bit,
// ownership rules must hold, unregistered semirings must fall back.
#include "mock_combblas.hpp"

#include <cstdio>
#include <cmath>
#include <cstring>
#include <random>
#include <thread>

#include "gbcomb/combblas_shim.hpp"

namespace app {
template <class T1, class T2>
struct Select2ndMinSR {  // an application-defined semiring, as in FastSV.h
    typedef T1 T_promote;
    static T1 add(const T1 &a, const T1 &b) { return std::min(a, b); }
    static T1 multiply(const T1 &, const T2 &b) { return b; }
};
template <class T1, class T2>
struct MaxTimes {  // not registered: must run the reference template
    typedef T1 T_promote;
    static T1 add(const T1 &a, const T1 &b) { return std::max(a, b); }
    static T1 multiply(const T1 &a, const T2 &b) { return a * b; }
};
}  // namespace app
typedef app::Select2ndMinSR<int64_t, int64_t> S2M;
GBCOMB_REGISTER_SEMIRING(S2M, GBC_SR_SELECT2NDMIN, GBC_I64)

using namespace combblas;
typedef int64_t I;

static int failures = 0;
#define EXPECT(...)                                                    \
    do {                                                               \
        if (!(__VA_ARGS__)) {                                                  \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #__VA_ARGS__); \
            ++failures;                                                \
        }                                                              \
    } while (0)

template <class NT>
SpDCCols<I, NT> *random_dcsc(I m, I n, double density, double empty_cols, unsigned seed)
{
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    std::vector<I> cp{0}, jc, ir;
    std::vector<NT> v;
    for (I j = 0; j < n; ++j) {
        if (u(g) < empty_cols) continue;
        I cnt = 0;
        for (I r = 0; r < m; ++r)
            if (u(g) < density) {
                ir.push_back(r);
                v.push_back((NT)(std::is_floating_point<NT>::value ? 1.0 - u(g) : (double)(1 + (int)(u(g) * 40))));
                ++cnt;
            }
        if (cnt) {
            jc.push_back(j);
            cp.push_back(cp.back() + cnt);
        }
    }
    return new SpDCCols<I, NT>(m, n, cp, jc, ir, v);
}

template <class NT>
bool same(const SpTuples<I, NT> *a, const SpTuples<I, NT> *b)
{
    if (a->getnnz() != b->getnnz() || a->getnrow() != b->getnrow() || a->getncol() != b->getncol()) return false;
    for (int64_t p = 0; p < a->getnnz(); ++p) {
        if (std::get<0>(a->tuples[p]) != std::get<0>(b->tuples[p])) return false;
        if (std::get<1>(a->tuples[p]) != std::get<1>(b->tuples[p])) return false;
        NT x = std::get<2>(a->tuples[p]), y = std::get<2>(b->tuples[p]);
        if (std::memcmp(&x, &y, sizeof(NT)) != 0) return false;
    }
    return true;
}

int main()
{
    typedef PlusTimesSRing<double, double> PT;
    // 1. PlusTimes fp64 over DCSC with the ordered fold, bit-exact against
    //    the CPU product (the exact fold is checked within 1e-12 at the end)
    gbcomb::set_fold(GBC_FOLD_ORDERED);
    SpDCCols<I, double> *A = random_dcsc<double>(700, 500, 0.02, 0.3, 1);
    SpDCCols<I, double> *B = random_dcsc<double>(500, 400, 0.03, 0.3, 2);
    const int fb0 = fallback_calls();
    SpTuples<I, double> *g = gbcomb::LocalHybridSpGEMM<PT, double>(*A, *B, false, false);
    EXPECT(fallback_calls() == fb0);  // ran on the GPU
    SpTuples<I, double> *c = combblas::LocalHybridSpGEMM<PT, double>(*A, *B, false, false);
    EXPECT(g->getnnz() > 0 && same(g, c));
    EXPECT(g->sorted_ && g->opnew_);
    SpTuples<I, double> *h = gbcomb::LocalSpGEMMHash<PT, double>(*A, *B, false, false, true);
    EXPECT(same(h, c));
    SpTuples<I, double> *l = gbcomb::LocalSpGEMM<PT, double>(*A, *B, false, false);
    EXPECT(same(l, c));
    delete g;
    delete c;
    delete h;
    delete l;
    // 2. clearA / clearB delete the inputs
    const int del0 = SpDCCols<I, double>::deleted;
    SpTuples<I, double> *d = gbcomb::LocalHybridSpGEMM<PT, double>(*A, *B, true, true);
    EXPECT(SpDCCols<I, double>::deleted == del0 + 2);
    delete d;
    // 3. an empty operand gives an empty product of the right shape
    SpDCCols<I, double> Z(700, 500, {0}, {}, {}, {});
    SpDCCols<I, double> *B2 = random_dcsc<double>(500, 40, 0.05, 0.0, 3);
    SpTuples<I, double> *e = gbcomb::LocalHybridSpGEMM<PT, double>(Z, *B2, false, false);
    EXPECT(e->getnnz() == 0 && e->getnrow() == 700 && e->getncol() == 40);
    delete e;
    // 4. an application semiring registered by the application
    SpDCCols<I, int64_t> *Ai = random_dcsc<int64_t>(300, 300, 0.03, 0.2, 4);
    SpTuples<I, int64_t> *gi = gbcomb::LocalHybridSpGEMM<S2M, int64_t>(*Ai, *Ai, false, false);
    SpTuples<I, int64_t> *ci = combblas::LocalHybridSpGEMM<S2M, int64_t>(*Ai, *Ai, false, false);
    EXPECT(gi->getnnz() > 0 && same(gi, ci));
    delete gi;
    delete ci;
    // 5. an unregistered semiring runs the reference template
    SpDCCols<I, double> *Bs = random_dcsc<double>(500, 500, 0.01, 0.0, 5);
    const int fb1 = fallback_calls();
    SpTuples<I, double> *mx = gbcomb::LocalHybridSpGEMM<app::MaxTimes<double, double>, double>(*Bs, *Bs, false, false);
    EXPECT(fallback_calls() == fb1 + 1);
    delete mx;
    // ... and so does a registered semiring with other value types
    const int fb2 = fallback_calls();
    SpTuples<I, float> *f = gbcomb::LocalHybridSpGEMM<PT, float>(*Bs, *Bs, false, false);
    EXPECT(fallback_calls() == fb2 + 1);
    delete f;
    // 6. the CSC overload
    {
        std::vector<I> cp{0}, ir;
        std::vector<double> v;
        const Dcsc<I, double> *dd = B2->GetDCSC();
        I q = 0;
        for (I j = 0; j < B2->getncol(); ++j) {
            if (q < dd->nzc && dd->jc[q] == j) {
                for (I p = dd->cp[q]; p < dd->cp[q + 1]; ++p) {
                    ir.push_back(dd->ir[p]);
                    v.push_back(dd->numx[p]);
                }
                ++q;
            }
            cp.push_back((I)ir.size());
        }
        SpCCols<I, double> Bc(B2->getnrow(), B2->getncol(), cp, ir, v);
        std::vector<I> acp{0}, air;
        std::vector<double> av;
        const Dcsc<I, double> *ad = Bs->GetDCSC();
        q = 0;
        for (I j = 0; j < Bs->getncol(); ++j) {
            if (q < ad->nzc && ad->jc[q] == j) {
                for (I p = ad->cp[q]; p < ad->cp[q + 1]; ++p) {
                    air.push_back(ad->ir[p]);
                    av.push_back(ad->numx[p]);
                }
                ++q;
            }
            acp.push_back((I)air.size());
        }
        SpCCols<I, double> Ac(Bs->getnrow(), Bs->getncol(), acp, air, av);
        SpTuples<I, double> *gc = gbcomb::LocalHybridSpGEMM<PT, double>(Ac, Bc, false, false);
        SpTuples<I, double> *cc = combblas::LocalHybridSpGEMM<PT, double>(*Bs, *B2, false, false);
        EXPECT(gc->getnnz() > 0 && same(gc, cc));
        delete gc;
        delete cc;
        // 7. SpMXSpV over the application's Select2ndMin on a square CSC
        std::vector<I> scp{0}, sir;
        std::vector<int64_t> sv;
        for (I j = 0; j < Ac.getncol(); ++j) {
            for (I p = acp[j]; p < acp[j + 1]; ++p) {
                sir.push_back(air[p]);
                sv.push_back(1);
            }
            scp.push_back((I)sir.size());
        }
        Csc<I, int64_t> csc;
        csc.jc = scp.data();
        csc.ir = sir.data();
        csc.num = sv.data();
        csc.n = Ac.getncol();
        csc.nz = (I)sir.size();
        std::vector<int32_t> indx{3, 17, 40, 41, 250, 499};
        std::vector<int64_t> numx{9, 2, 7, 7, 1, 5};
        std::vector<int32_t> indy{-1};  // results are appended
        std::vector<int64_t> numy{-1};
        PreAllocatedSPA<int64_t> spa;
        gbcomb::SpMXSpV<S2M>(csc, (int32_t)Ac.getnrow(), indx.data(), numx.data(), (int32_t)indx.size(), indy, numy,
                             spa);
        std::map<I, int64_t> ref;
        for (size_t t = 0; t < indx.size(); ++t)
            for (I p = scp[indx[t]]; p < scp[indx[t] + 1]; ++p) {
                auto it = ref.find(sir[p]);
                if (it == ref.end()) ref[sir[p]] = numx[t];
                else it->second = std::min(it->second, numx[t]);
            }
        EXPECT(indy.size() == ref.size() + 1 && indy[0] == -1 && numy[0] == -1);
        size_t k = 1;
        for (auto &e : ref) {
            EXPECT(k < indy.size() && indy[k] == e.first && numy[k] == e.second);
            ++k;
        }
        gbcomb::forget_matrices();  // before the matrix's memory is freed
    }
    // 7b. the other SpMXSpV semirings on a rectangular matrix (300 x 900):
    // SelectMax and PlusTimes through the Csc overload, Select2nd through the
    // Dcsc optbuf overload with three receivers; one device copy per matrix
    {
        std::mt19937_64 rng(77);
        const I m = 300, n = 900;
        std::vector<I> cp{0}, ir, jc, dcp{0};
        std::vector<double> val;
        std::vector<bool> dummy;
        for (I j = 0; j < n; ++j) {
            std::vector<I> rows;
            if (j % 3 != 1)
                for (I r = 0; r < m; ++r)
                    if (rng() % 100 < 3) rows.push_back(r);
            for (I r : rows) {
                ir.push_back(r);
                val.push_back(double(rng() % 2000) / 1000.0 - 1.0);
            }
            cp.push_back((I)ir.size());
            if (!rows.empty()) {
                jc.push_back(j);
                dcp.push_back((I)ir.size());
            }
        }
        Csc<I, double> csc;
        csc.jc = cp.data();
        csc.ir = ir.data();
        csc.num = val.data();
        csc.n = n;
        csc.nz = (I)ir.size();
        std::vector<int32_t> indx;
        std::vector<int64_t> xi;
        std::vector<double> xd;
        for (int32_t c = 0; c < n; c += 1 + (int32_t)(rng() % 5)) {
            indx.push_back(c);
            xi.push_back((int64_t)(rng() % 100000) - 50000);
            xd.push_back(double(rng() % 1000) / 997.0);
        }
        // CPU expectations: ascending columns, first stored, later folded
        std::map<I, int64_t> emax, elast;
        std::map<I, double> esum;
        for (size_t t = 0; t < indx.size(); ++t)
            for (I p = cp[indx[t]]; p < cp[indx[t] + 1]; ++p) {
                const I r = ir[p];
                const double prod = val[p] * xd[t];
                if (!emax.count(r)) {
                    emax[r] = xi[t];
                    esum[r] = prod;
                } else {
                    emax[r] = std::max(emax[r], xi[t]);
                    esum[r] = esum[r] + prod;
                }
                elast[r] = xi[t];
            }
        typedef SelectMaxSRing<bool, int64_t> SMAX;
        typedef Select2ndSRing<bool, int64_t, int64_t> S2ND;
        Csc<I, bool> bcsc;
        std::unique_ptr<bool[]> bv(new bool[ir.size() + 1]);
        bcsc.jc = cp.data();
        bcsc.ir = ir.data();
        bcsc.num = bv.get();
        bcsc.n = n;
        bcsc.nz = (I)ir.size();
        const int fb = fallback_calls();
        const long long builds = gbcomb::detail::plan_builds();
        PreAllocatedSPA<int64_t> spa;
        for (int rep = 0; rep < 2; ++rep) {
            std::vector<int32_t> indy;
            std::vector<int64_t> numy;
            gbcomb::SpMXSpV<SMAX>(bcsc, (int32_t)m, indx.data(), xi.data(), (int32_t)indx.size(), indy, numy, spa);
            EXPECT(indy.size() == emax.size());
            size_t k = 0;
            for (auto &e : emax) {
                EXPECT(k < indy.size() && indy[k] == e.first && numy[k] == e.second);
                ++k;
            }
        }
        EXPECT(gbcomb::detail::plan_builds() == builds + 1);  // the second call reused the device copy
        PreAllocatedSPA<double> dspa;
        std::vector<int32_t> indy;
        std::vector<double> numy;
        gbcomb::SpMXSpV<PT>(csc, (int32_t)m, indx.data(), xd.data(), (int32_t)indx.size(), indy, numy, dspa);
        EXPECT(indy.size() == esum.size());
        size_t k = 0;
        for (auto &e : esum) {
            EXPECT(k < indy.size() && indy[k] == e.first && numy[k] == e.second);
            ++k;
        }
        Dcsc<I, bool> d;
        d.cp = dcp.data();
        d.jc = jc.data();
        d.ir = ir.data();
        d.numx = bv.get();
        d.nz = (I)ir.size();
        d.nzc = (I)jc.size();
        std::vector<int32_t> oind(m);
        std::vector<int64_t> onum(m);
        int cnts[3], dspls[3] = {0, 100, 200};
        gbcomb::SpMXSpV<S2ND>(d, (int32_t)m, indx.data(), xi.data(), (int32_t)indx.size(), oind.data(), onum.data(),
                              cnts, dspls, 3);
        int got[3] = {0, 0, 0};
        for (auto &e : elast) {
            const int p = std::min((int)(e.first / (m / 3)), 2);
            const int q = dspls[p] + got[p]++;
            EXPECT(q < m && oind[q] == e.first - (m / 3) * p && onum[q] == e.second);
        }
        EXPECT(cnts[0] == got[0] && cnts[1] == got[1] && cnts[2] == got[2]);
        EXPECT(fallback_calls() == fb);
        gbcomb::forget_matrices();
        EXPECT(gbcomb::detail::plan_cache().empty());
    }
    // 7c. SpMXSpV_ForThreading over one row piece (300 x 900): the boolean
    // Dcsc piece under Select2nd (outputs replaced, rows plus the offset; the
    // SPA buffers left as they were), the Csc piece under SelectMax (outputs
    // appended), PlusTimes fp64 on a Csc piece falling through (the heap's
    // order shows in fp sums), and four host threads calling at once
    {
        std::mt19937_64 rng(91);
        const I m = 300, n = 900;
        const int32_t off = 1200;
        std::vector<I> cp{0}, ir, jc, dcp{0};
        std::vector<double> val;
        for (I j = 0; j < n; ++j) {
            if (j % 4 == 2) {
                cp.push_back((I)ir.size());
                continue;
            }
            for (I r = 0; r < m; ++r)
                if (rng() % 100 < 4) {
                    ir.push_back(r);
                    val.push_back(double(rng() % 1000) / 999.0);
                }
            cp.push_back((I)ir.size());
            if (cp[j + 1] > cp[j]) {
                jc.push_back(j);
                dcp.push_back((I)ir.size());
            }
        }
        std::unique_ptr<bool[]> bv(new bool[ir.size() + 1]);
        for (size_t q = 0; q < ir.size(); ++q) bv[q] = true;
        Dcsc<I, bool> d;
        d.cp = dcp.data();
        d.jc = jc.data();
        d.ir = ir.data();
        d.numx = bv.get();
        d.nz = (I)ir.size();
        d.nzc = (I)jc.size();
        Csc<I, bool> bcsc;
        bcsc.jc = cp.data();
        bcsc.ir = ir.data();
        bcsc.num = bv.get();
        bcsc.n = n;
        bcsc.nz = (I)ir.size();
        Csc<I, double> csc;
        csc.jc = cp.data();
        csc.ir = ir.data();
        csc.num = val.data();
        csc.n = n;
        csc.nz = (I)ir.size();
        std::vector<int32_t> indx;
        std::vector<int64_t> xi;
        std::vector<double> xd;
        for (int32_t c = 0; c < n; c += 1 + (int32_t)(rng() % 4)) {
            indx.push_back(c);
            xi.push_back((int64_t)(rng() % 100000) - 50000);
            xd.push_back(double(rng() % 1000) / 997.0);
        }
        std::map<I, int64_t> elast, emax;
        for (size_t t = 0; t < indx.size(); ++t)
            for (I p = cp[indx[t]]; p < cp[indx[t] + 1]; ++p) {
                const I r = ir[p];
                emax[r] = emax.count(r) ? std::max(emax[r], xi[t]) : xi[t];
                elast[r] = xi[t];
            }
        typedef SelectMaxSRing<bool, int64_t> SMAX;
        typedef Select2ndSRing<bool, int64_t, int64_t> S2ND;
        auto check_rows = [&](const std::map<I, int64_t> &e, const std::vector<int32_t> &iy,
                              const std::vector<int64_t> &ny, size_t skip) {
            EXPECT(iy.size() == e.size() + skip && ny.size() == iy.size());
            size_t k = skip;
            for (auto &x : e) {
                EXPECT(k < iy.size() && iy[k] == (int32_t)x.first + off && ny[k] == x.second);
                ++k;
            }
        };
        const int fb = fallback_calls();
        std::vector<int32_t> indy{-5, -6};
        std::vector<int64_t> numy{7, 8};
        gbcomb::SpMXSpV_ForThreading<S2ND>(d, (int32_t)m, indx.data(), xi.data(), (int32_t)indx.size(), indy, numy,
                                           off);
        check_rows(elast, indy, numy, 0);
        std::vector<int64_t> localy(m, 42);
        BitMap isthere(m);
        std::vector<uint32_t> nzinds(5, 3u);
        gbcomb::SpMXSpV_ForThreading<S2ND>(d, (int32_t)m, indx.data(), xi.data(), (int32_t)indx.size(), indy, numy,
                                           off, localy, isthere, nzinds);
        check_rows(elast, indy, numy, 0);
        EXPECT(nzinds.size() == 5 && localy[0] == 42 && !isthere.get_bit(0));
        std::vector<int32_t> cy{77};
        std::vector<int64_t> cn{78};
        gbcomb::SpMXSpV_ForThreading<SMAX>(bcsc, (int32_t)m, indx.data(), xi.data(), (int32_t)indx.size(), cy, cn,
                                           off);
        EXPECT(cy[0] == 77 && cn[0] == 78);
        check_rows(emax, cy, cn, 1);
        EXPECT(fallback_calls() == fb);
        // the Dcsc overload with vector outputs (appended, global rows)
        PreAllocatedSPA<int64_t> spa;
        std::vector<int32_t> dy{3};
        std::vector<int64_t> dn{4};
        gbcomb::SpMXSpV<SMAX>(d, (int32_t)m, indx.data(), xi.data(), (int32_t)indx.size(), dy, dn, spa);
        EXPECT(dy.size() == emax.size() + 1 && dy[0] == 3 && dn[0] == 4);
        {
            size_t k = 1;
            for (auto &x : emax) {
                EXPECT(k < dy.size() && dy[k] == (int32_t)x.first && dn[k] == x.second);
                ++k;
            }
        }
        EXPECT(fallback_calls() == fb);
        std::vector<int32_t> fy;
        std::vector<double> fn;
        gbcomb::SpMXSpV_ForThreading<PT>(csc, (int32_t)m, indx.data(), xd.data(), (int32_t)indx.size(), fy, fn, off);
        EXPECT(fallback_calls() == fb + 1);
        std::vector<int32_t> sy2;
        std::vector<int64_t> sn2;
        gbcomb::SpMXSpV<S2ND>(d, (int32_t)m, indx.data(), xi.data(), (int32_t)indx.size(), sy2, sn2, spa);
        EXPECT(fallback_calls() == fb + 2);  // last writer in heap order: the reference runs
        std::vector<std::vector<int32_t>> ty(4);
        std::vector<std::vector<int64_t>> tn(4);
        std::vector<std::thread> pool;
        for (int t = 0; t < 4; ++t)
            pool.emplace_back([&, t]() {
                for (int rep = 0; rep < 3; ++rep)
                    gbcomb::SpMXSpV_ForThreading<S2ND>(d, (int32_t)m, indx.data(), xi.data(), (int32_t)indx.size(),
                                                       ty[t], tn[t], off);
            });
        for (auto &th : pool) th.join();
        for (int t = 0; t < 4; ++t) check_rows(elast, ty[t], tn[t], 0);
        gbcomb::forget_matrices();
    }
    // 8. MultiwayMerge of three products of one shape (GPU) against the CPU merge
    {
        SpDCCols<I, double> *X = random_dcsc<double>(600, 300, 0.02, 0.1, 8);
        std::vector<SpTuples<I, double> *> lists, lists_cpu;
        for (unsigned k = 0; k < 3; ++k) {
            SpDCCols<I, double> *Y = random_dcsc<double>(300, 200, 0.03, 0.2, 20 + k);
            lists.push_back(combblas::LocalHybridSpGEMM<PT, double>(*X, *Y, false, false));
            lists_cpu.push_back(combblas::LocalHybridSpGEMM<PT, double>(*X, *Y, false, false));
            delete Y;
        }
        const int fb = fallback_calls();
        SpTuples<I, double> *mg = gbcomb::MultiwayMerge<PT>(lists, (I)600, (I)200, true);
        EXPECT(fallback_calls() == fb);
        SpTuples<I, double> *mc = combblas::MultiwayMerge<PT>(lists_cpu, (I)600, (I)200, true);
        EXPECT(mg->getnnz() > 0 && same(mg, mc) && !mg->opnew_);
        std::vector<SpTuples<I, double> *> bad{new SpTuples<I, double>(0, 600, 200),
                                              new SpTuples<I, double>(0, 601, 200)};
        SpTuples<I, double> *mb = gbcomb::MultiwayMerge<PT>(bad, (I)600, (I)200, true);
        EXPECT(mb->getnnz() == 0 && mb->getnrow() == 0);
        delete mb;
        delete bad[0];
        delete bad[1];
        delete mg;
        delete mc;
        delete X;
    }
    // 9. dcsc_gespmv over MinPlus int64 (order-free: bit-exact) on the GPU
    {
        typedef MinPlusSRing<int64_t, int64_t> MP;
        SpDCCols<I, int64_t> *M = random_dcsc<int64_t>(900, 400, 0.01, 0.2, 9);
        std::vector<int64_t> x(400), yg(900), yc(900);
        for (int j = 0; j < 400; ++j) x[j] = (j * 37) % 101;
        for (int r = 0; r < 900; ++r) yg[r] = yc[r] = 50 + (r * 13) % 77;
        const int fb = fallback_calls();
        const long long builds = gbcomb::detail::plan_builds();
        gbcomb::dcsc_gespmv<MP>(*M, x.data(), yg.data());
        EXPECT(fallback_calls() == fb);
        combblas::dcsc_gespmv<MP>(*M, x.data(), yc.data());
        EXPECT(yg == yc);
        // a second product with the same matrix reuses its device plan
        gbcomb::dcsc_gespmv<MP>(*M, x.data(), yg.data());
        combblas::dcsc_gespmv<MP>(*M, x.data(), yc.data());
        EXPECT(yg == yc && gbcomb::detail::plan_builds() == builds + 1);
        gbcomb::forget_matrices();  // before the matrix's memory is freed
        delete M;
    }
    delete B2;
    delete Bs;
    delete Ai;
    // 10. the default exact fold: same pattern, every value within 1e-12
    {
        gbcomb::set_fold(GBC_FOLD_EXACT);
        SpDCCols<I, double> *X = random_dcsc<double>(700, 500, 0.02, 0.3, 11);
        SpDCCols<I, double> *Y = random_dcsc<double>(500, 400, 0.03, 0.3, 12);
        SpTuples<I, double> *gx = gbcomb::LocalHybridSpGEMM<PT, double>(*X, *Y, false, false);
        SpTuples<I, double> *cx = combblas::LocalHybridSpGEMM<PT, double>(*X, *Y, false, false);
        bool ok = gx->getnnz() == cx->getnnz() && gx->getnnz() > 0;
        for (int64_t p = 0; ok && p < gx->getnnz(); ++p) {
            ok = std::get<0>(gx->tuples[p]) == std::get<0>(cx->tuples[p]) &&
                 std::get<1>(gx->tuples[p]) == std::get<1>(cx->tuples[p]);
            const double x = std::get<2>(gx->tuples[p]), y = std::get<2>(cx->tuples[p]);
            ok = ok && std::fabs(x - y) <= 1e-12 * std::fabs(y);
        }
        EXPECT(ok);
        delete gx;
        delete cx;
        delete X;
        delete Y;
    }
    if (failures == 0) std::printf("OK\n");
    return failures == 0 ? 0 : 1;
}
