// Compiles include/gbcomb/combblas_shim.hpp against the reference's own
// headers and forces every entry point of it -- GPU and fall-through paths --
// to instantiate with the real combblas types.  Compile-only check.
#include "CombBLAS/CombBLAS.h"
#include "CombBLAS/mtSpGEMM.h"
#include "gbcomb/combblas_shim.hpp"

namespace app {
template <class T1, class T2>
struct Select2ndMinSR {  // an application-defined semiring (FastSV.h defines its own)
    typedef typename combblas::promote_trait<T1, T2>::T_promote T_promote;
    static T_promote id() { return std::numeric_limits<T_promote>::max(); }
    static bool returnedSAID() { return false; }
    static MPI_Op mpi_op() { return MPI_MIN; }
    static T_promote add(const T_promote &a, const T_promote &b) { return std::min(a, b); }
    static T_promote multiply(const T1 &, const T2 &b) { return static_cast<T_promote>(b); }
    static void axpy(const T1 a, const T2 &x, T_promote &y) { y = add(y, multiply(a, x)); }
};
}  // namespace app
typedef app::Select2ndMinSR<int64_t, int64_t> S2M;
GBCOMB_REGISTER_SEMIRING(S2M, GBC_SR_SELECT2NDMIN, GBC_I64)

using namespace combblas;
typedef PlusTimesSRing<double, double> PTD;
typedef PlusTimesSRing<float, float> PTF;
typedef MinPlusSRing<int64_t, int64_t> MPI64;

template SpTuples<int64_t, double> *gbcomb::LocalHybridSpGEMM<PTD, double, int64_t, double, double>(
    const SpDCCols<int64_t, double> &, const SpDCCols<int64_t, double> &, bool, bool, int64_t *);
template SpTuples<int64_t, float> *gbcomb::LocalSpGEMM<PTF, float, int64_t, float, float>(
    const SpDCCols<int64_t, float> &, const SpDCCols<int64_t, float> &, bool, bool);
template SpTuples<int64_t, int64_t> *gbcomb::LocalSpGEMMHash<MPI64, int64_t, int64_t, int64_t, int64_t>(
    const SpDCCols<int64_t, int64_t> &, const SpDCCols<int64_t, int64_t> &, bool, bool, bool);
template SpTuples<int64_t, int64_t> *gbcomb::LocalHybridSpGEMM<S2M, int64_t, int64_t, int64_t, int64_t>(
    const SpDCCols<int64_t, int64_t> &, const SpDCCols<int64_t, int64_t> &, bool, bool, int64_t *);
template SpTuples<int64_t, double> *gbcomb::LocalHybridSpGEMM<PTD, double, int64_t, double, double>(
    const SpCCols<int64_t, double> &, const SpCCols<int64_t, double> &, bool, bool);
// fall-through: 32-bit indices are not offloaded
template SpTuples<int32_t, double> *gbcomb::LocalHybridSpGEMM<PTD, double, int32_t, double, double>(
    const SpDCCols<int32_t, double> &, const SpDCCols<int32_t, double> &, bool, bool, int32_t *);
template SpTuples<int32_t, double> *gbcomb::LocalSpGEMM<PTD, double, int32_t, double, double>(
    const SpDCCols<int32_t, double> &, const SpDCCols<int32_t, double> &, bool, bool);
template SpTuples<int32_t, double> *gbcomb::LocalSpGEMMHash<PTD, double, int32_t, double, double>(
    const SpDCCols<int32_t, double> &, const SpDCCols<int32_t, double> &, bool, bool, bool);
template SpTuples<int32_t, double> *gbcomb::LocalHybridSpGEMM<PTD, double, int32_t, double, double>(
    const SpCCols<int32_t, double> &, const SpCCols<int32_t, double> &, bool, bool);
template void gbcomb::SpMXSpV<PTD, int64_t, double, double, double>(
    const Csc<int64_t, double> &, int32_t, const int32_t *, const double *, int32_t, std::vector<int32_t> &,
    std::vector<double> &, PreAllocatedSPA<double> &);
template void gbcomb::SpMXSpV<S2M, int64_t, int64_t, int64_t, int64_t>(
    const Csc<int64_t, int64_t> &, int32_t, const int32_t *, const int64_t *, int32_t, std::vector<int32_t> &,
    std::vector<int64_t> &, PreAllocatedSPA<int64_t> &);

// the other SpMXSpV semirings: boolean Select2nd through the optbuf Dcsc
// overload (TopDownBFS), SelectMax and PlusTimes through the Csc overload
typedef Select2ndSRing<bool, int64_t, int64_t> S2ND;
typedef SelectMaxSRing<bool, int64_t> SMAX;
template void gbcomb::SpMXSpV<S2ND, int64_t, bool, int64_t, int64_t>(const Dcsc<int64_t, bool> &, int32_t,
                                                                     const int32_t *, const int64_t *, int32_t,
                                                                     int32_t *, int64_t *, int *, int *, int);
template void gbcomb::SpMXSpV<SMAX, int64_t, bool, int64_t, int64_t>(
    const Csc<int64_t, bool> &, int32_t, const int32_t *, const int64_t *, int32_t, std::vector<int32_t> &,
    std::vector<int64_t> &, PreAllocatedSPA<int64_t> &);
// fall-through: 32-bit indices
template void gbcomb::SpMXSpV<S2ND, int32_t, bool, int64_t, int64_t>(const Dcsc<int32_t, bool> &, int32_t,
                                                                     const int32_t *, const int64_t *, int32_t,
                                                                     int32_t *, int64_t *, int *, int *, int);

// the Dcsc overload with vector outputs: GPU for order-free semirings,
// the reference's heap for Select2nd
template void gbcomb::SpMXSpV<SMAX, int64_t, bool, int64_t, int64_t>(
    const Dcsc<int64_t, bool> &, int32_t, const int32_t *, const int64_t *, int32_t, std::vector<int32_t> &,
    std::vector<int64_t> &, PreAllocatedSPA<int64_t> &);
template void gbcomb::SpMXSpV<S2ND, int64_t, bool, int64_t, int64_t>(
    const Dcsc<int64_t, bool> &, int32_t, const int32_t *, const int64_t *, int32_t, std::vector<int32_t> &,
    std::vector<int64_t> &, PreAllocatedSPA<int64_t> &);

// the threaded SpMSpV over row pieces: GPU for boolean Dcsc pieces (both
// overloads) and order-free semirings on Csc pieces; fall-through for fp
// PlusTimes and non-boolean Dcsc pieces
template void gbcomb::SpMXSpV_ForThreading<S2ND, int64_t, bool, int64_t, int64_t>(
    const Dcsc<int64_t, bool> &, int32_t, const int32_t *, const int64_t *, int32_t, std::vector<int32_t> &,
    std::vector<int64_t> &, int32_t);
template void gbcomb::SpMXSpV_ForThreading<S2ND, int64_t, bool, int64_t, int64_t>(
    const Dcsc<int64_t, bool> &, int32_t, const int32_t *, const int64_t *, int32_t, std::vector<int32_t> &,
    std::vector<int64_t> &, int32_t, std::vector<int64_t> &, BitMap &, std::vector<uint32_t> &);
template void gbcomb::SpMXSpV_ForThreading<SMAX, int64_t, bool, int64_t, int64_t>(
    const Csc<int64_t, bool> &, int32_t, const int32_t *, const int64_t *, int32_t, std::vector<int32_t> &,
    std::vector<int64_t> &, int32_t);
template void gbcomb::SpMXSpV_ForThreading<S2M, int64_t, bool, int64_t, int64_t>(
    const Csc<int64_t, bool> &, int32_t, const int32_t *, const int64_t *, int32_t, std::vector<int32_t> &,
    std::vector<int64_t> &, int32_t, std::vector<int64_t> &, BitMap &, std::vector<uint32_t> &);
template void gbcomb::SpMXSpV_ForThreading<PTD, int64_t, double, double, double>(
    const Csc<int64_t, double> &, int32_t, const int32_t *, const double *, int32_t, std::vector<int32_t> &,
    std::vector<double> &, int32_t);
template void gbcomb::SpMXSpV_ForThreading<PTD, int64_t, double, double, double>(
    const Dcsc<int64_t, double> &, int32_t, const int32_t *, const double *, int32_t, std::vector<int32_t> &,
    std::vector<double> &, int32_t);

template SpTuples<int64_t, double> *gbcomb::MultiwayMerge<PTD, int64_t, double>(
    std::vector<SpTuples<int64_t, double> *> &, int64_t, int64_t, bool);
template SpTuples<int32_t, double> *gbcomb::MultiwayMerge<PTD, int32_t, double>(
    std::vector<SpTuples<int32_t, double> *> &, int32_t, int32_t, bool);

template void gbcomb::dcsc_gespmv<PTD, int64_t, double, double, double>(const SpDCCols<int64_t, double> &,
                                                                       const double *, double *);
template void gbcomb::dcsc_gespmv<PTD, int32_t, double, double, double>(const SpDCCols<int32_t, double> &,
                                                                       const double *, double *);

int main() { return 0; }
