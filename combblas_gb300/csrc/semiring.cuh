// Device semirings: one static-method struct per reference semiring, the same
// shape as the reference's SR::multiply / SR::add / SR::id (Semirings.h).
// one() is the value of an entry stored without a value array (a pattern
// matrix); unit() is the multiplicative identity: mul(unit(), x) == x.
// Floating-point multiply and add use the _rn intrinsics so that the
// compiler can never fuse them into an FMA: each product is rounded before
// it is added, as in the reference's `SR::add(SR::multiply(a, b), acc)`.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbc {

template <typename T>
struct PlusTimes;

template <>
struct PlusTimes<double> {
    typedef double V;
    static __device__ __forceinline__ V mul(V a, V b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ V add(V a, V b) { return __dadd_rn(a, b); }
    static __host__ __device__ __forceinline__ V one() { return 1.0; }
    static __host__ __device__ __forceinline__ V unit() { return 1.0; }
};

template <>
struct PlusTimes<float> {
    typedef float V;
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd_rn(a, b); }
    static __host__ __device__ __forceinline__ V one() { return 1.0f; }
    static __host__ __device__ __forceinline__ V unit() { return 1.0f; }
};

// Integer PlusTimes wraps modulo 2^64 (the reference's signed overflow on
// x86-64 and Arm behaves the same way).
template <>
struct PlusTimes<int64_t> {
    typedef int64_t V;
    static __device__ __forceinline__ V mul(V a, V b) { return (V)((uint64_t)a * (uint64_t)b); }
    static __device__ __forceinline__ V add(V a, V b) { return (V)((uint64_t)a + (uint64_t)b); }
    static __host__ __device__ __forceinline__ V one() { return 1; }
    static __host__ __device__ __forceinline__ V unit() { return 1; }
};

// PlusTimesSRing<bool,bool>: promote_trait<bool,bool> is bool, so add is
// logical or and multiply logical and (values are stored as 0/1 bytes).
struct BoolOrAnd {
    typedef uint8_t V;
    static __device__ __forceinline__ V mul(V a, V b) { return (V)((a != 0) & (b != 0)); }
    static __device__ __forceinline__ V add(V a, V b) { return (V)((a != 0) | (b != 0)); }
    static __host__ __device__ __forceinline__ V one() { return 1; }
    static __host__ __device__ __forceinline__ V unit() { return 1; }
};

// MinPlusSRing (Semirings.h:235-255) with inf_plus (Semirings.h:40-47):
// the type's max() is infinity and absorbs in multiply.
template <typename T>
struct MinPlus;

template <>
struct MinPlus<double> {
    typedef double V;
    static __device__ __forceinline__ V inf() { return 1.7976931348623157e308; }
    static __device__ __forceinline__ V mul(V a, V b) { return (a == inf() || b == inf()) ? inf() : __dadd_rn(a, b); }
    static __device__ __forceinline__ V add(V a, V b) { return (b < a) ? b : a; }  // std::min(a, b)
    static __host__ __device__ __forceinline__ V one() { return 1.0; }
    static __host__ __device__ __forceinline__ V unit() { return 0.0; }
};

template <>
struct MinPlus<int64_t> {
    typedef int64_t V;
    static __device__ __forceinline__ V inf() { return INT64_MAX; }
    static __device__ __forceinline__ V mul(V a, V b)
    {
        return (a == inf() || b == inf()) ? inf() : (V)((uint64_t)a + (uint64_t)b);
    }
    static __device__ __forceinline__ V add(V a, V b) { return (b < a) ? b : a; }
    static __host__ __device__ __forceinline__ V one() { return 1; }
    static __host__ __device__ __forceinline__ V unit() { return 0; }
};

// Select2ndMinSR (Applications/FastSV.h:25-44): multiply returns the second
// operand, add is min.
template <typename T>
struct Select2ndMin {
    typedef T V;
    static __device__ __forceinline__ V mul(V, V b) { return b; }
    static __device__ __forceinline__ V add(V a, V b) { return (b < a) ? b : a; }
    static __host__ __device__ __forceinline__ V one() { return 1; }
    static __host__ __device__ __forceinline__ V unit() { return 0; }  // any value: mul returns b
};

}  // namespace gbc
