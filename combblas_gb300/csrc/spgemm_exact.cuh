// Order-free exact accumulation for PlusTimes<double> SpGEMM columns.
//
// The reference folds each output entry as acc = add(mrhs, acc) over the B
// column's entries in ascending order (mtSpGEMM.h:396-412).  In fp64 that
// left fold is order dependent, so reproducing it on the GPU forces every
// product of one row to be applied in k order.  These kernels remove the
// order instead: every product p = fl(a * b) (rounded exactly as the
// reference rounds it) is an integer multiple of 2^(ebase - 1075), where
// ebase is the smallest product exponent of the column, so the column's
// products are added EXACTLY as integers, and each output entry is the exact
// sum rounded once to the nearest double (ties to even).  Integer addition
// is associative, so any interleaving of the products -- lane-parallel
// shared-memory atomics from all warps, unsorted buckets -- gives the same
// bits: repeated runs are bit-identical, and each value is the correctly
// rounded sum of the reference's own products, within the reference's own
// summation error of its hash-path and heap-path results.
//
// Dense accumulator: kXW signed 32-bit words per row, word i holding a
// signed multiple of 2^(kXP * i); a product's 53-bit mantissa is split into
// at most four kXP-bit pieces added with 32-bit shared atomics (about five
// times the rate of 64-bit shared atomics on this GPU).  Words are
// normalised (carries moved up) after at most kXNorm B entries, so no word
// overflows.  A column is admitted when all its products are normal and
// finite and
//   span + 53 <= kXP * kXW               (every piece has a word)
//   span + 53 + lg(nnz(B(:,j))) <= 125   (the exact sum fits 126 bits)
// with span = (largest - smallest product exponent) bounded from per-column
// exponent ranges of A and the B values; other columns (subnormal values,
// possible underflow, inf/nan, very wide ranges) are listed for the ordered
// kernel.
#pragma once

#include <stdint.h>

#include "semiring.cuh"
#include "spgemm_kernels.cuh"

namespace gbc {

constexpr int kXP = 19;                      // payload bits per accumulator word
constexpr int kXW = 6;                       // words per row
constexpr uint32_t kXMask = (1u << kXP) - 1;
constexpr int kXOMax = kXP * kXW - 53;       // largest product exponent above the base (61)
constexpr int kXNorm = 2047;                 // B entries between carry normalisations
// Accumulator tiles and block shapes of k_numeric_x: RS rows (24 B of words
// + 1 flag byte each) in shared memory; 4096 rows with 512 threads (two
// blocks per SM) or 8192 rows with 1024 threads (one block per SM).
constexpr int kXRows = 4096;
constexpr int kXThreads = 512;
constexpr int kXRowsBig = 8192;
constexpr int kXThreadsBig = 1024;

// Phase clocks of k_numeric_x for profiling builds (-DGBC_XPROF): thread 0
// of every block adds the cycles between two block barriers to a counter.
#ifdef GBC_XPROF
__device__ unsigned long long g_xprof[32];
#define XPROF_T0 long long xp_t = clock64()
#define XPROF_LAP(id)                                                          \
    do {                                                                       \
        if (threadIdx.x == 0) {                                                \
            const long long xp_n = clock64();                                  \
            atomicAdd(&g_xprof[id], (unsigned long long)(xp_n - xp_t));        \
            xp_t = xp_n;                                                       \
        }                                                                      \
    } while (0)
#define XPROF_ADD(id, v)                                                       \
    do {                                                                       \
        if (threadIdx.x == 0) atomicAdd(&g_xprof[id], (unsigned long long)(v)); \
    } while (0)
extern "C" int gbc_xprof_read(unsigned long long *out, int reset)
{
    cudaMemcpyFromSymbol(out, g_xprof, sizeof(g_xprof));
    if (reset) {
        static const unsigned long long z[32] = {};
        cudaMemcpyToSymbol(g_xprof, z, sizeof(z));
    }
    return (int)cudaDeviceSynchronize();
}
#else
#define XPROF_T0
#define XPROF_LAP(id)
#define XPROF_ADD(id, v)
#endif

// Per column of A: smallest and largest biased exponent of its nonzero
// values, packed as (int16 min) | (int16 max << 16).  Subnormal values count
// as exponent -64 (their products can underflow: such columns take the
// ordered kernel); a column without nonzero values gets min > max.
static __global__ void k_aexp_f64(int64_t ncol, const int64_t *acp, const double *aval, int32_t *aexp)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t c = warp; c < ncol; c += nwarps) {
        int lo = 32767, hi = -32768;
        for (int64_t p = acp[c] + lane; p < acp[c + 1]; p += 32) {
            const uint64_t bits = (uint64_t)__double_as_longlong(aval ? aval[p] : 1.0);
            int e = (int)((bits >> 52) & 0x7ff);
            const bool zero = (bits << 1) == 0;
            if (e == 0) e = -64;
            if (!zero) {
                lo = min(lo, e);
                hi = max(hi, e);
            }
        }
        lo = __reduce_min_sync(0xffffffffu, lo);
        hi = __reduce_max_sync(0xffffffffu, hi);
        if (lane == 0) aexp[c] = (int32_t)(((uint32_t)(uint16_t)(int16_t)lo) | ((uint32_t)(uint16_t)(int16_t)hi << 16));
    }
}

// Round-to-nearest-even product of two nonzero normal doubles whose exact
// product is normal and finite (what admitted columns hold), restated in
// integer arithmetic from IEEE 754: the 53-bit mantissas are multiplied
// exactly (106 bits), rounded to 53 bits, ties to even.  Returns the 53-bit
// mantissa q (2^52 <= q < 2^53) and the biased exponent e, so that
// |a * b| rounds to q * 2^(e - 1075).  (GB300's fp64 pipe issues about two
// multiplies per SM clock; the integer units do this several times faster,
// and the accumulator needs the integer mantissa anyway.)
__device__ __forceinline__ void x_mul(uint64_t abits, uint64_t bbits, uint64_t &q, int &e)
{
    const uint64_t ma = (abits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const uint64_t mb = (bbits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    e = (int)((abits >> 52) & 0x7ff) + (int)((bbits >> 52) & 0x7ff) - 1023;
    const uint64_t lo = ma * mb, hi = __umul64hi(ma, mb);  // 2^104 <= ma * mb < 2^106
    const int top = (int)(hi >> 41);                        // 1 when bit 105 is set
    const int sh = 52 + top;                                // bits below the kept 53
    q = (hi << (64 - sh)) | (lo >> sh);
    const uint64_t rem = lo & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    q += (rem > half || (rem == half && (q & 1))) ? 1ull : 0ull;
    e += top;
    if (q >> 53) {  // rounded up to 2^53
        q >>= 1;
        ++e;
    }
}

// The product's double (bit pattern): +-0 when a factor is zero.
__device__ __forceinline__ uint64_t x_mul_bits(uint64_t abits, uint64_t bbits)
{
    const uint64_t sign = (abits ^ bbits) & (1ull << 63);
    if ((abits << 1) == 0 || (bbits << 1) == 0) return sign;
    uint64_t q;
    int e;
    x_mul(abits, bbits, q, e);
    return sign | ((uint64_t)e << 52) | (q & 0xFFFFFFFFFFFFFull);
}

// Add the product a * b (bit patterns of two values of an admitted column:
// zero or normal, product normal) to row r of the accumulator (words at
// acc[i * stride + r]) and mark the row touched in its flag byte (bit 0
// touched, bit 1 touched by something other than -0.0, which decides the
// sign of an exact zero sum); a row's first touch counts it in band[r / 256]
// (touched rows per 256-row band, the write-out's offsets).  Returns false when the product lies outside
// the column's admitted exponent window (cannot happen for admitted
// columns; nothing is added then).
__device__ __forceinline__ bool x_add(int32_t *acc, int stride, uint32_t *tw, int32_t *band, int r, uint64_t abits,
                                      uint64_t bbits, int ebase)
{
    const bool neg = ((abits ^ bbits) >> 63) != 0;
    const int sh8 = (r & 3) << 3;
    const bool zero = (abits << 1) == 0 || (bbits << 1) == 0;  // a zero product: +0.0 or -0.0
    const uint32_t old = atomicOr(&tw[r >> 2], ((zero && neg) ? 1u : 3u) << sh8);
    if (((old >> sh8) & 0xff) == 0) atomicAdd(&band[r >> 8], 1);  // first touch: count the row in its band
    if (zero) return true;
    uint64_t m;
    int ex;
    x_mul(abits, bbits, m, ex);
    const int o = ex - ebase;
    if ((unsigned)o > (unsigned)kXOMax) return false;
    const int w0 = o / kXP;
    const int bsh = o - kXP * w0;
    const uint64_t lo = m << bsh;
    const uint64_t hi = bsh ? (m >> (64 - bsh)) : 0ull;
    int32_t q0 = (int32_t)(lo & kXMask);
    int32_t q1 = (int32_t)((lo >> kXP) & kXMask);
    int32_t q2 = (int32_t)((lo >> (2 * kXP)) & kXMask);
    int32_t q3 = (int32_t)((lo >> (3 * kXP)) | (hi << (64 - 3 * kXP)));
    if (neg) {
        q0 = -q0;
        q1 = -q1;
        q2 = -q2;
        q3 = -q3;
    }
    // the top nonzero piece is in word (o + 52) / kXP <= kXW - 1
    int32_t *base = acc + w0 * stride + r;
    if (q0) atomicAdd(base, q0);
    if (q1) atomicAdd(base + stride, q1);
    if (q2) atomicAdd(base + 2 * stride, q2);
    if (q3) atomicAdd(base + 3 * stride, q3);
    return true;
}

// Move the carries of row r's words up (word i keeps its value mod 2^kXP,
// the top word keeps the rest).
__device__ __forceinline__ void x_normalise(int32_t *acc, int stride, int r)
{
    int32_t carry = 0;
#pragma unroll
    for (int i = 0; i < kXW - 1; ++i) {
        const int32_t v = acc[i * stride + r] + carry;
        acc[i * stride + r] = (int32_t)((uint32_t)v & kXMask);
        carry = v >> kXP;
    }
    acc[(kXW - 1) * stride + r] += carry;
}

// Round a signed 128-bit integer M (two's complement hi:lo), times
// 2^(ebase - 1075), to the nearest double (ties to even), in integer
// arithmetic (IEEE 754 rounding of the exact value; GB300's fp64 units are
// slow).  flag bit 1 says whether some term was other than -0.0: an exact
// zero sum is then +0.0, else -0.0 (what the left fold of the reference
// gives).  For admitted columns |M| < 2^126 and the result is finite.
__device__ __forceinline__ double x_round(uint64_t hi, uint64_t lo, uint32_t flag, int ebase)
{
    const bool neg = (int64_t)hi < 0;
    if (neg) {
        lo = ~lo + 1;
        hi = ~hi + (lo == 0 ? 1ull : 0ull);
    }
    if ((hi | lo) == 0) return (flag & 2) ? 0.0 : -0.0;
    const int tb = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);  // top bit of |M|
    const int e = tb + ebase - 52;  // biased exponent when the result is normal
    uint64_t bits;
    if (e <= 0) {
        // subnormal: |M| * 2^(ebase - 1) < 2^52 is the exact subnormal mantissa
        bits = lo << (ebase - 1);
    } else if (tb <= 52) {
        bits = ((uint64_t)e << 52) + ((lo << (52 - tb)) & 0xFFFFFFFFFFFFFull);  // exact
    } else {
        const int sh = tb - 52;  // 1..73 bits below the 53 kept
        uint64_t m, rnd, sticky;
        if (sh < 64) {
            m = (lo >> sh) | (sh ? (hi << (64 - sh)) : 0ull);
            rnd = (lo >> (sh - 1)) & 1;
            sticky = (sh > 1 && (lo << (65 - sh)) != 0) ? 1 : 0;
        } else {
            m = hi >> (sh - 64);
            rnd = sh == 64 ? (lo >> 63) : ((hi >> (sh - 65)) & 1);
            sticky = (lo & (sh == 64 ? 0x7FFFFFFFFFFFFFFFull : ~0ull)) != 0 ||
                     (sh > 65 && (hi << (129 - sh)) != 0);
        }
        m += (rnd && (sticky || (m & 1))) ? 1 : 0;  // may carry into 2^53: the exponent field absorbs it
        bits = ((uint64_t)(e - 1) << 52) + m;
    }
    return __longlong_as_double((long long)(bits | (neg ? (1ull << 63) : 0ull)));
}

// The exact sum of row r's words, rounded (x_round); clears the words.
__device__ __forceinline__ double x_value(int32_t *acc, int stride, int r, uint32_t flag, int ebase)
{
    uint64_t lo = 0, hi = 0;
#pragma unroll
    for (int i = 0; i < kXW; ++i) {
        const int64_t s = acc[i * stride + r];
        acc[i * stride + r] = 0;
        const int sh = kXP * i;
        uint64_t pl, ph;
        if (sh == 0) {
            pl = (uint64_t)s;
            ph = (uint64_t)(s >> 63);
        } else if (sh < 64) {
            pl = (uint64_t)s << sh;
            ph = (uint64_t)(s >> (64 - sh));
        } else {
            pl = 0;
            ph = (uint64_t)s << (sh - 64);
        }
        lo += pl;
        hi += ph + (lo < pl ? 1ull : 0ull);
    }
    return x_round(hi, lo, flag, ebase);
}

// Add product p (a double of an admitted column) exactly to a register
// accumulator hi:lo (units of 2^(ebase - 1075)); flag as in x_add.  False
// when p is outside the window.
__device__ __forceinline__ bool x_acc128(uint64_t &hi, uint64_t &lo, uint32_t &flag, double p, int ebase)
{
    const uint64_t bits = (uint64_t)__double_as_longlong(p);
    const int ex = (int)((bits >> 52) & 0x7ff);
    if (bits != (1ull << 63)) flag |= 2;
    if (ex == 0) return (bits << 1) == 0;
    const int o = ex - ebase;
    if ((unsigned)o > (unsigned)kXOMax) return false;
    const uint64_t m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const uint64_t pl = m << o;
    const uint64_t ph = o ? (m >> (64 - o)) : 0ull;
    if (bits >> 63) {
        const uint64_t old = lo;
        lo -= pl;
        hi -= ph + (old < pl ? 1ull : 0ull);
    } else {
        lo += pl;
        hi += ph + (lo < pl ? 1ull : 0ull);
    }
    return true;
}

// Exponent window of one B entry's products (A column k's value range
// times b): updates emin (smallest product exponent) and emax (largest,
// allowing for rounding up).  Entries whose products are all zero are skipped.
__device__ __forceinline__ void x_window(int32_t ae, double b, bool has_b, int &emin, int &emax)
{
    const int amin = (int16_t)(ae & 0xffff), amax = (int16_t)((uint32_t)ae >> 16);
    const uint64_t bb = has_b ? (uint64_t)__double_as_longlong(b) : 0x3FF0000000000000ull;
    int eb = (int)((bb >> 52) & 0x7ff);
    if (amin > amax || (bb << 1) == 0) return;
    if (eb == 0) eb = -64;  // subnormal b
    emin = min(emin, amin + eb - 1023);
    emax = max(emax, amax + eb - 1022);
}

// Is a column with product exponents in [ebase, etop] and nb B entries
// summed exactly?  (Every product normal and finite, every piece inside the
// words, the exact sum inside 126 bits, the rounded result finite.)  An
// all-zero column (ebase > etop) is admitted with ebase 1.
__device__ __forceinline__ bool x_admit(int &ebase, int etop, int64_t nb)
{
    if (ebase > etop) {
        ebase = 1;
        return true;
    }
    const int lg = 64 - __clzll((long long)nb);
    return ebase >= 1 && etop <= 2046 - lg - 2 && (etop - ebase) <= kXOMax && (etop - ebase) + 53 + lg <= 125;
}

// Per column k of A, its row tiles as a compressed list (the DCSC of the
// column's tile structure): entries ptr[k] .. ptr[k+1]-1 hold, for each
// touched tile in order, the tile and the first position of A(:,k) inside
// it, followed by one end marker (tile 0xFFFF, start = the column's end).
static __global__ void k_ktl_count(int64_t ncol, const uint64_t *amask, int mask_words, int64_t *cnt)
{
    const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    int64_t n = 1;
    for (int w = 0; w < mask_words; ++w) n += __popcll(amask[c * mask_words + w]);
    cnt[c] = n;
}

// One warp per column; lanes test 32 tiles at a time.
static __global__ void k_ktl_fill(int64_t ncol, const uint32_t *tptr, int T, const int64_t *ptr, uint32_t *kstart,
                           uint16_t *ktile)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t c = warp; c < ncol; c += nwarps) {
        const uint32_t *tp = tptr + c * (int64_t)(T + 1);
        int64_t o = ptr[c];
        for (int t0 = 0; t0 < T; t0 += 32) {
            const int t = t0 + lane;
            const bool nz = t < T && tp[t + 1] > tp[t];
            const unsigned m = __ballot_sync(0xffffffffu, nz);
            if (nz) {
                const int64_t q = o + __popc(m & ((1u << lane) - 1));
                kstart[q] = tp[t];
                ktile[q] = (uint16_t)t;
            }
            o += __popc(m);
        }
        if (lane == 0) {
            kstart[o] = tp[T];
            ktile[o] = 0xFFFF;
        }
    }
}

// One segment of a bucketed column: A's positions [start, start + len)
// (one row tile of one A column) times the column's B entry e.
struct XSeg {
    uint32_t start, len, e;
};

constexpr int kXTMax = 256;                   // row tiles of a bucketed column
constexpr int kXRange = 4096;                 // products of one sorted range visit (at most; RS for smaller tiles)
#ifndef GBC_XDENSE
#define GBC_XDENSE 512
#endif
constexpr int kXDense = GBC_XDENSE;           // a tile with more products is a dense visit
constexpr int64_t kXScap = int64_t(1) << 18;  // bucketed segments of one column (per-block scratch)

// Numeric pass for the columns of the big list, one block per column
// (dynamic counter).  After the column's exponent window is admitted:
//  1. bucketing -- every (B entry, touched row tile of its A column) pair is
//     counted per tile (segments and products) and written, in any order,
//     into the block's scratch grouped by tile (a counting sort; the exact
//     sum makes the order irrelevant).  Each tile is then visited with its
//     own segments only, instead of looking up every B entry per tile.
//  2. visits in row order -- a tile with more than kXDense products is a
//     dense visit: products added with x_add into the shared-memory word
//     accumulator, touched rows written in row order.  Consecutive lighter
//     tiles are merged into one range of at most kXRange products (RS for
//     smaller tiles): the
//     products (x_mul) are staged in shared memory with (row, slot) keys,
//     radix sorted by row (stable LSD, 7-bit digits), and each run of one
//     row is summed exactly (x_acc128) and rounded (x_round).
// Columns with more than kXScap segments, or matrices with more than
// 2^20 / RS tiles, visit every touched tile and look up their B entries' A
// segments per tile (tptr) instead of step 1.  Columns outside the exact
// window are appended to fb_items for the ordered kernel.
template <int NT, int RS>
__global__ void __launch_bounds__(NT, 1024 / NT)
    k_numeric_x(const SpgemmArgs *args, const int64_t *items, int64_t nitems, const int64_t *ccp, int64_t ccp_base,
                const int64_t *cap, int64_t *out_cnt, int32_t *overflow, int64_t *cir, double *cval,
                unsigned long long *work, int64_t *fb_items, unsigned long long *fb_count, XSeg *scratch_all)
{
    constexpr int NW = NT / 32;  // RS: rows of the tile = word stride
    constexpr int TM = (1 << 20) / RS;             // tiles of a bucketed column
    constexpr int XR = RS < kXRange ? RS : kXRange;  // products of one range visit
    // TM <= NT: the bucketing's block-wide prefix gives every tile its offset
    static_assert(XR <= 4096 && XR >= kXDense && (NW * 128) % NT == 0 && RS % (32 * NW) == 0 &&
                      TM * RS <= (1 << 20) && TM <= kXTMax && TM <= NT,
                  "range keys: 20-bit row offset and 12-bit slot; eight sorted keys per thread");
    extern __shared__ __align__(16) int32_t xsm[];
    int32_t *acc = xsm;                                           // [kXW][RS]
    uint32_t *tw = reinterpret_cast<uint32_t *>(xsm + kXW * RS);  // [RS/4] flag bytes
    uint8_t *tfb = reinterpret_cast<uint8_t *>(tw);
    // range visits reuse the word area (it is cleared again before a dense visit)
    uint32_t *rk0 = reinterpret_cast<uint32_t *>(xsm);          // [XR] keys
    uint32_t *rk1 = rk0 + XR;                                   // [XR] keys (sort buffer)
    uint64_t *rval = reinterpret_cast<uint64_t *>(rk1 + XR);    // [XR] products
    uint32_t *rwh = reinterpret_cast<uint32_t *>(rval + XR);    // [NW][128] digit counts per warp
    static_assert(2 * XR * 4 + XR * 8 + NW * 128 * 4 <= kXW * RS * 4, "range area inside the words");
    __shared__ ChunkSmemN<NT> ch;
    static_assert(sizeof(ChunkSmemN<NT>) >= NW * 128 * 2, "write-out row lists fit the chunk table");
    __shared__ uint32_t ch_e[NT];
    __shared__ int32_t s_segcnt[TM], s_prodcnt[TM], s_off[TM + 1];
    __shared__ int32_t s_wsum[NW];
    __shared__ int32_t s_band[RS / 256];  // touched rows per 256-row band of the dense tile
    __shared__ int32_t s_emin[NW], s_emax[NW];
    __shared__ int64_t s_col;
    __shared__ SpgemmArgs sa;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1;
    XSeg *scratch = scratch_all + (int64_t)blockIdx.x * kXScap;
    for (int u = tid; u < kXW * RS + RS / 4; u += NT) xsm[u] = 0;
    for (int u = tid; u < RS / 256; u += NT) s_band[u] = 0;
    bool dirty = false;  // the word area holds a range visit's data
    bool first_item = true;
    XPROF_T0;

    // block-wide exclusive prefix of v over the threads (two barriers); *tot the sum
    auto block_prefix = [&](int v, int *tot) -> int {
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_wsum[warp] = x;
        __syncthreads();
        int before = 0, all = 0;
#pragma unroll
        for (int u = 0; u < NW; ++u) {
            const int ws = s_wsum[u];
            before += u < warp ? ws : 0;
            all += ws;
        }
        __syncthreads();
        *tot = all;
        return before + x - v;
    };

    // products of one chunk of segments (ch, ch_e) flattened over the warps:
    // f(b, idx, p) for product p of segment b at A position idx
    auto for_products = [&](int L, int nseg, auto &&f) {
        const int span = (((L + NW - 1) / NW) + 31) & ~31;
        const int wb = warp * span, we = min(L, wb + span);
        if (wb < we) {
            int bcur = chunk_find_nz(ch, nseg, wb);
            for (int p0 = wb; p0 < we; p0 += 32) {
                const int p = p0 + lane;
                const int b = window_seg(ch, nseg, bcur, p);
                if (p < we) f(b, (int64_t)(uint32_t)(ch.base[b] + (uint32_t)p), p);
                int bn = __shfl_sync(0xffffffffu, b, 31);
                if (bn + 1 < nseg && ch.off[bn + 1] <= p0 + 32) ++bn;
                bcur = bn;
            }
        }
    };

    for (;;) {
        if (tid == 0) {
            s_col = next_item(work, first_item);
            if (s_col < nitems) sa = args[item_pid(items[s_col])];
        }
        __syncthreads();
        const int64_t ci = s_col;
        if (ci >= nitems) break;
        const SpgemmArgs &a = sa;
        const int64_t i = item_col(items[ci]);
        const int64_t g = a.col_base + i;
        const double *aval = static_cast<const double *>(a.aval);
        const double *bval = static_cast<const double *>(a.bval);
        const int64_t bs = a.bcp[i], be = a.bcp[i + 1];
        const int64_t out0 = ccp[g - ccp_base];
        int64_t out = out0;
        const int64_t lim = cap ? out0 + cap[g] : ccp[g - ccp_base + 1];
        bool over = false, bad = false;

        // admission: the exponent window of the column's products
        {
            int emin = 1 << 30, emax = -(1 << 30);
            for (int64_t b = bs + tid; b < be; b += NT)
                x_window(a.aexp[a.brow[b]], bval ? bval[b] : 1.0, bval != nullptr, emin, emax);
            emin = __reduce_min_sync(0xffffffffu, emin);
            emax = __reduce_max_sync(0xffffffffu, emax);
            if (lane == 0) {
                s_emin[warp] = emin;
                s_emax[warp] = emax;
            }
        }
        __syncthreads();
        int ebase = 1 << 30, etop = -(1 << 30);
#pragma unroll
        for (int u = 0; u < NW; ++u) {
            ebase = min(ebase, s_emin[u]);
            etop = max(etop, s_emax[u]);
        }
        if (!x_admit(ebase, etop, be - bs)) {
            if (tid == 0) fb_items[atomicAdd(fb_count, 1ull)] = items[ci];
            __syncthreads();  // s_col / sa / s_emin reuse
            continue;
        }
        XPROF_LAP(0);

        // dense visit helpers: products of a chunk into the word accumulator,
        // and the write-out of tile row0's touched rows
        // (the loads of the next 32-product window are issued before the
        // current window's atomics, so their latency overlaps them)
        auto dense_products = [&](int L, int nseg, int row0) {
            const int span = (((L + NW - 1) / NW) + 31) & ~31;
            const int wb = warp * span, we = min(L, wb + span);
            if (wb >= we) return;
            int bcur = chunk_find_nz(ch, nseg, wb);
            int r_n = 0;
            uint64_t a_n = 0, b_n = 0;
            bool v_n = false;
            auto load = [&](int p0) {
                const int p = p0 + lane;
                const int b = window_seg(ch, nseg, bcur, p);
                v_n = p < we;
                if (v_n) {
                    const int64_t idx = (uint32_t)(ch.base[b] + (uint32_t)p);
                    r_n = a.arow[idx] - row0;
                    a_n = (uint64_t)__double_as_longlong(aval ? aval[idx] : 1.0);
                    b_n = (uint64_t)__double_as_longlong(bval ? bval[bs + ch_e[b]] : 1.0);
                }
                int bn = __shfl_sync(0xffffffffu, b, 31);
                if (bn + 1 < nseg && ch.off[bn + 1] <= p0 + 32) ++bn;
                bcur = bn;
            };
            load(wb);
            for (int p0 = wb; p0 < we; p0 += 32) {
                const int r = r_n;
                const uint64_t av = a_n, bv = b_n;
                const bool v = v_n;
                if (p0 + 32 < we) load(p0 + 32);  // warp-uniform
                if (v && !x_add(acc, RS, tw, s_band, r, av, bv, ebase)) bad = true;
            }
        };
        // (callers end the products with a block barrier)
        auto dense_writeout = [&](int row0) {
            // warp w writes the rows of 256-row bands w, w + NW, ... in order;
            // offsets from the bands' first-touch counts
            static_assert(RS / 256 <= 32, "bands fit one warp");
            const int nband = (a.R + 255) >> 8;
            const int bc = lane < nband ? s_band[lane] : 0;
            int inc = bc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += y;
            }
            const int tot = __shfl_sync(0xffffffffu, inc, 31);
            __syncthreads();  // every warp has read the band counts before they are reset
            XPROF_LAP(16);
            XPROF_ADD(18, tot);
            for (int bd = warp; bd < nband; bd += NW) {
                const int before = __shfl_sync(0xffffffffu, inc - bc, bd);
                if (lane == 0) s_band[bd] = 0;
                const int g0 = bd * 8, g1 = min(a.R >> 5, g0 + 8);
                int64_t pos = out + before;
            // touched rows of 4 groups at a time listed in order (the chunk
            // table's space, 128 rows per warp), then converted one per lane
            uint16_t *wl = reinterpret_cast<uint16_t *>(&ch) + warp * 128;
            for (int gb = g0; gb < g1; gb += 4) {
                int n = 0;
                for (int gg = gb; gg < min(g1, gb + 4); ++gg) {
                    const int r = gg * 32 + lane;
                    const bool f = tfb[r] != 0;
                    const unsigned m = __ballot_sync(0xffffffffu, f);
                    if (f) wl[n + __popc(m & lt)] = (uint16_t)r;
                    n += __popc(m);
                }
                __syncwarp();
                for (int k = lane; k < n; k += 32) {
                    const int r = wl[k];
                    const double v = x_value(acc, RS, r, tfb[r], ebase);
                    tfb[r] = 0;
                    const int64_t q = pos + k;
                    if (q < lim) {
                        cir[q] = (int64_t)row0 + r;
                        cval[q] = v;
                    } else {
                        over = true;
                    }
                }
                pos += n;
                __syncwarp();
            }
            }
            out += tot;
            XPROF_LAP(17);
            __syncthreads();
        };
        auto clean_words = [&]() {
            if (dirty) {
                for (int u = tid; u < kXW * RS; u += NT) xsm[u] = 0;
                dirty = false;
                __syncthreads();
            }
        };

        // ------------------------------------------------ 1. bucketing
        bool bucketed = a.T <= TM && a.ktl_ptr != nullptr;  // block-uniform
        if (bucketed) {
            for (int u = tid; u < a.T; u += NT) {
                s_segcnt[u] = 0;
                s_prodcnt[u] = 0;
            }
            __syncthreads();
            // pass 0 counts, pass 1 scatters: the (entry, tile) pairs of a
            // chunk of NT entries are flattened over the warps like products
            for (int pass = 0; pass < 2; ++pass) {
                for (int64_t cb = bs; cb < be; cb += NT) {
                    const int64_t e = cb + tid;
                    uint32_t s0 = 0;
                    int len = 0;
                    if (e < be) {
                        const int k = a.brow[e];
                        const int64_t p0 = a.ktl_ptr[k];
                        s0 = (uint32_t)p0;
                        len = (int)(a.ktl_ptr[k + 1] - p0) - 1;  // touched tiles (the end marker excluded)
                    }
                    int nseg;
                    const int L = compact_chunk<uint32_t, NT>(ch, s0, len, (uint32_t)(e - bs), ch_e, nseg);
                    for_products(L, nseg, [&](int b, int64_t q, int) {
                        const int t = a.ktl_tile[q];
                        const uint32_t st = a.ktl_start[q];
                        const int ln = (int)(a.ktl_start[q + 1] - st);
                        if (pass == 0) {
                            atomicAdd(&s_segcnt[t], 1);
                            atomicAdd(&s_prodcnt[t], ln);
                        } else {
                            const int pos = atomicAdd(&s_off[t], 1);
                            scratch[pos] = XSeg{st, (uint32_t)ln, ch_e[b]};
                        }
                    });
                }
                __syncthreads();
                if (pass == 0) {
                    // tile offsets; a column with too many segments is not bucketed
                    int tot;
                    const int ex = block_prefix(tid < a.T ? s_segcnt[tid] : 0, &tot);
                    if (tot > kXScap) {
                        bucketed = false;  // block-uniform: tot is
                        break;
                    }
                    if (tid < a.T) s_off[tid] = ex;
                    __syncthreads();
                }
            }
            // s_off[t] is now the end of tile t's segments
            XPROF_LAP(1);
            XPROF_ADD(bucketed ? 11 : 12, 1);
        }

        if (bucketed) {
            // -------------------------------------------- 2. visits in row order
            int t = 0;
            while (t < a.T) {
                const int nsg = s_segcnt[t];
                if (nsg == 0) {
                    ++t;
                    continue;
                }
                if (s_prodcnt[t] > kXDense) {
                    // dense visit of tile t
                    clean_words();
                    const int row0 = t * a.R;
                    const int sb = s_off[t] - nsg;
                    int since_norm = 0;
                    for (int c0 = 0; c0 < nsg; c0 += NT) {
                        const int nent = min(NT, nsg - c0);
                        if (since_norm + nent > kXNorm) {
                            __syncthreads();
                            for (int r = tid; r < a.R; r += NT)
                                if (tfb[r]) x_normalise(acc, RS, r);
                            since_norm = 0;
                        }
                        since_norm += nent;
                        uint32_t s0 = 0, e0 = 0;
                        int len = 0;
                        if (tid < nent) {
                            const XSeg sg = scratch[sb + c0 + tid];
                            s0 = sg.start;
                            len = (int)sg.len;
                            e0 = sg.e;
                        }
                        int nseg;
                        const int L = compact_chunk<uint32_t, NT>(ch, s0, len, e0, ch_e, nseg);
                        dense_products(L, nseg, row0);
                        XPROF_ADD(14, L);
                    }
                    __syncthreads();
                    XPROF_LAP(2);
                    dense_writeout(row0);
                    XPROF_LAP(3);
                    XPROF_ADD(8, 1);
                    if (tid == 0) atomicAdd(&work[1], 1ull);  // dense visits (statistics)
                    ++t;
                } else {
                    // range visit of light tiles t .. t1 (at most kXRange products)
                    int t1 = t, prods = s_prodcnt[t];
                    while (t1 + 1 < a.T && (s_segcnt[t1 + 1] == 0 ||
                                            (s_prodcnt[t1 + 1] <= kXDense && prods + s_prodcnt[t1 + 1] <= XR))) {
                        ++t1;
                        prods += s_prodcnt[t1];
                    }
                    while (s_segcnt[t1] == 0) --t1;  // end on a touched tile
                    const int rbase = t * a.R;
                    const int span_rows = (t1 - t + 1) * a.R;  // <= 2^20
                    const int sb = s_off[t] - s_segcnt[t], se = s_off[t1];
                    dirty = true;
                    // stage: key = (row - rbase) << 12 | slot, value = the product
                    int pbase = 0;
                    for (int c0 = sb; c0 < se; c0 += NT) {
                        uint32_t s0 = 0, e0 = 0;
                        int len = 0;
                        if (c0 + tid < se) {
                            const XSeg sg = scratch[c0 + tid];
                            s0 = sg.start;
                            len = (int)sg.len;
                            e0 = sg.e;
                        }
                        int nseg;
                        const int L = compact_chunk<uint32_t, NT>(ch, s0, len, e0, ch_e, nseg);
                        for_products(L, nseg, [&](int b, int64_t idx, int p) {
                            const int slot = pbase + p;
                            const double av = aval ? aval[idx] : 1.0;
                            const double bv = bval ? bval[bs + ch_e[b]] : 1.0;
                            rk0[slot] = ((uint32_t)(a.arow[idx] - rbase) << 12) | (uint32_t)slot;
                            rval[slot] = x_mul_bits((uint64_t)__double_as_longlong(av),
                                                    (uint64_t)__double_as_longlong(bv));
                        });
                        pbase += L;
                        __syncthreads();  // chunk table reuse
                    }
                    XPROF_LAP(4);
                    XPROF_ADD(9, 1);
                    if (tid == 0) atomicAdd(&work[2], 1ull);  // range visits (statistics)
                    XPROF_ADD(13, prods);
                    // stable LSD radix sort of the keys by row, 7-bit digits:
                    // warp w owns a contiguous run of keys, counts its digits,
                    // the (digit, warp) counts are scanned digit-major, and
                    // each warp scatters its keys in order (rank inside a
                    // 32-key window from seven ballots)
                    const int rbits = span_rows > 1 ? 32 - __clz(span_rows - 1) : 1;
                    uint32_t *src = rk0, *dst = rk1;
                    const int per = (((prods + NW - 1) / NW) + 31) & ~31;
                    const int k0 = min(prods, warp * per), k1 = min(prods, k0 + per);
                    uint32_t *wh = rwh + warp * 128;
                    for (int shift = 12; shift < 12 + rbits; shift += 7) {
                        for (int u = lane; u < 128; u += 32) wh[u] = 0;
                        __syncwarp();
                        for (int u = k0 + lane; u < k1; u += 32) atomicAdd(&wh[(src[u] >> shift) & 127], 1u);
                        __syncthreads();
                        {  // exclusive scan over (digit, warp), digit-major
                            constexpr int PER = NW * 128 / NT;
                            int loc[PER], sum = 0;
#pragma unroll
                            for (int j = 0; j < PER; ++j) {
                                const int idx = tid * PER + j, d = idx / NW, w = idx - d * NW;
                                loc[j] = (int)rwh[w * 128 + d];
                                sum += loc[j];
                            }
                            int tot;
                            int run = block_prefix(sum, &tot);
#pragma unroll
                            for (int j = 0; j < PER; ++j) {
                                const int idx = tid * PER + j, d = idx / NW, w = idx - d * NW;
                                rwh[w * 128 + d] = (uint32_t)run;
                                run += loc[j];
                            }
                        }
                        __syncthreads();
                        for (int b0 = k0; b0 < k1; b0 += 32) {
                            const int u = b0 + lane;
                            const bool act = u < k1;
                            const uint32_t key = act ? src[u] : 0u;
                            const int d = (int)((key >> shift) & 127);
                            unsigned same = __ballot_sync(0xffffffffu, act);
#pragma unroll
                            for (int bit = 0; bit < 7; ++bit) {
                                const unsigned bb = __ballot_sync(0xffffffffu, act && ((d >> bit) & 1));
                                same &= ((d >> bit) & 1) ? bb : ~bb;
                            }
                            const int rank = __popc(same & lt);
                            if (act) dst[wh[d] + rank] = key;
                            __syncwarp();
                            if (act && rank == 0) wh[d] += __popc(same);
                            __syncwarp();
                        }
                        __syncthreads();
                        uint32_t *tmp = src;
                        src = dst;
                        dst = tmp;
                    }
                    XPROF_LAP(5);
                    // runs of one row, one sorted key per thread and round:
                    // the thread holding a run's first key sums the run
                    // exactly (runs are short: a range's rows rarely repeat)
                    // and writes it; output positions from a block prefix of
                    // the run heads, so consecutive threads write
                    // consecutive entries
                    for (int u0 = 0; u0 < prods; u0 += NT) {
                        const int u = u0 + tid;
                        const bool act = u < prods;
                        const uint32_t key = act ? src[u] : 0u;
                        const bool head = act && (u == 0 || (src[u - 1] >> 12) != (key >> 12));
                        int tot;
                        const int64_t q = out + block_prefix(head ? 1 : 0, &tot);
                        if (head) {
                            const uint32_t row = key >> 12;
                            uint64_t hi = 0, lo = 0;
                            uint32_t fl = 0;
                            for (int v = u; v < prods; ++v) {
                                const uint32_t kv = src[v];
                                if ((kv >> 12) != row) break;
                                if (!x_acc128(hi, lo, fl, __longlong_as_double((long long)rval[kv & 4095]), ebase))
                                    bad = true;
                            }
                            if (q < lim) {
                                cir[q] = (int64_t)rbase + (int64_t)row;
                                cval[q] = x_round(hi, lo, fl, ebase);
                            } else {
                                over = true;
                            }
                        }
                        out += tot;
                    }
                    __syncthreads();
                    XPROF_LAP(6);
                    t = t1 + 1;
                }
            }
        } else {
            // ------------------------- enumeration mode: per tile, all entries
            clean_words();
            int mwi = 0;
            uint64_t msk = a.tmask[i * a.mask_words];
            auto next_tile = [&]() -> int {
                while (msk == 0) {
                    if (++mwi >= a.mask_words) return -1;
                    msk = a.tmask[i * a.mask_words + mwi];
                }
                const int tt = mwi * 64 + __ffsll((long long)msk) - 1;
                msk &= msk - 1;
                return tt;
            };
            int t = next_tile();
            while (t >= 0) {
                const int tn = next_tile();
                const int row0 = t * a.R;
                int since_norm = 0;
                for (int64_t cb = bs; cb < be; cb += NT) {
                    const int nent = (int)min((int64_t)NT, be - cb);
                    if (since_norm + nent > kXNorm) {
                        __syncthreads();
                        for (int r = tid; r < a.R; r += NT)
                            if (tfb[r]) x_normalise(acc, RS, r);
                        since_norm = 0;
                    }
                    since_norm += nent;
                    const int64_t e = cb + tid;
                    uint32_t s0 = 0;
                    int len = 0;
                    if (e < be) {
                        const uint32_t *tp = a.tptr + (int64_t)a.brow[e] * (a.T + 1);
                        s0 = tp[t];
                        len = (int)(tp[t + 1] - s0);
                    }
                    int nseg;
                    const int L = compact_chunk<uint32_t, NT>(ch, s0, len, (uint32_t)(e - bs), ch_e, nseg);
                    dense_products(L, nseg, row0);
                }
                __syncthreads();
                dense_writeout(row0);
                XPROF_LAP(7);
                XPROF_ADD(10, 1);
                t = tn;
            }
        }
        over = __syncthreads_or(over);
        bad = __syncthreads_or(bad);
        XPROF_LAP(15);
        if (tid == 0) {
            if (out_cnt) out_cnt[g] = out - out0;
            if (over) {
                if (overflow)
                    overflow[g] = 1;
                else
                    atomicOr(a.err, 128);  // exact sizing: counts disagree
            }
            if (bad) atomicOr(a.err, 512);  // a product outside the admitted window
        }
    }
}

}  // namespace gbc
