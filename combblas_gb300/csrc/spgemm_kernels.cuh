// Shared pieces of the SpGEMM kernels: launch constants, the operand view,
// block-wide scans and the chunked walk over B-column entries.
#pragma once

#include <stdint.h>

#include "gbc_internal.cuh"

namespace gbc {

constexpr int kThreads = 256;            // threads per SpGEMM block
constexpr int kWarps = kThreads / 32;    // owner warps per block
constexpr int kBuckets = kWarps;         // one staging bucket per owner warp
constexpr int kStage = 2048;             // products staged per sub-batch
constexpr int kRounds = kStage / kThreads;
constexpr int kTileRows = 8192;          // default rows of the dense accumulator tile (two blocks per SM at fp64)
constexpr int kSymRows = 1 << 18;        // rows of one symbolic bitmap pass (32 KB: five blocks per SM)
constexpr int kMaxMaskWords = 64;        // tile-mask words per column (64 tiles each)

// Device view of the operands after preparation.  Rows of A are int32 and
// split into T tiles of R rows; tptr[k*(T+1)+t] is the first position in
// column k of A whose row is >= t*R, so A(tile t, k) is the contiguous range
// [tptr[k][t], tptr[k][t+1]).
struct SpgemmArgs {
    int64_t m, kdim, n, nb;
    int R, T, mask_words;
    const int64_t *acp;
    const int32_t *arow;
    const uint32_t *tptr;
    const int64_t *bcp;
    const int32_t *brow;
    const int64_t *flop;
    int32_t *err;
    int64_t col_begin, col_end;  // stored columns [col_begin, col_end) of B
    const void *aval, *bval;     // values of A and B (nullptr: all ones)
    const uint64_t *tmask;       // [nb][mask_words] row tiles each output column touches
    int64_t col_base;            // this product's first column in batch-wide per-column arrays
    int key_bits;                // bits needed for a row id
    const int32_t *aexp;         // fp64 A: per-column exponent range of the values (exact accumulation), or nullptr
    const int64_t *ktl_ptr;      // exact accumulation: per column of A, its touched row tiles (or nullptr)
    const uint32_t *ktl_start;   //   ... first position of the column inside each listed tile, then the column end
    const uint16_t *ktl_tile;    //   ... the tiles (0xFFFF: end marker)
};

// A work item names one output column of one product of a batch.
__host__ __device__ __forceinline__ int64_t make_item(int pid, int64_t col) { return ((int64_t)pid << 32) | col; }
__host__ __device__ __forceinline__ int item_pid(int64_t it) { return (int)(it >> 32); }
__host__ __device__ __forceinline__ int64_t item_col(int64_t it) { return it & 0xffffffffll; }

// Next work item of a persistent block: its own index first (consecutive
// blocks sit on different SMs, so the heaviest items, listed first, start
// on different SMs), then the items handed out by the counter.
__device__ __forceinline__ int64_t next_item(unsigned long long *work, bool &first)
{
    if (first) {
        first = false;
        return (int64_t)blockIdx.x;
    }
    return (int64_t)gridDim.x + (int64_t)atomicAdd(work, 1ull);
}

// Block-wide exclusive sum (NT threads); *total gets the block total.
template <int NT = kThreads>
__device__ __forceinline__ int64_t block_exclusive_sum64(int64_t v, int64_t *total)
{
    constexpr int NW = NT / 32;
    static_assert(NW <= 32, "one warp scans the warp totals");
    __shared__ int64_t ws[NW];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int64_t s = lane < NW ? ws[lane] : 0;
#pragma unroll
        for (int o = 1; o < NW; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < NW) ws[lane] = s;
    }
    __syncthreads();
    int64_t base = wid ? ws[wid - 1] : 0;
    if (total) *total = ws[NW - 1];
    __syncthreads();
    return base + x - v;
}

// One chunk of up to NT consecutive entries of a B column (NT = threads of
// the block), as its non-empty A segments restricted to row tiles [t0, t1):
// off[] is the exclusive prefix of the segment lengths (off[nseg] = total),
// and product p of segment b (off[b] <= p < off[b+1]) sits at position
// base[b] + p of A's arrays (base = segment start - off, modulo 2^32).
template <int NT>
struct ChunkSmemN {
    uint32_t base[NT];
    int32_t off[NT + 1];
};
typedef ChunkSmemN<kThreads> ChunkSmem;

// Compact one chunk whose segments are already known per thread (start s,
// length len, B value bv; len 0 for threads past the chunk), keeping only
// the non-empty segments: ch.base / ch.off (and ch_bv) hold the nseg
// non-empty segments in entry order, ch.off[nseg] = total.  One block scan packs the
// segment length (high word) with a non-empty flag (low word), giving
// offsets and compacted positions together.  Returns the total.
template <typename V, int NT>
__device__ __forceinline__ int compact_chunk(ChunkSmemN<NT> &ch, uint32_t s, int len, V bv, V *ch_bv, int &nseg)
{
    const int tid = threadIdx.x;
    int64_t tot;
    const int64_t ex = block_exclusive_sum64<NT>(((int64_t)len << 32) | (len > 0 ? 1 : 0), &tot);
    if (len > 0) {
        const int c = (int)(ex & 0xffffffff);
        ch.off[c] = (int)(ex >> 32);
        ch.base[c] = s - (uint32_t)(ex >> 32);
        if (ch_bv) ch_bv[c] = bv;
    }
    nseg = (int)(tot & 0xffffffff);
    if (tid == 0) ch.off[nseg] = (int)(tot >> 32);
    __syncthreads();
    return (int)(tot >> 32);
}

// Load one chunk of B entries [cb, min(cb + NT, be)) restricted to row tiles
// [t0, t1) and compact it (compact_chunk).
template <typename V, int NT>
__device__ __forceinline__ int load_chunk_nz(const SpgemmArgs &a, ChunkSmemN<NT> &ch, int64_t cb, int64_t be, int t0,
                                             int t1, const V *bval, V *ch_bv, V one, int &nseg)
{
    const int64_t b = cb + threadIdx.x;
    int len = 0;
    uint32_t s = 0;
    V bv = one;
    if (b < be) {
        const int k = a.brow[b];
        const uint32_t *tp = a.tptr + (int64_t)k * (a.T + 1);
        s = tp[t0];
        len = (int)(tp[t1] - s);
        if (ch_bv && bval) bv = bval[b];
    }
    return compact_chunk<V, NT>(ch, s, len, bv, ch_bv, nseg);
}

// Largest segment b < nseg with ch.off[b] <= p (warp-uniform p: broadcast reads).
template <int NT>
__device__ __forceinline__ int chunk_find_nz(const ChunkSmemN<NT> &ch, int nseg, int p)
{
    int lo = 0, hi = nseg;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (ch.off[mid] <= p)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// Segment of product p for a warp whose 32-product window [p - lane,
// p - lane + 32) starts inside segment bcur (segments non-empty, so at most
// 31 boundaries follow the window start within it): lane k holds the
// boundary ch.off[bcur+1+k]; a window that ends before the first boundary
// lies in bcur, otherwise a five-step binary search over the lanes counts
// the boundaries <= p.  All lanes of the warp must call it.
template <int NT>
__device__ __forceinline__ int window_seg(const ChunkSmemN<NT> &ch, int nseg, int bcur, int p)
{
    const int lane = threadIdx.x & 31;
    const int o = ch.off[min(bcur + 1 + lane, nseg)];
    if (__shfl_sync(0xffffffffu, o, 0) > p - lane + 31) return bcur;  // warp-uniform
    int c = 0;
#pragma unroll
    for (int step = 16; step; step >>= 1) {
        const int v = __shfl_sync(0xffffffffu, o, c + step - 1);
        if (v <= p) c += step;
    }
    return bcur + c;
}

inline size_t numeric_smem_bytes(int R, size_t vsize, int sub)
{
    // acc[R] + sval[sub] (values) + bitmap[R/32] + srow[sub] (u16) + tag[R] (u8)
    size_t b = (size_t)R * vsize + (size_t)sub * vsize;
    b += (size_t)(R / 32) * 4;
    b += (size_t)sub * 2 + (size_t)R;
    return (b + 15) & ~size_t(15);
}

int prepare_operands(Workspace &ws, const DevMatrix &A, const DevMatrix &B, SpgemmArgs &a, int64_t **acp_out,
                     int tile_rows = 0);

template <class SR>
int spgemm_learned(Context *ctx, const DevMatrix &A, const DevMatrix &B, const gbc_spgemm_opts &opt, int vt,
                   gbc_result **C, gbc_spgemm_stats *st);

}  // namespace gbc
