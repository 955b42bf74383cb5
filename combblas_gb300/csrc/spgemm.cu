// Local semiring SpGEMM C = A * B on one GB300, column-wise Gustavson over
// CSC/DCSC -- the computation of LocalHybridSpGEMM (mtSpGEMM.h:213-460):
// column j of C is the semiring sum over B(k,j) != 0 of A(:,k) * B(k,j).
//
// Kernels (exact two-phase sizing):
//   k_prep_a      A: int64 rows -> int32, dense column pointers for DCSC input,
//                 row-tile boundaries tptr[k][t] (tiles of R rows), validation
//                 (rows in range, strictly ascending within a column).
//   k_prep_b      B: int64 rows -> int32 (they index A's columns), validation.
//   k_flop        flop per stored column of B (estimateFLOP, mtSpGEMM.h:1057).
//   k_symbolic    exact nnz per column (estimateNNZ_Hash, mtSpGEMM.h:806):
//                 a shared-memory bitmap over the rows, plus the mask of row
//                 tiles the column touches.
//   k_numeric     per column, per touched row tile: products staged in
//                 shared memory, stably partitioned to owner warps (owner =
//                 a hash of the row), and folded by the owner into a dense
//                 shared-memory accumulator in B-entry order.  Each output
//                 entry is therefore the left fold acc = add(mrhs, acc) over
//                 k ascending -- exactly the order of the reference's hash
//                 path (mtSpGEMM.h:385-400) -- so repeated runs are
//                 bit-identical.  Rows come out ascending (tile order, then
//                 bitmap order).  Runs of sparse tiles of one column are
//                 folded the same way into a shared-memory hash table and
//                 sorted by row on write-out.
#include <algorithm>
#include <cstdio>
#include <functional>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include "gbc_internal.cuh"
#include "semiring.cuh"
#include "spgemm_kernels.cuh"
#include "spgemm_small.cuh"
#include "spgemm_exact.cuh"
#include "mlp.cuh"

namespace gbc {

// ----------------------------------------------------------------- prepare
// One warp per column of A.  tptr[k*(T+1)+t] = first position of column k
// whose row is >= t*R (t = 0..T); arow = rows as int32.
__global__ void k_prep_a(int64_t ncol, int64_t nrow, const int64_t *cp, const int64_t *jc, int64_t nzc,
                         int64_t nnz, const int64_t *ir, int32_t *arow, uint32_t *tptr, int T, int R, int32_t *err)
{
    int lane = threadIdx.x & 31;
    int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp; i < nzc; i += nwarps) {
        int64_t s = cp[i], e = cp[i + 1];
        int64_t c = jc ? jc[i] : i;
        if (e < s || (i == 0 && s != 0) || e > nnz) {
            if (lane == 0) atomicOr(err, 1);
            continue;
        }
        if (c < 0 || c >= ncol || (jc && i > 0 && jc[i - 1] >= c)) {
            if (lane == 0) atomicOr(err, 2);
            continue;
        }
        uint32_t *tp = tptr + c * (int64_t)(T + 1);
        int last_t = -1;
        for (int64_t b = s; b < e; b += 32) {
            int64_t p = b + lane;
            int t = -1;
            int64_t r = -1;
            if (p < e) {
                r = ir[p];
                if (r < 0 || r >= nrow) {
                    atomicOr(err, 4);
                    r = 0;
                }
                if (p > s && ir[p - 1] >= ir[p]) atomicOr(err, 8);
                arow[p] = (int32_t)r;
                t = (int)(r / R);
            }
            int tprev = __shfl_up_sync(0xffffffffu, t, 1);
            if (lane == 0) tprev = last_t;
            if (p < e) {
                for (int u = tprev + 1; u <= t; ++u) tp[u] = (uint32_t)p;
            }
            // the highest valid lane carries the last tile seen
            unsigned vm = __ballot_sync(0xffffffffu, p < e);
            int hi = 31 - __clz(vm);
            last_t = __shfl_sync(0xffffffffu, t, hi);
        }
        if (lane == 0) {
            for (int u = last_t + 1; u <= T; ++u) tp[u] = (uint32_t)e;
        }
    }
}

// Dense column pointers of a DCSC matrix (acp[c] = start of column c).
__global__ void k_dense_colptr(int64_t ncol, int64_t nzc, const int64_t *cp, const int64_t *jc, int64_t *acp)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i > nzc) return;
    // out-of-order or out-of-range ids are reported by k_prep_a; here they
    // only must not write outside acp[0..ncol]
    int64_t lo = i == 0 ? 0 : jc[i - 1] + 1;
    int64_t hi = i == nzc ? ncol : jc[i];
    lo = lo < 0 ? 0 : lo;
    hi = hi > ncol ? ncol : hi;
    for (int64_t c = lo; c <= hi; ++c) acp[c] = cp[i];
}

// Columns of A that hold no entries at all still need tile pointers.
__global__ void k_fill_empty_tptr(int64_t ncol, const int64_t *acp, uint32_t *tptr, int T)
{
    int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    if (acp[c] >= acp[c + 1]) {
        uint32_t v = (uint32_t)acp[c];
        for (int u = 0; u <= T; ++u) tptr[c * (int64_t)(T + 1) + u] = v;
    }
}

__global__ void k_prep_b(int64_t nzc, int64_t nnz, const int64_t *cp, const int64_t *ir, int64_t kdim,
                         int32_t *brow, int32_t *err)
{
    int lane = threadIdx.x & 31;
    int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp; i < nzc; i += nwarps) {
        int64_t s = cp[i], e = cp[i + 1];
        if (e < s || (i == 0 && s != 0) || e > nnz) {
            if (lane == 0) atomicOr(err, 16);
            continue;
        }
        for (int64_t p = s + lane; p < e; p += 32) {
            int64_t r = ir[p];
            if (r < 0 || r >= kdim) {
                atomicOr(err, 32);
                r = 0;
            }
            if (p > s && ir[p - 1] >= ir[p]) atomicOr(err, 64);
            brow[p] = (int32_t)r;
        }
    }
}

// Row-tile mask of every column of A: bit t set when A(tile t, k) is nonempty.
__global__ void k_amask(int64_t ncol, const uint32_t *tptr, int T, int mask_words, uint64_t *amask)
{
    const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const uint32_t *tp = tptr + c * (int64_t)(T + 1);
    for (int w = 0; w < mask_words; ++w) {
        uint64_t m = 0;
        for (int b = 0; b < 64 && w * 64 + b < T; ++b) {
            const int t = w * 64 + b;
            if (tp[t + 1] > tp[t]) m |= 1ull << b;
        }
        amask[c * mask_words + w] = m;
    }
}

// flop[i] = sum over B(:,i) entries k of nnz(A(:,k)) (estimateFLOP), and the
// column's tile mask = OR of the masks of those A columns (exactly the row
// tiles the output column touches).
__global__ void k_flop_mask(int64_t nb, const int64_t *bcp, const int32_t *brow, const int64_t *acp,
                            const uint64_t *amask, int mask_words, int64_t *flop, uint64_t *tmask)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp; i < nb; i += nwarps) {
        int64_t f = 0;
        for (int64_t p = bcp[i] + lane; p < bcp[i + 1]; p += 32) {
            const int k = brow[p];
            f += acp[k + 1] - acp[k];
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
        if (lane == 0) flop[i] = f;
        for (int w = 0; w < mask_words; ++w) {
            uint64_t m = 0;
            for (int64_t p = bcp[i] + lane; p < bcp[i + 1]; p += 32) m |= amask[(int64_t)brow[p] * mask_words + w];
#pragma unroll
            for (int o = 16; o; o >>= 1) m |= __shfl_xor_sync(0xffffffffu, m, o);
            if (lane == 0) tmask[i * mask_words + w] = m;
        }
    }
}

// Split stored columns j0..j1-1 of one product by their flop count: empty
// (count 0), small (up to s2 multiplications: warp kernels, in four sizes)
// and big (block kernels).  The thresholds are tuning parameters (s1 <=
// kSmall1, s2 <= kSmall2).  Lists are appended in any order; every column is
// written to its own output range, so the order does not affect the result.
constexpr int kSmall1 = 256;
constexpr int kSmall2 = 4096;
// Warp-kernel classes: at most s1, kSmallMid, kSmallMid2 and s2
// multiplications, each run by a kernel sized for its largest column (a
// smaller kernel keeps more warps resident: shared memory per warp is
// proportional to the products it holds).
constexpr int kSmallMid = 1024;
constexpr int kSmallMid2 = 2048;
constexpr int kWarpClasses = 4;
#ifndef GBC_SMALL2
#define GBC_SMALL2 kSmall2
#endif

// Big columns are binned by flop (> 2^23, > 2^21, > 2^19, the rest) and
// listed heaviest bin first, so the longest columns start early and do not
// run alone at the end of a launch (a scale-20 R-MAT hub column holds up to
// 2*10^7 products, most of one block's share of a phase).
constexpr int kBigBins = 4;
constexpr int kBigList = kWarpClasses;            // index of the big list in Lists
constexpr int kLists = kWarpClasses + kBigBins;  // list slots while classifying

__global__ void k_classify(const int64_t *flop, int pid, int64_t col_base, int64_t j0, int64_t j1, int64_t s1,
                           int64_t s2, int64_t *lbuf, int64_t stride, unsigned long long *counts, int64_t *cnt_zero,
                           const int32_t *only_flagged)
{
    const int64_t i = j0 + int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int cls = -1;
    if (i < j1 && (!only_flagged || only_flagged[col_base + i])) {
        const int64_t f = flop[i];
        if (f == 0) {
            if (cnt_zero) cnt_zero[col_base + i] = 0;
        } else if (f <= s1) {
            cls = 0;
        } else if (f <= s2) {
            cls = f <= kSmallMid ? 1 : f <= kSmallMid2 ? 2 : 3;
        } else {
            cls = kWarpClasses + (f > (1ll << 23) ? 0 : f > (1ll << 21) ? 1 : f > (1ll << 19) ? 2 : 3);
        }
    }
#pragma unroll
    for (int c = 0; c < kLists; ++c) {
        const unsigned m = __ballot_sync(0xffffffffu, cls == c);
        if (!m) continue;
        const int leader = __ffs(m) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(&counts[c], (unsigned long long)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        int64_t *list = lbuf + c * stride;
        if (cls == c) list[base + __popc(m & ((1u << lane) - 1))] = make_item(pid, i);
    }
}

// ---------------------------------------------------------------- symbolic
// One block per listed column (dynamic work counter).  Bitmap over a
// super-tile of sup_rows rows (a whole number of R-row tiles); products set
// bits; the column's count is the popcount.
__global__ void __launch_bounds__(kThreads) k_symbolic(const SpgemmArgs *args, const int64_t *items,
                                                       int64_t nitems, int64_t *cnt, unsigned long long *work)
{
    extern __shared__ uint32_t bm[];
    __shared__ ChunkSmem ch;
    __shared__ int64_t s_col;
    __shared__ int64_t s_red[kThreads / 32];
    __shared__ SpgemmArgs sa;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    bool first_item = true;
    for (;;) {
        if (tid == 0) {
            s_col = next_item(work, first_item);
            if (s_col < nitems) sa = args[item_pid(items[s_col])];
        }
        __syncthreads();
        const int64_t ci = s_col;
        __syncthreads();
        if (ci >= nitems) break;
        const SpgemmArgs &a = sa;
        const int64_t i = item_col(items[ci]);
        const int sup_rows = (int)((min((int64_t)kSymRows, (int64_t)a.T * a.R) / a.R) * a.R);
        const int tiles_per_sup = sup_rows / a.R;
        int64_t bs = a.bcp[i], be = a.bcp[i + 1];
        int64_t total = 0;
        if (a.flop[i] > 0) {
            for (int t0 = 0; t0 < a.T; t0 += tiles_per_sup) {
                int t1 = min(a.T, t0 + tiles_per_sup);
                int64_t row0 = int64_t(t0) * a.R;
                int rows = (int)((a.m - row0) < (int64_t)sup_rows ? (a.m - row0) : (int64_t)sup_rows);
                int words = (rows + 31) >> 5;
                for (int w = tid; w < words; w += kThreads) bm[w] = 0;
                __syncthreads();
                for (int64_t cb = bs; cb < be; cb += kThreads) {
                    int nseg;
                    const int L = load_chunk_nz<int>(a, ch, cb, be, t0, t1, nullptr, nullptr, 0, nseg);
                    // warp w takes a contiguous span of products in 32-product windows
                    const int span = ((L + kThreads - 1) / kThreads) * 32;
                    const int wb = warp * span, we = min(L, wb + span);
                    if (wb < we) {
                        int bcur = chunk_find_nz(ch, nseg, wb);
                        for (int P = wb; P < we; P += 32) {
                            const int p = P + lane;
                            const int b = window_seg(ch, nseg, bcur, p);
                            if (p < we) {
                                const int64_t idx = (uint32_t)(ch.base[b] + (uint32_t)p);
                                const int r = a.arow[idx] - (int)row0;
                                atomicOr(&bm[r >> 5], 1u << (r & 31));
                            }
                            int bn = __shfl_sync(0xffffffffu, b, 31);
                            if (bn + 1 < nseg && ch.off[bn + 1] <= P + 32) ++bn;
                            bcur = bn;
                        }
                    }
                    __syncthreads();
                }
                int64_t c = 0;
                for (int w = tid; w < words; w += kThreads) c += __popc(bm[w]);
                total += c;
                __syncthreads();
            }
        }
        // block reduce of total
        int64_t v = total;
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) s_red[tid >> 5] = v;
        __syncthreads();
        if (tid == 0) {
            int64_t s = 0;
            for (int w = 0; w < kThreads / 32; ++w) s += s_red[w];
            cnt[a.col_base + i] = s;
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------- numeric
// One block per column (dynamic counter); for every row tile t the column
// touches:
//  * dense accumulator acc[R] and touched bitmap in shared memory;
//  * the column's B entries are walked in chunks of kThreads; the chunk's A
//    segments restricted to tile t form a flattened product list, processed
//    in sub-batches of SUB products (only the rounds of kThreads products
//    that hold any are executed).  Empty segments are dropped when the
//    chunk is loaded; the first segment of every 32-product window comes
//    from a binary search (one thread per window), the segments of its
//    lanes from a five-step search over the next 32 boundaries held in
//    registers (window_seg);
//  * staging: all threads load the sub-batch's rows and values with
//    coalesced reads (one load per product, k-major order) and multiply by
//    B(k,j); a stable partition by owner warp (row_owner: a hash of the
//    row), ranked with three ballots and one block scan of the group sizes,
//    writes each product into its owner's bucket in shared memory, keeping
//    k order inside every bucket;
//  * folding: each warp walks its bucket in 32-product windows.  Equal rows
//    in a window are grouped (row tag winner + shared-memory group masks) and
//    the lowest lane folds the group in lane order.  Each output entry is thus the left fold
//    acc = add(mrhs, acc) over k ascending, with no atomics on values.
// Owner warp of tile row o: the top bits of a multiplicative hash.  Every
// bit of an R-MAT row id is skewed (set with probability c + d), so any
// owner taken from a few row bits gets a fixed share far above 1/kWarps;
// the hash spreads rows evenly and leaves only single hot rows.
template <int LB>
__device__ __forceinline__ int row_owner(int o) { return (int)(((uint32_t)o * 0x9E3779B1u) >> (32 - LB)); }

// NT threads per block (256 or 512), SUB products per sub-batch.
template <int NT, int SUB>
constexpr int numeric_min_blocks() { return NT == 512 ? 2 : SUB <= 1024 ? 4 : SUB <= 2048 ? 2 : 1; }

template <class SR, int SUB, int NT>
__global__ void __launch_bounds__(NT, numeric_min_blocks<NT, SUB>()) k_numeric(const SpgemmArgs *args, const int64_t *items, int64_t nitems,
                                                         const int64_t *ccp, int64_t ccp_base, const int64_t *cap,
                                                         int64_t *out_cnt, int32_t *overflow, int64_t *cir,
                                                         void *cval_v, unsigned long long *work,
                                                         const unsigned long long *dyn_n)
{
    // a device-side item count (columns handed over by another kernel)
    if (dyn_n) nitems = min(nitems, (int64_t)*dyn_n);
    typedef typename SR::V V;
    constexpr int kSub = SUB;
    constexpr int NW = NT / 32;                      // warps = owners
    constexpr int LB = NW == 16 ? 4 : 3;             // owner bits
    static_assert(NW == (1 << LB), "8 or 16 warps");
    constexpr int kSubPerThread = SUB / NT;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ ChunkSmemN<NT> ch;
    __shared__ V ch_bv[NT];
    __shared__ int32_t s_cnt[NW * kSubPerThread * NW + 1];  // [owner][round][warp]
    __shared__ int32_t s_wsum[NW];
    __shared__ int32_t s_win[SUB / 32];
    __shared__ uint32_t s_grp[NT];  // per warp: group mask of each winner lane
    __shared__ int32_t s_hist[256];  // range visits: products per row tile
    __shared__ int64_t s_col;
    __shared__ SpgemmArgs sa;
    V *cval = static_cast<V *>(cval_v);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1;
    constexpr int NC = NW * kSubPerThread * NW;
    // Range visits (see below): a hash table of HS slots in the accumulator
    // area, keys shifted by 13 bits in the sort.
    constexpr int HS = 2 * SUB;
    constexpr int HSB = SUB == 1024 ? 11 : SUB == 2048 ? 12 : 13;
    static_assert((1 << HSB) == HS && HS <= 8192, "hash slots");
    constexpr bool kRanges = sizeof(V) == 8;

    bool first_item = true;
    for (;;) {
        if (tid == 0) {
            s_col = next_item(work, first_item);
            if (s_col < nitems) sa = args[item_pid(items[s_col])];
        }
        __syncthreads();
        const int64_t ci = s_col;
        __syncthreads();
        if (ci >= nitems) break;
        const SpgemmArgs &a = sa;
        const int64_t i = item_col(items[ci]);
        const int64_t g = a.col_base + i;
        V *acc = reinterpret_cast<V *>(smem);                            // [R]
        V *sval = acc + a.R;                                             // [kSub] owner buckets
        uint32_t *bm = reinterpret_cast<uint32_t *>(sval + kSub);        // [R/32]
        uint16_t *srow = reinterpret_cast<uint16_t *>(bm + (a.R >> 5));  // [kSub]
        uint8_t *tag = reinterpret_cast<uint8_t *>(srow + kSub);         // [R] window row tags
        const V *aval = static_cast<const V *>(a.aval);
        const V *bval = static_cast<const V *>(a.bval);
        const int words = a.R >> 5;
        const int64_t bs = a.bcp[i], be = a.bcp[i + 1];
        // ccp is indexed by batch-wide column relative to ccp_base
        const int64_t out0 = ccp[g - ccp_base];
        int64_t out = out0;
        const int64_t lim = cap ? out0 + cap[g] : ccp[g - ccp_base + 1];
        bool over = false;
        // the touched bitmap starts clear (its place depends on this
        // product's R); every tile's write-out clears it again.  The barriers
        // of the first chunk load order this before any fold.
        for (int w = tid; w < words; w += NT) bm[w] = 0;
        // Touched row tiles in order; next_tile() gives the next one, or -1.
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
        // A column of at most NT entries is one chunk: thread tid keeps its
        // entry's A column in bk, and the segment bounds of the next touched
        // tile are loaded one tile ahead (ps, pe), so the chunk of a tile
        // waits on no dependent global loads.
        const bool single = be - bs <= NT;
        int bk = -1;
        uint32_t ps = 0, pe = 0;
        int t = next_tile();
        if (single && tid < be - bs) {
            bk = a.brow[bs + tid];
            if (t >= 0) {
                const uint32_t *tp = a.tptr + (int64_t)bk * (a.T + 1);
                ps = tp[t];
                pe = tp[t + 1];
            }
        }
        // Range visits.  A sparse column visits most of its row tiles with a
        // few hundred products each, and a tile visit costs about the same
        // whatever its size.  So a single-chunk column of at most 2^18
        // products first counts its products per tile (hist), and a run of
        // consecutive touched tiles holding at most SUB products together is
        // visited once: its products are folded (same owner partition and
        // ordered fold) into a hash table of HS slots keyed by the row and
        // held in the accumulator area (hval, hkey, plus hrow, the rows of the
        // staged products), then the occupied slots are sorted by row
        // (bitonic, in the staging area) and written in row order.  Tiles with
        // more products keep the dense visit.
        const bool ranges = kRanges && single && a.T > 1 && a.T <= 256 && a.R >= HS &&
                            (size_t)HS * (sizeof(V) + 4) + (size_t)SUB * 4 <= (size_t)a.R * sizeof(V) &&
                            a.flop[i] <= (1 << 18);
        V *hval = acc;                                                 // [HS]
        int32_t *hkey = reinterpret_cast<int32_t *>(acc + HS);         // [HS] row, -1 empty
        int32_t *hrow = hkey + HS;                                     // [SUB]
        uint64_t *skey = reinterpret_cast<uint64_t *>(sval);           // [SUB] sort keys
        int32_t *hist = s_hist;                                        // [T]
        if (ranges) {
            for (int tt = tid; tt < a.T; tt += NT) hist[tt] = 0;
            ch.base[tid] = (uint32_t)bk;  // the column's A columns, for all threads
            __syncthreads();
            const int nb = (int)(be - bs), npairs = nb * a.T;
            for (int p0 = tid; p0 < npairs; p0 += 4 * NT) {
                int len[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int pp = p0 + u * NT;
                    len[u] = 0;
                    if (pp < npairs) {
                        const int e = pp / a.T, tt = pp - e * a.T;
                        const uint32_t *tp = a.tptr + (int64_t)(int)ch.base[e] * (a.T + 1);
                        len[u] = (int)(tp[tt + 1] - tp[tt]);
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (len[u] > 0) atomicAdd(&hist[(p0 + u * NT) % a.T], len[u]);
            }
            __syncthreads();
        }
        while (t >= 0) {
            int tn = next_tile();
            int tlast = t;
            if (ranges && hist[t] <= SUB) {
                int rsum = hist[t];
                while (tn >= 0 && hist[tn] <= SUB - rsum) {
                    rsum += hist[tn];
                    tlast = tn;
                    tn = next_tile();
                }
            }
            const bool hashed = tlast > t;  // block-uniform
            if (hashed)
                for (int u = tid; u < HS; u += NT) hkey[u] = -1;
            const int row0 = t * a.R;
            for (int64_t cb = bs; cb < be; cb += NT) {
                int nseg, L;
                if (single) {
                    const uint32_t s0 = ps;
                    uint32_t e0 = pe;
                    if (hashed && bk >= 0) e0 = a.tptr[(int64_t)bk * (a.T + 1) + tlast + 1];
                    const int len0 = bk >= 0 ? (int)(e0 - s0) : 0;
                    const V bv = (bk >= 0 && bval) ? bval[bs + tid] : SR::one();
                    if (bk >= 0 && tn >= 0) {
                        const uint32_t *tp = a.tptr + (int64_t)bk * (a.T + 1);
                        ps = tp[tn];
                        pe = tp[tn + 1];
                    }
                    L = compact_chunk<V, NT>(ch, s0, len0, bv, ch_bv, nseg);
                    if (hashed && L > kSub) {  // cannot happen: the run was cut at SUB products
                        if (tid == 0) atomicOr(a.err, 256);
                        L = 0;
                    }
                } else {
                    L = load_chunk_nz<V>(a, ch, cb, be, t, t + 1, bval, ch_bv, SR::one(), nseg);
                }
                // Sub-batches are software pipelined: the global loads of
                // sub-batch q + kSub are issued right after sub-batch q is
                // scattered, so their latency overlaps q's fold.
                // Raw loads of a sub-batch, kept unconsumed until its
                // partition: row (-1: no product), A value, segment.
                int ar_[kSubPerThread];
                V av_[kSubPerThread];
                int sg_[kSubPerThread];
                // 1. first segment of every 32-product window of a sub-batch:
                //    one binary search per window, in parallel
                // 2. load: round r covers products [r*NT, (r+1)*NT) of the
                //    sub-batch, warp w its window at r*NT + 32w
                //    (coalesced; the unrolled rounds keep all loads in flight);
                //    the lanes' segments come from window_seg.  Nothing reads
                //    the loaded registers here, so the loads stay in flight
                //    through the fold that follows; the product with B(k,j)
                //    is formed at the scatter
                auto load_sub = [&](int q0) {
                    const int n0 = min(kSub, L - q0);
                    const int rounds0 = (n0 + NT - 1) / NT;
#pragma unroll
                    for (int r = 0; r < kSubPerThread; ++r) {
                        ar_[r] = -1;
                        const int P = q0 + r * NT + warp * 32;
                        if (r < rounds0 && P < q0 + n0) {  // warp-uniform
                            const int p = P + lane;
                            const int b = window_seg(ch, nseg, s_win[r * NW + warp], p);
                            if (p < q0 + n0) {
                                const int64_t idx = (uint32_t)(ch.base[b] + (uint32_t)p);
                                ar_[r] = a.arow[idx];
                                av_[r] = aval ? aval[idx] : SR::one();
                                sg_[r] = b;
                            }
                        }
                    }
                };
                if (L > 0) {
                    if (tid < (min(kSub, L) + 31) >> 5) s_win[tid] = chunk_find_nz(ch, nseg, tid * 32);
                    __syncthreads();
                    load_sub(0);
                }
                for (int q = 0; q < L; q += kSub) {
                    const int n = min(kSub, L - q);
                    const int rounds = (n + NT - 1) / NT;  // block-uniform
                    // 3. stable partition by owner warp (row_owner): rank
                    //    within (round, warp) from LB + 1 ballots; counts laid out
                    //    [owner][round][warp] so the scan follows product order
                    int rk_[kSubPerThread];
#pragma unroll
                    for (int r = 0; r < kSubPerThread; ++r) {
                        if (r < rounds) {
                            const bool act = ar_[r] >= 0;
                            const int w = row_owner<LB>(ar_[r] - row0);
                            const unsigned va = __ballot_sync(0xffffffffu, act);
                            unsigned bb[LB];
#pragma unroll
                            for (int i = 0; i < LB; ++i) bb[i] = __ballot_sync(0xffffffffu, act && ((w >> i) & 1));
                            unsigned same = va;
#pragma unroll
                            for (int i = 0; i < LB; ++i) same &= ((w >> i) & 1) ? bb[i] : ~bb[i];
                            rk_[r] = __popc(same & lt);
                            // lanes 0..NW-1 publish the size of owner `lane`'s group
                            if (lane < NW) {
                                unsigned sl = va;
#pragma unroll
                                for (int i = 0; i < LB; ++i) sl &= ((lane >> i) & 1) ? bb[i] : ~bb[i];
                                s_cnt[(lane * kSubPerThread + r) * NW + warp] = __popc(sl);
                            }
                        } else if (lane < NW) {
                            s_cnt[(lane * kSubPerThread + r) * NW + warp] = 0;
                        }
                    }
                    __syncthreads();
                    // 4. exclusive scan of the (owner, round, warp) counts: PER
                    //    consecutive counts per thread, warp scan, one barrier for
                    //    the warp totals
                    {
                        constexpr int PER = NC / NT;
                        static_assert(PER * NT == NC, "counts split evenly over the threads");
                        int loc[PER];
                        int sum = 0;
#pragma unroll
                        for (int u = 0; u < PER; ++u) {
                            loc[u] = s_cnt[tid * PER + u];
                            sum += loc[u];
                        }
                        int x = sum;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const int y = __shfl_up_sync(0xffffffffu, x, o);
                            if (lane >= o) x += y;
                        }
                        if (lane == 31) s_wsum[warp] = x;
                        __syncthreads();
                        int base = x - sum, tot = 0;
#pragma unroll
                        for (int u = 0; u < NW; ++u) {
                            const int ws = s_wsum[u];
                            base += u < warp ? ws : 0;
                            tot += ws;
                        }
#pragma unroll
                        for (int u = 0; u < PER; ++u) {
                            s_cnt[tid * PER + u] = base;
                            base += loc[u];
                        }
                        if (tid == 0) s_cnt[NC] = tot;
                    }
                    __syncthreads();
                    // 5. scatter into owner buckets
#pragma unroll
                    for (int r = 0; r < kSubPerThread; ++r) {
                        if (r < rounds && ar_[r] >= 0) {
                            const int o = ar_[r] - row0;
                            const int w = row_owner<LB>(o);
                            const int pos = s_cnt[(w * kSubPerThread + r) * NW + warp] + rk_[r];
                            if (hashed)
                                hrow[pos] = o;
                            else
                                srow[pos] = (uint16_t)o;
                            sval[pos] = SR::mul(av_[r], ch_bv[sg_[r]]);
                        }
                    }
                    // windows of the next sub-batch (s_win was last read by its
                    // own loads, issued before this sub-batch's barriers)
                    const int qn = q + kSub;
                    if (qn < L && tid < (min(kSub, L - qn) + 31) >> 5)
                        s_win[tid] = chunk_find_nz(ch, nseg, qn + tid * 32);
                    __syncthreads();
                    if (qn < L) load_sub(qn);  // the registers of q were consumed by the scatter
                    // 6. each warp folds its bucket in staging (= k) order.  Every
                    //    lane stores its id at its row's tag and reads back the
                    //    row's winner; a window whose rows are distinct folds
                    //    lane-parallel.  Otherwise each lane ORs its bit into the
                    //    winner's group mask (shared memory, one word per lane),
                    //    and the lowest lane of each group folds it in lane
                    //    order.  (The atomic group masks cost far less than
                    //    __match_any_sync, whose throughput falls to about one per
                    //    64 SM cycles on windows of distinct rows.)
                    {
                        const int beg = s_cnt[warp * NW * kSubPerThread];
                        const int end = s_cnt[(warp + 1) * NW * kSubPerThread];
                        uint32_t *gm = s_grp + warp * 32;
                        for (int p0 = beg; p0 < end; p0 += 32) {
                            const int p = p0 + lane;
                            const bool act = p < end;
                            int o = 0;  // accumulator index: the tile row, or the row's hash slot
                            if (act && !hashed) {
                                o = srow[p];
                            } else if (act) {
                                // linear probing; the table holds at most SUB rows of HS slots
                                const int row = hrow[p];
                                int h = (int)(((uint32_t)row * 0x85EBCA6Bu) >> (32 - HSB));
                                for (;;) {
                                    const int k = ((volatile int32_t *)hkey)[h];
                                    if (k == row) break;
                                    if (k < 0) {
                                        const int old = atomicCAS(&hkey[h], -1, row);
                                        if (old < 0 || old == row) break;
                                    }
                                    h = (h + 1) & (HS - 1);
                                }
                                o = h;
                            }
                            if (act) tag[o] = (uint8_t)lane;
                            gm[lane] = 0;
                            __syncwarp();
                            const int wl = act ? (int)tag[o] : lane;
                            unsigned grp = 1u << lane;
                            if (__ballot_sync(0xffffffffu, wl != lane)) {
                                if (act) atomicOr(&gm[wl], 1u << lane);
                                __syncwarp();
                                if (act) grp = gm[wl];
                            }
                            if (act && (grp & lt) == 0) {
                                const uint32_t bit = 1u << (o & 31);
                                const bool touched = (bm[o >> 5] & bit) != 0;
                                V *ap = acc + o;
                                V cur = touched ? SR::add(sval[p], *ap) : sval[p];
                                unsigned rest = grp & ~(1u << lane);
                                while (rest) {
                                    const int m = __ffs(rest) - 1;
                                    rest &= rest - 1;
                                    cur = SR::add(sval[p0 + m], cur);
                                }
                                *ap = cur;
                                if (!touched) atomicOr(&bm[o >> 5], bit);
                            }
                            __syncwarp();
                        }
                    }
                    __syncthreads();
                }
            }
            if (hashed) {
                // range visit: the occupied slots, as (row << 13 | slot) keys,
                // are sorted (bitonic, in the staging area: at most SUB of
                // them) and written in row order; the slot bits are cleared
                constexpr int SPT = HS / NT;
                int c = 0;
#pragma unroll
                for (int u = 0; u < SPT; ++u) c += hkey[tid * SPT + u] >= 0;
                int x = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane == 31) s_wsum[warp] = x;
                __syncthreads();
                int q = x - c, tot = 0;
#pragma unroll
                for (int u = 0; u < NW; ++u) {
                    const int ws = s_wsum[u];
                    q += u < warp ? ws : 0;
                    tot += ws;
                }
#pragma unroll
                for (int u = 0; u < SPT; ++u) {
                    const int sl = tid * SPT + u;
                    const int k = hkey[sl];
                    if (k >= 0) skey[q++] = ((uint64_t)(uint32_t)k << 13) | (uint64_t)sl;
                }
                int N = 1;
                while (N < tot) N <<= 1;
                for (int u = tot + tid; u < N; u += NT) skey[u] = ~0ull;
                __syncthreads();
                for (int k2 = 2; k2 <= N; k2 <<= 1) {
                    for (int j = k2 >> 1; j > 0; j >>= 1) {
                        for (int u = tid; u < (N >> 1); u += NT) {
                            const int lo = ((u & ~(j - 1)) << 1) | (u & (j - 1)), hi = lo + j;
                            const uint64_t x0 = skey[lo], x1 = skey[hi];
                            if ((x0 > x1) == ((lo & k2) == 0)) {
                                skey[lo] = x1;
                                skey[hi] = x0;
                            }
                        }
                        __syncthreads();
                    }
                }
                for (int u = tid; u < tot; u += NT) {
                    const uint64_t key = skey[u];
                    const int64_t pos = out + u;
                    if (pos < lim) {
                        cir[pos] = (int64_t)row0 + (int64_t)(key >> 13);
                        cval[pos] = hval[key & (HS - 1)];
                    } else {
                        over = true;
                    }
                }
                for (int w = tid; w < (HS >> 5); w += NT) bm[w] = 0;
                out += tot;
            } else
            // write the tile's entries in row order: each thread takes its
            // words of the touched bitmap (clearing them for the next
            // tile), entries are staged in row order in shared memory and
            // stored by consecutive threads
            {
                int wl = 0;
                const int wpt = (words + NT - 1) / NT;
                const int w0 = min(words, tid * wpt), w1 = min(words, (tid + 1) * wpt);
                for (int w = w0; w < w1; ++w) wl += __popc(bm[w]);
                int x = wl;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane == 31) s_wsum[warp] = x;
                __syncthreads();
                int before = 0, tot = 0;
#pragma unroll
                for (int u = 0; u < NW; ++u) {
                    const int ws = s_wsum[u];
                    before += u < warp ? ws : 0;
                    tot += ws;
                }
                if (tot <= kSub) {
                    // stage the tile's entries in row order in shared memory,
                    // then store them with consecutive threads on
                    // consecutive positions
                    int q = before + x - wl;
                    for (int w = w0; w < w1; ++w) {
                        uint32_t bits = bm[w];
                        bm[w] = 0;  // clear for the next tile
                        while (bits) {
                            const int o = w * 32 + __ffs(bits) - 1;
                            bits &= bits - 1;
                            srow[q] = (uint16_t)o;
                            sval[q] = acc[o];
                            ++q;
                        }
                    }
                    __syncthreads();
                    for (int p = tid; p < tot; p += NT) {
                        const int64_t pos = out + p;
                        if (pos < lim) {
                            cir[pos] = (int64_t)row0 + srow[p];
                            cval[pos] = sval[p];
                        } else {
                            over = true;  // never write past the column's range
                        }
                    }
                } else {
                    int64_t pos = out + before + x - wl;
                    for (int w = w0; w < w1; ++w) {
                        uint32_t bits = bm[w];
                        bm[w] = 0;  // clear for the next tile
                        while (bits) {
                            const int o = w * 32 + __ffs(bits) - 1;
                            bits &= bits - 1;
                            if (pos < lim) {
                                cir[pos] = (int64_t)row0 + o;
                                cval[pos] = acc[o];
                            } else {
                                over = true;
                            }
                            ++pos;
                        }
                    }
                }
                out += tot;
            }
            __syncthreads();
            t = tn;
        }
        over = __syncthreads_or(over);
        if (tid == 0) {
            if (out_cnt) out_cnt[g] = out - out0;
            if (over) {
                if (overflow)
                    overflow[g] = 1;
                else
                    atomicOr(a.err, 128);  // exact sizing: counts disagree
            }
        }
    }
}

// Columns of B with a nonzero output, for the SpDCCols view of C.
__global__ void k_nonempty_flags(int64_t n, const int64_t *cnt, int64_t *flags)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = cnt[i] > 0;
}

__global__ void k_compact_cols(int64_t n, const int64_t *cnt, const int64_t *pos, const int64_t *ccp_full,
                               const int64_t *bjc, int64_t *cp, int64_t *jc)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && cnt[i] > 0) {
        cp[pos[i]] = ccp_full[i];
        jc[pos[i]] = bjc ? bjc[i] : i;
    }
    if (i == n - 1) cp[pos[n]] = ccp_full[n];
}

__global__ void k_iota_jc(int64_t n, const int64_t *bjc, int64_t *jc)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) jc[i] = bjc ? bjc[i] : i;
}

// ------------------------------------------------------------------ driver
static int grid_for(Context *c, int64_t work, int per_sm)
{
    int64_t g = (int64_t)c->num_sms * per_sm;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, work));
}

// Blocks of `kernel` that fit on one SM at once (registers, shared memory,
// threads), at most cap.  Persistent kernels launch exactly this many per
// SM: every block then starts at once and takes its first item (the
// heaviest first) without waiting for another block to exit.  Memoized per
// device, kernel, block size and shared memory, so a stream capture that
// repeats an earlier launch makes no query.
template <class K>
static int resident_blocks(K kernel, int threads, size_t dyn_smem, int cap)
{
    static std::mutex mu;
    static std::map<std::tuple<int, const void *, int, size_t>, int> known;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_tuple(dev, (const void *)kernel, threads, dyn_smem);
    auto it = known.find(key);
    if (it == known.end()) {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, dyn_smem) != cudaSuccess || n < 1) {
            cudaGetLastError();
            n = 1;
        }
        it = known.emplace(key, n).first;
    }
    return std::min(it->second, cap);
}

// Raise a kernel's dynamic shared-memory limit once (per device and kernel,
// only upwards), so replays and graph captures make no attribute calls.
template <class K>
static int set_smem(K kernel, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> done;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    size_t &cur = done[{dev, (const void *)kernel}];
    if (cur >= bytes) return GBC_OK;
    GBC_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
    return GBC_OK;
}

int prepare_operands(Workspace &ws, const DevMatrix &A, const DevMatrix &B, SpgemmArgs &a, int64_t **acp_out,
                     int tile_rows)
{
    Context *ctx = ws.ctx;
    cudaStream_t s = ctx->stream;
    a.m = A.nrow;
    a.kdim = A.ncol;
    a.n = B.ncol;
    a.nb = B.nzc;
    // default tile: 4096 rows (four blocks per SM) up to 2^18 rows, else
    // 8192 (two blocks per SM, half the tile passes per column)
    const int rows = (tile_rows == 4096 || tile_rows == 8192 || tile_rows == 16384) ? tile_rows
                     : (A.nrow <= (int64_t(1) << 18))                             ? 4096
                                                                                   : kTileRows;
    a.R = (int)std::min<int64_t>(rows, ((A.nrow + kThreads - 1) / kThreads) * kThreads);
    if (a.R < kThreads) a.R = kThreads;
    a.T = (int)((A.nrow + a.R - 1) / a.R);
    if (a.T < 1) a.T = 1;
    a.mask_words = (a.T + 63) / 64;
    if (a.mask_words > kMaxMaskWords) return fail(GBC_EOVERFLOW, "too many rows for the tile mask");
    if (A.nnz >= (int64_t(1) << 32)) return fail(GBC_EOVERFLOW, "nnz(A) must be below 2^32");
    int32_t *err = nullptr;
    GBC_TRY(ws.alloc_n(&err, 4));
    GBC_CUDA_TRY(cudaMemsetAsync(err, 0, 4 * sizeof(int32_t), s));
    int32_t *arow = nullptr;
    int64_t *acp = nullptr;
    uint32_t *tptr = nullptr;
    GBC_TRY(ws.alloc_n(&arow, A.nnz + 1));
    GBC_TRY(ws.alloc_n(&tptr, (size_t)A.ncol * (a.T + 1) + 1));
    if (A.jc) {
        GBC_TRY(ws.alloc_n(&acp, A.ncol + 1));
        k_dense_colptr<<<(unsigned)((A.nzc + 1 + 255) / 256), 256, 0, s>>>(A.ncol, A.nzc, A.cp, A.jc, acp);
        note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    } else {
        acp = const_cast<int64_t *>(A.cp);
    }
    if (A.nzc > 0) {
        k_prep_a<<<grid_for(ctx, (A.nzc + 7) / 8, 8), 256, 0, s>>>(A.ncol, A.nrow, A.cp, A.jc, A.nzc, A.nnz,
                                                                     A.ir, arow, tptr, a.T, a.R, err);
        note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    if (A.ncol > 0) {
        k_fill_empty_tptr<<<(unsigned)((A.ncol + 255) / 256), 256, 0, s>>>(A.ncol, acp, tptr, a.T);
        note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    int32_t *brow = nullptr;
    GBC_TRY(ws.alloc_n(&brow, B.nnz + 1));
    if (B.nzc > 0) {
        k_prep_b<<<grid_for(ctx, (B.nzc + 7) / 8, 8), 256, 0, s>>>(B.nzc, B.nnz, B.cp, B.ir, A.ncol, brow, err);
        note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    int32_t herr[4];
    GBC_CUDA_TRY(cudaMemcpyAsync(herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr[0]) {
        char buf[160];
        snprintf(buf, sizeof buf, "malformed input matrix (code 0x%x): %s%s%s", herr[0],
                 (herr[0] & 0x13) ? "bad column pointers or ids; " : "",
                 (herr[0] & 0x24) ? "row id out of range; " : "",
                 (herr[0] & 0x48) ? "rows not strictly ascending within a column" : "");
        return fail(GBC_EINVAL, buf);
    }
    a.err = err;
    a.acp = acp;
    a.arow = arow;
    a.tptr = tptr;
    a.bcp = B.cp;
    a.brow = brow;
    a.col_begin = 0;
    a.col_end = B.nzc;
    *acp_out = acp;
    return GBC_OK;
}

// Everything the passes need, built once: one descriptor per product of a
// batch (a single product is a batch of one).
struct Plan {
    std::vector<SpgemmArgs> h;        // host copies of the descriptors
    SpgemmArgs *d = nullptr;          // device array
    int64_t total_cols = 0;           // stored columns of all B's
    int max_R = 0, max_key_bits = 0;
    size_t max_sym_smem = 0;
    int64_t s1 = kSmall1, s2 = GBC_SMALL2;  // flop thresholds of the column classes
    int tile_rows = 0;                   // accumulator tile height (0: default)
    unsigned long long *work = nullptr;  // kernel work counters
    int64_t *lbuf = nullptr;             // column lists (kLists x (total_cols + 1))
    bool s2_set = false;                 // the caller chose s2
    unsigned long long *lcnt = nullptr;  // list lengths
    bool want_aexp = false;              // PlusTimes fp64, exact accumulation (k_numeric_x)
    int64_t *fb_items = nullptr;         // big columns the exact kernel hands to the ordered one
    unsigned long long *fb_cnt = nullptr;
    XSeg *xscratch = nullptr;            // exact kernel: bucketing scratch, kXScap segments per block
    int x_blocks = 0;                    // exact kernel: its grid (resident blocks)
    SpgemmArgs &a() { return h[0]; }
};

// PlusTimes fp64 under GBC_FOLD_EXACT: every admitted column is summed
// exactly (big columns by k_numeric_x).  Its accumulator tile is kXRows
// high by default (8192-row tiles, one 1024-thread block per SM, made the
// scale-20 product 19 % slower) and kXRowsBig at most; the tile height is a
// tuning knob only, so a larger request is lowered.
template <class SR>
static void plan_fold(Context *ctx, Plan &P)
{
    if (std::is_same<SR, PlusTimes<double>>::value && ctx->fold == GBC_FOLD_EXACT) {
        P.want_aexp = true;
        if (P.tile_rows == 0)
            P.tile_rows = kXRows;
        else if (P.tile_rows > kXRowsBig)
            P.tile_rows = kXRowsBig;
        // columns of more than kSmallMid multiplications go to the exact
        // block kernel (R-MAT s14: 2.1x faster than the larger warp kernel)
        if (!P.s2_set) P.s2 = std::min<int64_t>(P.s2, kSmallMid);
    }
}

template <class SR>
static bool use_exact(const Plan &P)
{
    return std::is_same<SR, PlusTimes<double>>::value && P.want_aexp && P.max_R <= kXRowsBig;
}

// shared memory of k_numeric_x for a tile of RS rows
static size_t x_smem(int RS) { return (size_t)kXW * RS * 4 + RS; }

struct Lists {
    // [0, kWarpClasses): the warp-kernel classes (up to s1, kSmallMid,
    // kSmallMid2, s2 multiplications); [kBigList]: the big list
    const int64_t *l[kWarpClasses + 1] = {};
    int64_t n[kWarpClasses + 1] = {};
    int64_t total() const
    {
        int64_t t = 0;
        for (int c = 0; c <= kWarpClasses; ++c) t += n[c];
        return t;
    }
};

// Prepare one product (A*B) and append it to the plan.
static int plan_add(Workspace &ws, Plan &P, const DevMatrix &A, const DevMatrix &B)
{
    Context *ctx = ws.ctx;
    cudaStream_t s = ctx->stream;
    SpgemmArgs a{};
    int64_t *acp = nullptr;
    GBC_TRY(prepare_operands(ws, A, B, a, &acp, P.tile_rows));
    const int64_t nb = B.nzc;
    int64_t m1 = A.nrow > 1 ? A.nrow - 1 : 0;
    a.key_bits = 0;
    while (m1 > 0) {
        ++a.key_bits;
        m1 >>= 1;
    }
    uint64_t *amask = nullptr, *tmask = nullptr;
    int64_t *flop = nullptr;
    GBC_TRY(ws.alloc_n(&amask, (size_t)A.ncol * a.mask_words + 1));
    GBC_TRY(ws.alloc_n(&flop, nb + 1));
    GBC_TRY(ws.alloc_n(&tmask, (size_t)nb * a.mask_words + 1));
    if (A.ncol > 0) {
        k_amask<<<(unsigned)((A.ncol + 255) / 256), 256, 0, s>>>(A.ncol, a.tptr, a.T, a.mask_words, amask);
        note_launch();
    }
    if (nb > 0) {
        k_flop_mask<<<grid_for(ctx, (nb + 7) / 8, 8), 256, 0, s>>>(nb, B.cp, a.brow, acp, amask, a.mask_words, flop,
                                                                     tmask);
        note_launch();
    }
    GBC_CUDA_TRY(cudaGetLastError());
    a.flop = flop;
    a.tmask = tmask;
    a.aexp = nullptr;
    a.ktl_ptr = nullptr;
    a.ktl_start = nullptr;
    a.ktl_tile = nullptr;
    if (P.want_aexp) {
        int32_t *aexp = nullptr;
        GBC_TRY(ws.alloc_n(&aexp, (size_t)A.ncol + 1));
        if (A.ncol > 0) {
            k_aexp_f64<<<grid_for(ctx, (A.ncol + 7) / 8, 8), 256, 0, s>>>(A.ncol, acp,
                                                                         static_cast<const double *>(A.num), aexp);
            note_launch();
        }
        a.aexp = aexp;
        if (a.T <= (1 << 20) / std::max(a.R, kXRows) && A.ncol > 0) {
            // per-column tile lists of A (bucketing in the exact kernel)
            int64_t *kptr = nullptr;
            GBC_TRY(ws.alloc_n(&kptr, (size_t)A.ncol + 1));
            k_ktl_count<<<(unsigned)((A.ncol + 255) / 256), 256, 0, s>>>(A.ncol, amask, a.mask_words, kptr);
            note_launch();
            GBC_TRY(exclusive_scan_i64(ws, kptr, kptr, A.ncol, s));
            int64_t nent = 0;
            GBC_TRY(read_i64(ctx, kptr + A.ncol, &nent));
            uint32_t *kst = nullptr;
            uint16_t *ktt = nullptr;
            GBC_TRY(ws.alloc_n(&kst, (size_t)nent + 1));
            GBC_TRY(ws.alloc_n(&ktt, (size_t)nent + 1));
            k_ktl_fill<<<grid_for(ctx, (A.ncol + 7) / 8, 8), 256, 0, s>>>(A.ncol, a.tptr, a.T, kptr, kst, ktt);
            note_launch();
            GBC_CUDA_TRY(cudaGetLastError());
            a.ktl_ptr = kptr;
            a.ktl_start = kst;
            a.ktl_tile = ktt;
        }
    }
    a.aval = A.num;
    a.bval = B.num;
    a.col_base = P.total_cols;
    P.total_cols += nb;
    P.max_R = std::max(P.max_R, a.R);
    P.max_key_bits = std::max(P.max_key_bits, a.key_bits);
    int sup_rows = (int)std::min<int64_t>((int64_t)kSymRows, (int64_t)a.T * a.R);
    sup_rows = (sup_rows / a.R) * a.R;
    P.max_sym_smem = std::max(P.max_sym_smem, (size_t)sup_rows / 8);
    P.h.push_back(a);
    return GBC_OK;
}

static int plan_finalize(Workspace &ws, Plan &P)
{
    GBC_TRY(ws.alloc_n(&P.d, P.h.size() + 1));
    GBC_TRY(ws.alloc_n(&P.work, 16));
    GBC_CUDA_TRY(cudaMemsetAsync(P.work, 0, 16 * sizeof(unsigned long long), ws.ctx->stream));
    GBC_TRY(ws.alloc_n(&P.lbuf, kLists * ((size_t)P.total_cols + 1)));
    GBC_TRY(ws.alloc_n(&P.lcnt, kLists));
    if (P.want_aexp) {
        GBC_TRY(ws.alloc_n(&P.fb_items, (size_t)P.total_cols + 1));
        GBC_TRY(ws.alloc_n(&P.fb_cnt, 1));
        // bucketing scratch of the exact kernel: kXScap segments per resident block
        if (P.max_R > kXRows) {
            const size_t smem = x_smem(kXRowsBig);
            GBC_TRY(set_smem(k_numeric_x<kXThreadsBig, kXRowsBig>, smem));
            P.x_blocks = ws.ctx->num_sms *
                         resident_blocks(k_numeric_x<kXThreadsBig, kXRowsBig>, kXThreadsBig, smem, 1);
        } else {
            const size_t smem = x_smem(kXRows);
            GBC_TRY(set_smem(k_numeric_x<kXThreads, kXRows>, smem));
            P.x_blocks = ws.ctx->num_sms * resident_blocks(k_numeric_x<kXThreads, kXRows>, kXThreads, smem, 2);
        }
        GBC_TRY(ws.alloc_n(&P.xscratch, (size_t)P.x_blocks * kXScap));
    }
    GBC_CUDA_TRY(cudaMemcpyAsync(P.d, P.h.data(), P.h.size() * sizeof(SpgemmArgs), cudaMemcpyHostToDevice,
                                 ws.ctx->stream));
    return GBC_OK;
}

static void plan_options(Plan &P, const gbc_spgemm_opts &opt)
{
    P.tile_rows = opt.tile_rows;
    if (opt.tiny_limit >= 0) P.s1 = std::min<int64_t>(opt.tiny_limit, kSmall1);
    if (opt.small_limit >= 0) {
        P.s2 = std::min<int64_t>(std::max(opt.small_limit, P.s1), kSmall2);
        P.s2_set = true;
    }
}

static int plan_build(Workspace &ws, const DevMatrix &A, const DevMatrix &B, Plan &P)
{
    GBC_TRY(plan_add(ws, P, A, B));
    return plan_finalize(ws, P);
}

// Column lists: for every product (or only `pid` >= 0) its stored columns
// [j0, j1) (j1 < 0: all), optionally only the flagged ones; empty columns
// get cnt 0 in cnt_zero.
static int plan_classify(Plan &P, cudaStream_t s, int pid, int64_t j0, int64_t j1, Lists &L, int64_t *cnt_zero,
                         const int32_t *flagged = nullptr)
{
    constexpr int NL = kLists;
    GBC_CUDA_TRY(cudaMemsetAsync(P.lcnt, 0, NL * sizeof(unsigned long long), s));
    const int64_t stride = P.total_cols + 1;
    int64_t *lbig = P.lbuf + kWarpClasses * stride;
    for (int q = 0; q < (int)P.h.size(); ++q) {
        if (pid >= 0 && q != pid) continue;
        const SpgemmArgs &a = P.h[q];
        const int64_t lo = pid >= 0 ? j0 : 0, hi = (pid >= 0 && j1 >= 0) ? j1 : a.nb;
        if (hi > lo) {
            k_classify<<<(unsigned)((hi - lo + 255) / 256), 256, 0, s>>>(a.flop, q, a.col_base, lo, hi, P.s1, P.s2,
                                                                         P.lbuf, stride, P.lcnt, cnt_zero, flagged);
            note_launch();
        }
    }
    GBC_CUDA_TRY(cudaGetLastError());
    unsigned long long h[NL];
    GBC_CUDA_TRY(cudaMemcpyAsync(h, P.lcnt, sizeof(h), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    // the big list: bin 0 (heaviest) in place, the other bins appended
    int64_t nbig = (int64_t)h[kWarpClasses];
    for (int c = 1; c < kBigBins; ++c) {
        const int64_t nc = (int64_t)h[kWarpClasses + c];
        if (nc > 0)
            GBC_CUDA_TRY(
                cudaMemcpyAsync(lbig + nbig, lbig + c * stride, nc * sizeof(int64_t), cudaMemcpyDeviceToDevice, s));
        nbig += nc;
    }
    for (int c = 0; c < kWarpClasses; ++c) {
        L.l[c] = P.lbuf + c * stride;
        L.n[c] = (int64_t)h[c];
    }
    L.l[kBigList] = lbig;
    L.n[kBigList] = nbig;
    return GBC_OK;
}

// Warp-kernel counts of one class's columns (a TS-slot table per warp).
template <int TS, int WPB>
static int launch_small_count(Context *ctx, Plan &P, const int64_t *items, int64_t n, int64_t *cnt)
{
    const size_t sm = (size_t)WPB * TS * 4;
    GBC_TRY(set_smem(k_small_count<TS, WPB>, sm));
    const int per_sm = std::max(1, (int)(ctx->smem_optin / (sm + 1024)));
    k_small_count<TS, WPB><<<grid_for(ctx, (n + WPB - 1) / WPB, per_sm), WPB * 32, sm, ctx->stream>>>(P.d, items, n,
                                                                                                      cnt);
    note_launch();
    return GBC_OK;
}

// Exact nnz per listed column (estimateNNZ_Hash's result), into the
// batch-wide array cnt.
static int run_symbolic(Context *ctx, Plan &P, const Lists &L, int64_t *cnt)
{
    cudaStream_t s = ctx->stream;
    if (L.n[0] > 0) {
        constexpr int WPB = 8, TS = 2 * kSmall1;
        const size_t sm = (size_t)WPB * TS * 4;
        GBC_TRY(set_smem(k_small_count<TS, WPB>, sm));
        k_small_count<TS, WPB><<<grid_for(ctx, (L.n[0] + WPB - 1) / WPB, 8), WPB * 32, sm, s>>>(P.d, L.l[0], L.n[0],
                                                                                                 cnt);
        note_launch();
    }
    if (L.n[1] > 0) GBC_TRY((launch_small_count<2 * kSmallMid, 8>(ctx, P, L.l[1], L.n[1], cnt)));
    if (L.n[2] > 0) GBC_TRY((launch_small_count<2 * kSmallMid2, 4>(ctx, P, L.l[2], L.n[2], cnt)));
    if (L.n[3] > 0) GBC_TRY((launch_small_count<2 * kSmall2, 4>(ctx, P, L.l[3], L.n[3], cnt)));
    if (L.n[kBigList] > 0) {
        const size_t sym_smem = P.max_sym_smem;
        GBC_TRY(set_smem(k_symbolic, sym_smem));
        const int per_sm = resident_blocks(k_symbolic, kThreads, sym_smem, 8);
        GBC_CUDA_TRY(cudaMemsetAsync(P.work, 0, sizeof(unsigned long long), s));
        k_symbolic<<<grid_for(ctx, L.n[kBigList], per_sm), kThreads, sym_smem, s>>>(P.d, L.l[kBigList],
                                                                                     L.n[kBigList], cnt, P.work);
        note_launch();
    }
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

template <class SR, int FS, int WPB, bool PACK>
static int launch_small(Context *ctx, Plan &P, const int64_t *items, int64_t n, const int64_t *ccp, int64_t ccp_base,
                        const int64_t *cap, int64_t *out_cnt, int32_t *overflow, int64_t *cir, void *cval)
{
    typedef typename SR::V V;
    const size_t sm = WPB * small_warp_smem<FS, V, PACK>();
    GBC_TRY(set_smem(k_small_numeric<SR, FS, WPB, PACK>, sm));
    int per_sm = std::max(1, (int)(ctx->smem_optin / (sm + 1024)));
    k_small_numeric<SR, FS, WPB, PACK><<<grid_for(ctx, (n + WPB - 1) / WPB, std::min(per_sm, 8)), WPB * 32, sm,
                                         ctx->stream>>>(P.d, items, n, ccp, ccp_base, cap, out_cnt, overflow, cir,
                                                        cval);
    note_launch();
    return GBC_OK;
}

// The ordered (k-order fold) block kernel over `items`; with dyn_n the
// item count is read on the device (at most nitems).
template <class SR>
static int launch_big_ordered(Context *ctx, Plan &P, const int64_t *items, int64_t nitems,
                              const unsigned long long *dyn_n, const int64_t *ccp, int64_t ccp_base,
                              const int64_t *cap, int64_t *out_cnt, int32_t *overflow, int64_t *cir, void *cval)
{
    typedef typename SR::V V;
    cudaStream_t s = ctx->stream;
    GBC_CUDA_TRY(cudaMemsetAsync(P.work + 1, 0, sizeof(unsigned long long), s));
    if (P.max_R > 8192) {
        const size_t num_smem = numeric_smem_bytes(P.max_R, sizeof(V), 4096);
        GBC_TRY(set_smem(k_numeric<SR, 4096, kThreads>, num_smem));
        const int per_sm = resident_blocks(k_numeric<SR, 4096, kThreads>, kThreads, num_smem, 8);
        k_numeric<SR, 4096, kThreads><<<grid_for(ctx, nitems, per_sm), kThreads, num_smem, s>>>(
            P.d, items, nitems, ccp, ccp_base, cap, out_cnt, overflow, cir, cval, P.work + 1, dyn_n);
    } else if (P.max_R <= 4096) {
        const size_t num_smem = numeric_smem_bytes(P.max_R, sizeof(V), 1024);
        GBC_TRY(set_smem(k_numeric<SR, 1024, kThreads>, num_smem));
        const int per_sm = resident_blocks(k_numeric<SR, 1024, kThreads>, kThreads, num_smem, 4);
        k_numeric<SR, 1024, kThreads><<<grid_for(ctx, nitems, per_sm), kThreads, num_smem, s>>>(
            P.d, items, nitems, ccp, ccp_base, cap, out_cnt, overflow, cir, cval, P.work + 1, dyn_n);
    } else {
        // 8192-row tiles: 512-thread blocks, two per SM (64 registers)
        const size_t num_smem = numeric_smem_bytes(P.max_R, sizeof(V), 2048);
        GBC_TRY(set_smem(k_numeric<SR, 2048, 512>, num_smem));
        const int per_sm = resident_blocks(k_numeric<SR, 2048, 512>, 512, num_smem, 2);
        k_numeric<SR, 2048, 512><<<grid_for(ctx, nitems, per_sm), 512, num_smem, s>>>(
            P.d, items, nitems, ccp, ccp_base, cap, out_cnt, overflow, cir, cval, P.work + 1, dyn_n);
    }
    note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

// Exact (order-free) block kernel for PlusTimes fp64 over the big list;
// the columns it does not admit go to the ordered kernel afterwards
// (device-side count, no host synchronisation: graph capture stays valid).
template <class SR>
static int launch_big_exact(Context *ctx, Plan &P, const Lists &L, const int64_t *ccp, int64_t ccp_base,
                            const int64_t *cap, int64_t *out_cnt, int32_t *overflow, int64_t *cir, void *cval)
{
    cudaStream_t s = ctx->stream;
    const int grid = (int)std::min<int64_t>(P.x_blocks, L.n[kBigList]);  // the scratch holds P.x_blocks blocks
    GBC_CUDA_TRY(cudaMemsetAsync(P.work + 1, 0, 3 * sizeof(unsigned long long), s));
    GBC_CUDA_TRY(cudaMemsetAsync(P.fb_cnt, 0, sizeof(unsigned long long), s));
    if (P.max_R > kXRows)
        k_numeric_x<kXThreadsBig, kXRowsBig><<<grid, kXThreadsBig, x_smem(kXRowsBig), s>>>(
            P.d, L.l[kBigList], L.n[kBigList], ccp, ccp_base, cap, out_cnt, overflow, cir, static_cast<double *>(cval),
            P.work + 1, P.fb_items, P.fb_cnt, P.xscratch);
    else
        k_numeric_x<kXThreads, kXRows><<<grid, kXThreads, x_smem(kXRows), s>>>(
            P.d, L.l[kBigList], L.n[kBigList], ccp, ccp_base, cap, out_cnt, overflow, cir, static_cast<double *>(cval),
            P.work + 1, P.fb_items, P.fb_cnt, P.xscratch);
    note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    return launch_big_ordered<SR>(ctx, P, P.fb_items, L.n[kBigList], P.fb_cnt, ccp, ccp_base, cap, out_cnt, overflow, cir,
                                  cval);
}

// Numeric pass over the listed columns.  Exact sizing: cap == nullptr and
// ccp holds the exact offsets.  Learned sizing: cap gives each column's room
// at ccp[g - ccp_base]; out_cnt/overflow receive actual counts and flags.
// All per-column arrays are indexed by batch-wide column g.
template <class SR>
static int run_numeric(Context *ctx, Plan &P, const Lists &L, const int64_t *ccp, int64_t ccp_base, const int64_t *cap,
                       int64_t *out_cnt, int32_t *overflow, int64_t *cir, void *cval)
{
    const bool pack = P.max_key_bits <= 20;
    if (L.n[0] > 0) {
        if (pack)
            GBC_TRY((launch_small<SR, kSmall1, 8, true>(ctx, P, L.l[0], L.n[0], ccp, ccp_base, cap, out_cnt, overflow,
                                                         cir, cval)));
        else
            GBC_TRY((launch_small<SR, kSmall1, 8, false>(ctx, P, L.l[0], L.n[0], ccp, ccp_base, cap, out_cnt,
                                                          overflow, cir, cval)));
    }
    if (L.n[1] > 0) {
        if (pack)
            GBC_TRY((launch_small<SR, kSmallMid, 4, true>(ctx, P, L.l[1], L.n[1], ccp, ccp_base, cap, out_cnt,
                                                           overflow, cir, cval)));
        else
            GBC_TRY((launch_small<SR, kSmallMid, 4, false>(ctx, P, L.l[1], L.n[1], ccp, ccp_base, cap, out_cnt,
                                                            overflow, cir, cval)));
    }
    if (L.n[2] > 0) {
        if (pack)
            GBC_TRY((launch_small<SR, kSmallMid2, 2, true>(ctx, P, L.l[2], L.n[2], ccp, ccp_base, cap, out_cnt,
                                                            overflow, cir, cval)));
        else
            GBC_TRY((launch_small<SR, kSmallMid2, 2, false>(ctx, P, L.l[2], L.n[2], ccp, ccp_base, cap, out_cnt,
                                                             overflow, cir, cval)));
    }
    if (L.n[3] > 0) {
        if (pack)
            GBC_TRY((launch_small<SR, kSmall2, 2, true>(ctx, P, L.l[3], L.n[3], ccp, ccp_base, cap, out_cnt, overflow,
                                                         cir, cval)));
        else
            GBC_TRY((launch_small<SR, kSmall2, 2, false>(ctx, P, L.l[3], L.n[3], ccp, ccp_base, cap, out_cnt,
                                                          overflow, cir, cval)));
    }
    if (L.n[kBigList] > 0) {
        if (use_exact<SR>(P))
            GBC_TRY(launch_big_exact<SR>(ctx, P, L, ccp, ccp_base, cap, out_cnt, overflow, cir, cval));
        else
            GBC_TRY(launch_big_ordered<SR>(ctx, P, L.l[kBigList], L.n[kBigList], nullptr, ccp, ccp_base, cap,
                                           out_cnt, overflow,
                                           cir, cval));
    }
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

static int check_err(Context *ctx, const Plan &P)
{
    for (const SpgemmArgs &a : P.h) {
        int32_t herr = 0;
        GBC_CUDA_TRY(cudaMemcpyAsync(&herr, a.err, sizeof(herr), cudaMemcpyDeviceToHost, ctx->stream));
        GBC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        if (herr) return fail(GBC_ECUDA, "internal error: numeric and symbolic counts disagree");
    }
    return GBC_OK;
}

// Turn per-column exact counts into the result's column structure (keeping
// or dropping empty output columns) -- shared by every sizing mode.
static int finish_columns(Context *ctx, Workspace &ws, const DevMatrix &B, const gbc_spgemm_opts &opt, int64_t nb,
                          const int64_t *cnt, gbc_result *C)
{
    cudaStream_t s = ctx->stream;
    if (opt.keep_empty || nb == 0) {
        C->nzc = nb;
        GBC_TRY(device_alloc(ctx, (void **)&C->jc, (nb + 1) * sizeof(int64_t)));
        if (nb > 0) {
            k_iota_jc<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, B.jc, C->jc);
            note_launch();
        }
        return GBC_OK;
    }
    int64_t *flags = nullptr;
    GBC_TRY(ws.alloc_n(&flags, nb + 1));
    k_nonempty_flags<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, cnt, flags);
    note_launch();
    GBC_TRY(exclusive_scan_i64(ws, flags, flags, nb, s));
    int64_t nzc = 0;
    GBC_TRY(read_i64(ctx, flags + nb, &nzc));
    int64_t *cp2 = nullptr, *jc2 = nullptr;
    GBC_TRY(device_alloc(ctx, (void **)&cp2, (nzc + 1) * sizeof(int64_t)));
    int rc = device_alloc(ctx, (void **)&jc2, (nzc + 1) * sizeof(int64_t));
    if (rc != GBC_OK) {
        device_free(ctx, cp2);
        return rc;
    }
    GBC_CUDA_TRY(cudaMemsetAsync(cp2, 0, sizeof(int64_t), s));
    k_compact_cols<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, cnt, flags, C->cp, B.jc, cp2, jc2);
    note_launch();
    device_free(ctx, C->cp);
    C->cp = cp2;
    C->jc = jc2;
    C->nzc = nzc;
    return GBC_OK;
}

static int64_t sum_i64(Workspace &ws, Context *ctx, const int64_t *v, int64_t n)
{
    int64_t *tmp = nullptr;
    if (ws.alloc_n(&tmp, n + 1) != GBC_OK) return -1;
    if (exclusive_scan_i64(ws, v, tmp, n, ctx->stream) != GBC_OK) return -1;
    int64_t t = 0;
    if (read_i64(ctx, tmp + n, &t) != GBC_OK) return -1;
    return t;
}

template <class SR>
static int spgemm_exact(Context *ctx, const DevMatrix &A, const DevMatrix &B, const gbc_spgemm_opts &opt, int vt,
                        gbc_result **Cout, gbc_spgemm_stats *st)
{
    typedef typename SR::V V;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    cudaEventRecord(ctx->ev[0], s);
    Plan P;
    plan_options(P, opt);
    plan_fold<SR>(ctx, P);
    GBC_TRY(plan_build(ws, A, B, P));
    const int64_t nb = B.nzc;
    int64_t *cnt = nullptr, *ccp = nullptr;
    GBC_TRY(ws.alloc_n(&cnt, nb + 1));
    Lists L;
    GBC_TRY(plan_classify(P, s, -1, 0, -1, L, cnt));
    cudaEventRecord(ctx->ev[1], s);
    GBC_TRY(run_symbolic(ctx, P, L, cnt));
    GBC_TRY(device_alloc(ctx, (void **)&ccp, (nb + 1) * sizeof(int64_t)));
    gbc_result *C = new gbc_result();
    C->ctx = ctx;
    C->nrow = A.nrow;
    C->ncol = B.ncol;
    C->valtype = vt;
    C->cp = ccp;
    int rc = exclusive_scan_i64(ws, cnt, ccp, nb, s);
    int64_t nnzc = 0;
    if (rc == GBC_OK) rc = read_i64(ctx, ccp + nb, &nnzc);
    cudaEventRecord(ctx->ev[2], s);
    C->nnz = nnzc;
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&C->ir, (nnzc + 1) * sizeof(int64_t));
    if (rc == GBC_OK) rc = device_alloc(ctx, &C->num, (nnzc + 1) * sizeof(V));
    if (rc == GBC_OK && nnzc > 0) rc = run_numeric<SR>(ctx, P, L, ccp, 0, nullptr, nullptr, nullptr, C->ir, C->num);
    cudaEventRecord(ctx->ev[3], s);
    if (rc == GBC_OK) rc = finish_columns(ctx, ws, B, opt, nb, cnt, C);
    cudaEventRecord(ctx->ev[4], s);
    if (rc == GBC_OK) rc = check_err(ctx, P);
    if (rc != GBC_OK) {
        gbc_result_free(C);
        return rc;
    }
    if (st) {
        st->flops = sum_i64(ws, ctx, P.a().flop, nb);
        st->nnz = nnzc;
        st->overflow_cols = 0;
        st->alloc_entries = nnzc;
        float t04 = 0, t12 = 0, t23 = 0;
        cudaEventElapsedTime(&t04, ctx->ev[0], ctx->ev[4]);
        cudaEventElapsedTime(&t12, ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&t23, ctx->ev[2], ctx->ev[3]);
        st->ms_total = t04;
        st->ms_symbolic = t12;
        st->ms_numeric = t23;
        st->tile_visits_dense = 0;
        st->tile_visits_range = 0;
        if (use_exact<SR>(P)) {
            GBC_TRY(read_i64(ctx, reinterpret_cast<const int64_t *>(P.work + 2), &st->tile_visits_dense));
            GBC_TRY(read_i64(ctx, reinterpret_cast<const int64_t *>(P.work + 3), &st->tile_visits_range));
        }
    }
    *Cout = C;
    return GBC_OK;
}

// ------------------------------------------------------- learned sizing
// Per-column features of the sizing MLP: log2(1+x) of nnz(B(:,j)), flop,
// the largest and the spread (standard deviation) of the referenced A
// column lengths, the number of 8192-row bands touched, and the row count.
__global__ void k_features(SpgemmArgs a, int64_t nb, float *feat)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp; i < nb; i += nwarps) {
        const int64_t bs = a.bcp[i], be = a.bcp[i + 1];
        double sum = 0, sq = 0, mx = 0;
        for (int64_t p = bs + lane; p < be; p += 32) {
            const int k = a.brow[p];
            const double len = (double)(a.acp[k + 1] - a.acp[k]);
            sum += len;
            sq += len * len;
            mx = fmax(mx, len);
        }
        // touched 8192-row bands, whatever the plan's tile height: groups
        // of f = 8192 / R tile bits are OR-folded (R a power of two that
        // divides 8192; other heights count their own tiles)
        const int f = (a.R <= 8192 && (8192 % a.R) == 0 && (a.R & (a.R - 1)) == 0) ? 8192 / a.R : 1;
        uint64_t keep = 0;  // bit 0 of every group of f
        for (int b = 0; b < 64; b += f) keep |= 1ull << b;
        int tiles = 0;
        for (int w = lane; w < a.mask_words; w += 32) {
            uint64_t m = a.tmask[i * a.mask_words + w];
            for (int sh = 1; sh < f; sh <<= 1) m |= m >> sh;
            tiles += __popcll(m & keep);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            sum += __shfl_xor_sync(0xffffffffu, sum, o);
            sq += __shfl_xor_sync(0xffffffffu, sq, o);
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            tiles += __shfl_xor_sync(0xffffffffu, tiles, o);
        }
        if (lane == 0) {
            const double nbj = (double)(be - bs);
            const double mean = nbj > 0 ? sum / nbj : 0.0;
            const double var = nbj > 0 ? fmax(sq / nbj - mean * mean, 0.0) : 0.0;
            float *f = feat + i * kNF;
            f[0] = log2f(1.f + (float)nbj);
            f[1] = log2f(1.f + (float)sum);
            f[2] = log2f(1.f + (float)mx);
            f[3] = log2f(1.f + sqrtf((float)var));
            f[4] = log2f(1.f + (float)tiles);
            f[5] = log2f(1.f + (float)a.m);
        }
    }
}

// capacity = 2^(prediction + margin) - 1, at least 1 and at most min(flop, m)
__global__ void k_capacity(int64_t nb, const int64_t *flop, const float *pred, float margin, int64_t m, int64_t *cap)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const int64_t f = flop[i];
    if (f == 0) {
        cap[i] = 0;
        return;
    }
    const float e = fminf(pred[i] + margin, 62.f);
    int64_t c = (int64_t)ceilf(exp2f(e)) - 1;
    if (c < 1) c = 1;
    const int64_t hi = f < m ? f : m;
    cap[i] = c > hi ? hi : c;
}

__global__ void k_masked_counts(int64_t nb, const int32_t *flag, const int64_t *cnt, int64_t *out)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < nb) out[i] = flag[i] ? cnt[i] : 0;
}

__global__ void k_final_counts(int64_t nb, const int32_t *flag, const int64_t *exact, int64_t *cnt)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < nb && flag[i]) cnt[i] = exact[i];
}

// Gather every column from its region (slots, or the overflow region for
// flagged columns) into the contiguous result.
template <typename V>
__global__ void k_compact(int64_t nb, const int64_t *cnt, const int64_t *dst, const int32_t *flag,
                          const int64_t *beg0, const int64_t *ir0, const V *v0, const int64_t *beg1,
                          const int64_t *ir1, const V *v1, int64_t *oir, V *ov)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp; i < nb; i += nwarps) {
        const bool o = flag[i] != 0;
        const int64_t b = o ? beg1[i] : beg0[i];
        const int64_t *sir = o ? ir1 : ir0;
        const V *sv = o ? v1 : v0;
        const int64_t d = dst[i];
        for (int64_t p = lane; p < cnt[i]; p += 32) {
            oir[d + p] = sir[b + p];
            ov[d + p] = sv[b + p];
        }
    }
}

// ------------------------------------------------------- column phases
// Checksums of one phase's output, independent of where each column's
// entries sit (contiguous, capacity slots, or the overflow region): per
// block, over a fixed contiguous range of the phase's columns, the sum of
// row ids, the sum of values as double (warp-column order, so equal only
// for equal phase cuts) and the wrap-around sum of a 64-bit mix of
// (column, row, value bits) -- equal for equal products whatever the phases.
__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 31;
    x *= 0x7fb5d329728ea185ull;
    x ^= x >> 27;
    x *= 0x81dadef4bc2dd44dull;
    x ^= x >> 33;
    return x;
}

template <typename V>
__device__ __forceinline__ uint64_t value_bits(V v)
{
    if constexpr (sizeof(V) == 8) {
        uint64_t u;
        memcpy(&u, &v, 8);
        return u;
    } else if constexpr (sizeof(V) == 4) {
        uint32_t u;
        memcpy(&u, &v, 4);
        return u;
    } else {
        return (uint64_t)(uint8_t)v;
    }
}

// One region of a phase's output: column i owns slots [start[i], start[i+1])
// of (ir, val), of which the first cnt[i] (all, when cnt is null) hold
// entries; columns with skip[i] set hold none here.
struct ChecksumRegion {
    int64_t ncols;
    const int64_t *col;    // global column id of each (B's jc), or null: j0 + i
    int64_t j0;
    const int64_t *start;  // [ncols+1]
    const int64_t *cnt;    // [ncols] or null
    const int32_t *skip;   // [ncols] or null
    const int64_t *ir;
    const void *val;
};

// Each block takes one contiguous range of slots, so long columns are
// shared among blocks; threads walk the columns that meet the range.
template <typename V>
__global__ void __launch_bounds__(256) k_phase_checksum(ChecksumRegion R, int64_t *rsum, double *vsum,
                                                        unsigned long long *hsum)
{
    __shared__ double sv[kWarps];
    __shared__ long long sr[kWarps];
    __shared__ unsigned long long sh[kWarps];
    __shared__ int64_t s_first;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t total = R.ncols > 0 ? R.start[R.ncols] : 0;
    const int64_t per = (total + gridDim.x - 1) / gridDim.x;
    const int64_t p0 = min(total, per * blockIdx.x), p1 = min(total, p0 + per);
    if (threadIdx.x == 0) {
        // last column whose start is <= p0 (upper bound - 1)
        int64_t lo = 0, hi = R.ncols;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (R.start[mid] <= p0) lo = mid + 1;
            else hi = mid;
        }
        s_first = lo > 0 ? lo - 1 : 0;
    }
    __syncthreads();
    const V *vv = static_cast<const V *>(R.val);
    double v = 0;
    long long r = 0;
    unsigned long long h = 0;
    if (p1 > p0) {
        for (int64_t i = s_first; i < R.ncols; ++i) {
            const int64_t cs = R.start[i];
            if (cs >= p1) break;
            if (R.skip && R.skip[i]) continue;
            const int64_t ce = R.cnt ? cs + R.cnt[i] : R.start[i + 1];
            const int64_t b = max(cs, p0), e = min(ce, p1);
            const uint64_t col = (uint64_t)(R.col ? R.col[i] : R.j0 + i);
            for (int64_t p = b + threadIdx.x; p < e; p += blockDim.x) {
                const int64_t row = R.ir[p];
                const V x = vv[p];
                v += (double)x;
                r += row;
                h += mix64((col << 32 ^ (uint64_t)row) * 0x9e3779b97f4a7c15ull ^ value_bits(x));
            }
        }
    }
#pragma unroll
    for (int k = 16; k; k >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, k);
        r += __shfl_xor_sync(0xffffffffu, r, k);
        h += __shfl_xor_sync(0xffffffffu, h, k);
    }
    if (lane == 0) {
        sv[w] = v;
        sr[w] = r;
        sh[w] = h;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tv = 0;
        long long tr = 0;
        unsigned long long th = 0;
        for (int k = 0; k < kWarps; ++k) {
            tv += sv[k];
            tr += sr[k];
            th += sh[k];
        }
        vsum[blockIdx.x] = tv;
        rsum[blockIdx.x] = tr;
        hsum[blockIdx.x] = th;
    }
}

// Grow-only device buffer owned by a Workspace.
template <typename T>
static int grow(Workspace &ws, T **p, int64_t *have, int64_t need)
{
    if (*p && *have >= need) return GBC_OK;
    const int64_t n = std::max<int64_t>(need, *have + *have / 2) + 1;
    GBC_TRY(ws.alloc_n(p, (size_t)n));
    *have = n;
    return GBC_OK;
}

static int learned_capacity(Context *ctx, Workspace &ws, Plan &P, int64_t nb, int64_t m, int64_t *cap)
{
    cudaStream_t s = ctx->stream;
    Mlp *mlp = static_cast<Mlp *>(ctx->mlp);
    if (!mlp || !mlp->trained)
        return fail(GBC_EINVAL, "learned sizing needs a trained model (gbc_context_set_mlp)");
    float *feat = nullptr, *pred = nullptr;
    GBC_TRY(ws.alloc_n(&feat, (size_t)nb * kNF + 1));
    GBC_TRY(ws.alloc_n(&pred, nb + 1));
    if (nb > 0) {
        k_features<<<grid_for(ctx, (nb + 7) / 8, 8), 256, 0, s>>>(P.a(), nb, feat);
        note_launch();
        GBC_TRY(mlp_predict_device(mlp, feat, nb, pred, s));
        k_capacity<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, P.a().flop, pred, mlp->margin, m, cap);
        note_launch();
    }
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

// C = A*B computed in phases of B's stored columns so that each phase's
// output holds at most max_phase_nnz entries -- the reference's column
// phases of MemEfficientSpGEMM (ParFriends.h:553-556, ColSplit).  Each
// phase's C is written to HBM and reduced to checksums; nothing is kept.
// Exact sizing cuts phases on the symbolic counts; learned sizing cuts them
// on predicted capacities, writes each column into its slots and recomputes
// the columns that overflowed exactly (symbolic + numeric) into a second
// region before the phase's checksum.
template <class SR>
static int spgemm_phased(Context *ctx, const DevMatrix &A, const DevMatrix &B, int64_t max_phase_nnz, int sizing,
                         gbc_phased_stats *st)
{
    typedef typename SR::V V;
    const bool learned = sizing == GBC_SIZING_LEARNED;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    cudaEventRecord(ctx->ev[0], s);
    Plan P;
    plan_fold<SR>(ctx, P);
    GBC_TRY(plan_build(ws, A, B, P));
    const int64_t nb = B.nzc;
    int64_t *size = nullptr;  // exact counts, or capacities when learned
    GBC_TRY(ws.alloc_n(&size, nb + 1));
    Lists L;
    cudaEventRecord(ctx->ev[1], s);
    if (learned) {
        GBC_TRY(learned_capacity(ctx, ws, P, nb, A.nrow, size));
    } else {
        GBC_TRY(plan_classify(P, s, -1, 0, -1, L, size));
        GBC_TRY(run_symbolic(ctx, P, L, size));
    }
    cudaEventRecord(ctx->ev[2], s);
    std::vector<int64_t> hsize(nb > 0 ? nb : 1);
    if (nb > 0) GBC_CUDA_TRY(cudaMemcpyAsync(hsize.data(), size, nb * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    const int64_t flops = sum_i64(ws, ctx, P.a().flop, nb);
    // phase boundaries (greedy; a column bigger than the budget is alone)
    std::vector<int64_t> bounds{0};
    int64_t acc = 0, maxp = 0, alloc = 0;
    for (int64_t j = 0; j < nb; ++j) {
        if (acc > 0 && acc + hsize[j] > max_phase_nnz) {
            bounds.push_back(j);
            maxp = std::max(maxp, acc);
            acc = 0;
        }
        acc += hsize[j];
        alloc += hsize[j];
    }
    maxp = std::max(maxp, acc);
    if (bounds.back() != nb) bounds.push_back(nb);
    int64_t maxcols = 0;
    for (size_t p = 0; p + 1 < bounds.size(); ++p) maxcols = std::max(maxcols, bounds[p + 1] - bounds[p]);
    const int csb = ctx->num_sms * 8;  // checksum blocks per region: enough warps to keep HBM busy
    const int np = (int)bounds.size() - 1;
    int64_t *ir = nullptr, *ccp = nullptr, *rsum = nullptr;
    V *num = nullptr;
    double *vsum = nullptr;
    unsigned long long *hsum = nullptr;
    GBC_TRY(ws.alloc_n(&ir, maxp + 1));
    GBC_TRY(ws.alloc_n(&num, maxp + 1));
    GBC_TRY(ws.alloc_n(&ccp, maxcols + 1));
    GBC_TRY(ws.alloc_n(&rsum, (size_t)csb * 2 * (np + 1)));
    GBC_TRY(ws.alloc_n(&vsum, (size_t)csb * 2 * (np + 1)));
    GBC_TRY(ws.alloc_n(&hsum, (size_t)csb * 2 * (np + 1)));
    // learned: per-column counts, overflow flags and the exact-rerun region
    int64_t *cnt = nullptr, *exact = nullptr, *masked = nullptr, *beg1 = nullptr, *ir1 = nullptr;
    V *num1 = nullptr;
    int32_t *flag = nullptr;
    int64_t have1 = 0, have1v = 0, overflow_cols = 0, total = 0;
    if (learned) {
        GBC_TRY(ws.alloc_n(&cnt, nb + 1));
        GBC_TRY(ws.alloc_n(&exact, nb + 1));
        GBC_TRY(ws.alloc_n(&masked, maxcols + 1));
        GBC_TRY(ws.alloc_n(&beg1, maxcols + 1));
        GBC_TRY(ws.alloc_n(&flag, nb + 1));
        GBC_CUDA_TRY(cudaMemsetAsync(flag, 0, (nb + 1) * sizeof(int32_t), s));
        GBC_CUDA_TRY(cudaMemsetAsync(cnt, 0, (nb + 1) * sizeof(int64_t), s));
    }
    double ms_num = 0, ms_rerun = 0;
    for (int p = 0; p < np; ++p) {
        const int64_t j0 = bounds[p], j1 = bounds[p + 1], nc = j1 - j0;
        Lists Lp;
        GBC_TRY(plan_classify(P, s, 0, j0, j1, Lp, nullptr));
        GBC_TRY(exclusive_scan_i64(ws, size + j0, ccp, nc, s));
        cudaEventRecord(ctx->ev[5], s);
        if (learned)
            GBC_TRY(run_numeric<SR>(ctx, P, Lp, ccp, j0, size, cnt, flag, ir, num));
        else
            GBC_TRY(run_numeric<SR>(ctx, P, Lp, ccp, j0, nullptr, nullptr, nullptr, ir, num));
        cudaEventRecord(ctx->ev[6], s);
        ChecksumRegion R0{nc, B.jc ? B.jc + j0 : nullptr, j0, ccp, nullptr, nullptr, ir, num};
        ChecksumRegion R1{0, nullptr, j0, nullptr, nullptr, nullptr, nullptr, nullptr};
        if (learned) {
            Lists Lo;
            GBC_TRY(plan_classify(P, s, 0, j0, j1, Lo, nullptr, flag));
            const int64_t no = Lo.total();
            overflow_cols += no;
            if (no > 0) {
                cudaEventRecord(ctx->ev[3], s);
                GBC_TRY(run_symbolic(ctx, P, Lo, exact));
                k_masked_counts<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(nc, flag + j0, exact + j0, masked);
                note_launch();
                GBC_TRY(exclusive_scan_i64(ws, masked, beg1, nc, s));
                int64_t tot1 = 0;
                GBC_TRY(read_i64(ctx, beg1 + nc, &tot1));
                GBC_TRY(grow(ws, &ir1, &have1, tot1));
                GBC_TRY(grow(ws, &num1, &have1v, tot1));
                GBC_TRY(run_numeric<SR>(ctx, P, Lo, beg1, j0, nullptr, nullptr, nullptr, ir1, num1));
                k_final_counts<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(nc, flag + j0, exact + j0, cnt + j0);
                note_launch();
                cudaEventRecord(ctx->ev[4], s);
                GBC_CUDA_TRY(cudaEventSynchronize(ctx->ev[4]));
                float ms = 0;
                cudaEventElapsedTime(&ms, ctx->ev[3], ctx->ev[4]);
                ms_rerun += ms;
            }
            R0.cnt = cnt + j0;
            R0.skip = flag + j0;
            if (no > 0) R1 = ChecksumRegion{nc, R0.col, j0, beg1, nullptr, nullptr, ir1, num1};
        }
        const size_t o0 = (size_t)(2 * p) * csb, o1 = o0 + csb;
        GBC_CUDA_TRY(cudaMemsetAsync(rsum + o0, 0, 2 * csb * sizeof(int64_t), s));
        GBC_CUDA_TRY(cudaMemsetAsync(vsum + o0, 0, 2 * csb * sizeof(double), s));
        GBC_CUDA_TRY(cudaMemsetAsync(hsum + o0, 0, 2 * csb * sizeof(unsigned long long), s));
        if (nc > 0) {
            k_phase_checksum<V><<<csb, kThreads, 0, s>>>(R0, rsum + o0, vsum + o0, hsum + o0);
            note_launch();
        }
        if (R1.ncols > 0) {
            k_phase_checksum<V><<<csb, kThreads, 0, s>>>(R1, rsum + o1, vsum + o1, hsum + o1);
            note_launch();
        }
        GBC_CUDA_TRY(cudaGetLastError());
        GBC_CUDA_TRY(cudaEventSynchronize(ctx->ev[6]));
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]);
        ms_num += ms;
    }
    if (learned) {
        total = sum_i64(ws, ctx, cnt, nb);
    } else {
        total = alloc;
    }
    cudaEventRecord(ctx->ev[4], s);
    const size_t nparts = (size_t)csb * 2 * np;
    std::vector<int64_t> hr(nparts + 1);
    std::vector<double> hv(nparts + 1);
    std::vector<unsigned long long> hh(nparts + 1);
    if (np > 0) {
        GBC_CUDA_TRY(cudaMemcpyAsync(hr.data(), rsum, nparts * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(hv.data(), vsum, nparts * sizeof(double), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(hh.data(), hsum, nparts * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
    }
    GBC_TRY(check_err(ctx, P));
    if (st) {
        float t04 = 0, t12 = 0;
        cudaEventElapsedTime(&t04, ctx->ev[0], ctx->ev[4]);
        cudaEventElapsedTime(&t12, ctx->ev[1], ctx->ev[2]);
        st->flops = flops;
        st->nnz = total;
        st->phases = np;
        st->ms_total = t04;
        st->ms_sizing = t12;
        st->ms_numeric = ms_num;
        st->ms_rerun = ms_rerun;
        st->overflow_cols = overflow_cols;
        st->alloc_nnz = alloc;
        int64_t rs = 0;
        double vs = 0;
        uint64_t hs = 0;
        for (size_t k = 0; k < nparts; ++k) {
            rs += hr[k];
            vs += hv[k];
            hs += hh[k];
        }
        st->row_checksum = rs;
        st->val_checksum = vs;
        st->content_hash = hs;
        st->max_phase_nnz = maxp;
    }
    return GBC_OK;
}

// The learned product before compaction: column i holds cnt[i] entries at
// beg0[i] of (ir0, v0), or -- when flag[i] (capacity overflow, recomputed
// exactly) -- at beg1[i] of (ir1, v1).  Allocations live in `ws`.
struct LearnedOut {
    int64_t *beg0 = nullptr, *ir0 = nullptr, *beg1 = nullptr, *ir1 = nullptr, *cnt = nullptr;
    void *v0 = nullptr, *v1 = nullptr;
    int32_t *flag = nullptr;
    int64_t nb = 0, alloc = 0, overflow_cols = 0, flops = 0;
    double ms_predict = 0, ms_numeric = 0, ms_rerun = 0;
};

template <class SR>
static int learned_into_slots(Context *ctx, Workspace &ws, const DevMatrix &A, const DevMatrix &B, Plan &P,
                              LearnedOut &O)
{
    typedef typename SR::V V;
    cudaStream_t s = ctx->stream;
    Mlp *mlp = static_cast<Mlp *>(ctx->mlp);
    if (!mlp || !mlp->trained)
        return fail(GBC_EINVAL, "learned sizing needs a trained model (gbc_context_set_mlp)");
    GBC_TRY(plan_build(ws, A, B, P));
    const int64_t nb = B.nzc;
    O.nb = nb;
    Lists L;
    GBC_TRY(plan_classify(P, s, -1, 0, -1, L, nullptr));
    float *feat = nullptr, *pred = nullptr;
    GBC_TRY(ws.alloc_n(&feat, (size_t)nb * kNF + 1));
    GBC_TRY(ws.alloc_n(&pred, nb + 1));
    GBC_TRY(ws.alloc_n(&O.cnt, nb + 1));
    GBC_TRY(ws.alloc_n(&O.flag, nb + 1));
    GBC_TRY(ws.alloc_n(&O.beg0, nb + 1));
    int64_t *cap = nullptr;
    GBC_TRY(ws.alloc_n(&cap, nb + 1));
    GBC_CUDA_TRY(cudaMemsetAsync(O.flag, 0, (nb + 1) * sizeof(int32_t), s));
    GBC_CUDA_TRY(cudaMemsetAsync(O.cnt, 0, (nb + 1) * sizeof(int64_t), s));
    cudaEventRecord(ctx->ev[5], s);
    if (nb > 0) {
        k_features<<<grid_for(ctx, (nb + 7) / 8, 8), 256, 0, s>>>(P.a(), nb, feat);
        note_launch();
        GBC_TRY(mlp_predict_device(mlp, feat, nb, pred, s));
        k_capacity<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, P.a().flop, pred, mlp->margin, A.nrow, cap);
        note_launch();
    }
    GBC_TRY(exclusive_scan_i64(ws, cap, O.beg0, nb, s));
    GBC_TRY(read_i64(ctx, O.beg0 + nb, &O.alloc));
    cudaEventRecord(ctx->ev[6], s);
    GBC_TRY(ws.alloc_n(&O.ir0, O.alloc + 1));
    GBC_TRY(ws.alloc(&O.v0, (O.alloc + 1) * sizeof(V)));
    GBC_TRY(run_numeric<SR>(ctx, P, L, O.beg0, 0, cap, O.cnt, O.flag, O.ir0, O.v0));
    cudaEventRecord(ctx->ev[7], s);
    // columns that overflowed their capacity: exact symbolic + numeric
    Lists Lo;
    GBC_TRY(plan_classify(P, s, -1, 0, -1, Lo, nullptr, O.flag));
    {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]);
        O.ms_predict = ms;
        cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]);
        O.ms_numeric = ms;
    }
    O.overflow_cols = Lo.total();
    GBC_TRY(ws.alloc_n(&O.beg1, nb + 1));
    if (O.overflow_cols > 0) {
        cudaEventRecord(ctx->ev[5], s);
        int64_t *exact = nullptr, *masked = nullptr;
        GBC_TRY(ws.alloc_n(&exact, nb + 1));
        GBC_TRY(ws.alloc_n(&masked, nb + 1));
        GBC_TRY(run_symbolic(ctx, P, Lo, exact));
        k_masked_counts<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, O.flag, exact, masked);
        note_launch();
        GBC_TRY(exclusive_scan_i64(ws, masked, O.beg1, nb, s));
        int64_t tot = 0;
        GBC_TRY(read_i64(ctx, O.beg1 + nb, &tot));
        GBC_TRY(ws.alloc_n(&O.ir1, tot + 1));
        GBC_TRY(ws.alloc(&O.v1, (tot + 1) * sizeof(V)));
        GBC_TRY(run_numeric<SR>(ctx, P, Lo, O.beg1, 0, nullptr, nullptr, nullptr, O.ir1, O.v1));
        k_final_counts<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, O.flag, exact, O.cnt);
        note_launch();
        cudaEventRecord(ctx->ev[6], s);
        GBC_CUDA_TRY(cudaEventSynchronize(ctx->ev[6]));
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]);
        O.ms_rerun = ms;
    } else {
        O.ir1 = O.ir0;
        O.v1 = O.v0;
        GBC_CUDA_TRY(cudaMemsetAsync(O.beg1, 0, (nb + 1) * sizeof(int64_t), s));
    }
    O.flops = sum_i64(ws, ctx, P.a().flop, nb);
    return check_err(ctx, P);
}

template <class SR>
int spgemm_learned(Context *ctx, const DevMatrix &A, const DevMatrix &B, const gbc_spgemm_opts &opt, int vt,
                   gbc_result **Cout, gbc_spgemm_stats *st)
{
    typedef typename SR::V V;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    cudaEventRecord(ctx->ev[0], s);
    Plan P;
    plan_options(P, opt);
    plan_fold<SR>(ctx, P);
    LearnedOut O;
    GBC_TRY(learned_into_slots<SR>(ctx, ws, A, B, P, O));
    const int64_t nb = O.nb;
    int64_t *ccp = nullptr;
    GBC_TRY(device_alloc(ctx, (void **)&ccp, (nb + 1) * sizeof(int64_t)));
    gbc_result *C = new gbc_result();
    C->ctx = ctx;
    C->nrow = A.nrow;
    C->ncol = B.ncol;
    C->valtype = vt;
    C->cp = ccp;
    int rc = exclusive_scan_i64(ws, O.cnt, ccp, nb, s);
    int64_t nnzc = 0;
    if (rc == GBC_OK) rc = read_i64(ctx, ccp + nb, &nnzc);
    C->nnz = nnzc;
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&C->ir, (nnzc + 1) * sizeof(int64_t));
    if (rc == GBC_OK) rc = device_alloc(ctx, &C->num, (nnzc + 1) * sizeof(V));
    if (rc == GBC_OK && nb > 0) {
        k_compact<V><<<grid_for(ctx, (nb + 7) / 8, 8), 256, 0, s>>>(
            nb, O.cnt, ccp, O.flag, O.beg0, O.ir0, static_cast<const V *>(O.v0), O.beg1, O.ir1,
            static_cast<const V *>(O.v1), C->ir, static_cast<V *>(C->num));
        note_launch();
    }
    if (rc == GBC_OK) rc = finish_columns(ctx, ws, B, opt, nb, O.cnt, C);
    cudaEventRecord(ctx->ev[4], s);
    if (rc == GBC_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = fail(GBC_ECUDA, "learned spgemm failed");
    if (rc != GBC_OK) {
        gbc_result_free(C);
        return rc;
    }
    if (st) {
        float t04 = 0;
        cudaEventElapsedTime(&t04, ctx->ev[0], ctx->ev[4]);
        st->flops = O.flops;
        st->nnz = nnzc;
        st->overflow_cols = O.overflow_cols;
        st->alloc_entries = O.alloc;
        st->ms_total = t04;
        st->ms_symbolic = O.ms_predict;
        st->ms_numeric = O.ms_numeric + O.ms_rerun;
        st->tile_visits_dense = st->tile_visits_range = 0;
    }
    *Cout = C;
    return GBC_OK;
}

// Features and (optionally) exact counts of every stored column of B, the
// training data of the sizing model.
int spgemm_features(gbc_context *ctx, const gbc_matrix *Am, const gbc_matrix *Bm, float *feat_out,
                    int64_t *flop_out, int64_t *nnz_out, int where)
{
    if (!ctx || !Am || !Bm) return fail(GBC_EINVAL, "null argument");
    if (Am->ncol != Bm->nrow) return fail(GBC_EINVAL, "inner dimensions do not match");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    DevMatrix A, B;
    GBC_TRY(upload(ws, Am, GBC_F64, &A));
    GBC_TRY(upload(ws, Bm, GBC_F64, &B));
    Plan P;
    GBC_TRY(plan_build(ws, A, B, P));
    const int64_t nb = B.nzc;
    float *feat = nullptr;
    GBC_TRY(ws.alloc_n(&feat, (size_t)nb * kNF + 1));
    if (nb > 0) {
        k_features<<<grid_for(ctx, (nb + 7) / 8, 8), 256, 0, s>>>(P.a(), nb, feat);
        note_launch();
    }
    int64_t *cnt = nullptr;
    if (nnz_out) {
        GBC_TRY(ws.alloc_n(&cnt, nb + 1));
        Lists L;
        GBC_TRY(plan_classify(P, s, -1, 0, -1, L, cnt));
        GBC_TRY(run_symbolic(ctx, P, L, cnt));
    }
    cudaMemcpyKind k = where == GBC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (feat_out && nb) GBC_CUDA_TRY(cudaMemcpyAsync(feat_out, feat, (size_t)nb * kNF * sizeof(float), k, s));
    if (flop_out && nb) GBC_CUDA_TRY(cudaMemcpyAsync(flop_out, P.a().flop, nb * sizeof(int64_t), k, s));
    if (nnz_out && nb) GBC_CUDA_TRY(cudaMemcpyAsync(nnz_out, cnt, nb * sizeof(int64_t), k, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    return GBC_OK;
}

// MCL expansion step: C = A*A (PlusTimes fp32) then prune/select, with exact
// or learned sizing.  Learned sizing hands the select its slotted product
// directly (no compaction pass).
int mcl_select_device2(Context *ctx, int64_t nrow, int64_t n, const int64_t *cnt, const int32_t *flag,
                       const int64_t *beg0, const int64_t *ir0, const float *v0, const int64_t *beg1,
                       const int64_t *ir1, const float *v1, float thr, int64_t select, int64_t rnum, float rpct,
                       const int64_t *jc, gbc_result **out);

int mcl_expand(gbc_context *ctx, const gbc_matrix *Am, float thr, int64_t select, int64_t rnum, float rpct,
               int sizing, gbc_result **out, gbc_spgemm_stats *st)
{
    if (!ctx || !Am || !out) return fail(GBC_EINVAL, "null argument");
    if (Am->nrow != Am->ncol) return fail(GBC_EINVAL, "MCL needs a square matrix");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    DevMatrix A;
    GBC_TRY(upload(ws, Am, GBC_F32, &A));
    cudaEventRecord(ctx->ev[0], s);
    if (sizing == GBC_SIZING_LEARNED) {
        Plan P;
        LearnedOut O;
        GBC_TRY(learned_into_slots<PlusTimes<float>>(ctx, ws, A, A, P, O));
        int64_t *jc = nullptr;
        GBC_TRY(ws.alloc_n(&jc, O.nb + 1));
        if (O.nb > 0) {
            k_iota_jc<<<(unsigned)((O.nb + 255) / 256), 256, 0, s>>>(O.nb, A.jc, jc);
            note_launch();
        }
        GBC_TRY(mcl_select_device2(ctx, A.nrow, O.nb, O.cnt, O.flag, O.beg0, O.ir0, static_cast<const float *>(O.v0),
                                   O.beg1, O.ir1, static_cast<const float *>(O.v1), thr, select, rnum, rpct, jc,
                                   out));
        cudaEventRecord(ctx->ev[4], s);
        GBC_CUDA_TRY(cudaEventSynchronize(ctx->ev[4]));
        if (st) {
            float t = 0;
            cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[4]);
            st->flops = O.flops;
            st->nnz = (*out)->nnz;
            st->overflow_cols = O.overflow_cols;
            st->alloc_entries = O.alloc;
            st->ms_total = t;
            st->ms_symbolic = O.ms_predict;
            st->ms_numeric = O.ms_numeric + O.ms_rerun;
            st->tile_visits_dense = st->tile_visits_range = 0;
        }
        return GBC_OK;
    }
    gbc_result *C = nullptr;
    gbc_spgemm_opts opt{GBC_SIZING_EXACT, GBC_SORTED, 1, 0, -1, -1};
    gbc_spgemm_stats s1{};
    GBC_TRY(spgemm_exact<PlusTimes<float>>(ctx, A, A, opt, GBC_F32, &C, &s1));
    int rc = mcl_select_device2(ctx, C->nrow, C->nzc, nullptr, nullptr, C->cp, C->ir,
                                static_cast<const float *>(C->num), nullptr, nullptr, nullptr, thr, select, rnum, rpct,
                                C->jc, out);
    gbc_result_free(C);
    GBC_TRY(rc);
    cudaEventRecord(ctx->ev[4], s);
    GBC_CUDA_TRY(cudaEventSynchronize(ctx->ev[4]));
    if (st) {
        float t = 0;
        cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[4]);
        *st = s1;
        st->nnz = (*out)->nnz;
        st->ms_total = t;
    }
    return GBC_OK;
}

// ---------------------------------------------------------------- batches
// Many independent products in one plan: every pass is one launch per
// column class over all products' columns (work items name the product),
// and the symbolic + scan + numeric sequence is captured once into a CUDA
// graph that later runs replay.
struct Batch {
    Context *ctx = nullptr;
    Workspace *ws = nullptr;
    int sr = 0, vt = 0, np = 0;
    size_t vsize = 8;
    Plan P;
    Lists L;
    int64_t *cnt = nullptr, *ccp = nullptr, *ir = nullptr, *scan_tmp = nullptr;
    void *num = nullptr;
    int64_t nnz = 0;
    std::vector<int64_t> hccp;   // batch-wide column offsets (host copy)
    std::vector<int64_t> flops;  // per product
    std::function<int()> numeric;
    cudaGraphExec_t exec = nullptr;
    long long graph_kernels = 0;  // kernels one replay runs
};

static int batch_passes(Batch &b, bool with_symbolic)
{
    cudaStream_t s = b.ctx->stream;
    if (with_symbolic) {
        GBC_TRY(run_symbolic(b.ctx, b.P, b.L, b.cnt));
        GBC_TRY(exclusive_scan_i64_tmp(b.cnt, b.ccp, b.P.total_cols, b.scan_tmp, s));
    }
    return b.numeric();
}

template <class SR>
static int batch_build(Batch &b, const std::vector<DevMatrix> &A, const std::vector<DevMatrix> &B)
{
    Context *ctx = b.ctx;
    cudaStream_t s = ctx->stream;
    Workspace &ws = *b.ws;
    plan_fold<SR>(ctx, b.P);
    for (int p = 0; p < b.np; ++p) GBC_TRY(plan_add(ws, b.P, A[p], B[p]));
    GBC_TRY(plan_finalize(ws, b.P));
    const int64_t tc = b.P.total_cols;
    GBC_TRY(ws.alloc_n(&b.cnt, tc + 1));
    GBC_TRY(ws.alloc_n(&b.ccp, tc + 1));
    GBC_TRY(ws.alloc_n(&b.scan_tmp, scan_tmp_elems(tc) + 1));
    GBC_TRY(plan_classify(b.P, s, -1, 0, -1, b.L, b.cnt));
    GBC_TRY(run_symbolic(ctx, b.P, b.L, b.cnt));
    GBC_TRY(exclusive_scan_i64_tmp(b.cnt, b.ccp, tc, b.scan_tmp, s));
    GBC_TRY(read_i64(ctx, b.ccp + tc, &b.nnz));
    GBC_TRY(ws.alloc_n(&b.ir, b.nnz + 1));
    GBC_TRY(ws.alloc(&b.num, (b.nnz + 1) * sizeof(typename SR::V)));
    b.numeric = [&b]() { return run_numeric<SR>(b.ctx, b.P, b.L, b.ccp, 0, nullptr, nullptr, nullptr, b.ir, b.num); };
    GBC_TRY(b.numeric());
    GBC_TRY(check_err(ctx, b.P));
    b.hccp.resize(tc + 1);
    GBC_CUDA_TRY(cudaMemcpyAsync(b.hccp.data(), b.ccp, (tc + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    for (int p = 0; p < b.np; ++p) b.flops.push_back(sum_i64(ws, ctx, b.P.h[p].flop, b.P.h[p].nb));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    // capture symbolic + scan + numeric of the whole batch
    cudaGraph_t graph;
    const long long c0 = launch_count();
    GBC_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int rc = batch_passes(b, true);
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    b.graph_kernels = launch_count() - c0;
    note_launches(-b.graph_kernels);  // captured, not run
    if (rc != GBC_OK) return rc;
    if (e != cudaSuccess) return fail(GBC_ECUDA, std::string("batch capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(GBC_ECUDA, std::string("batch graph: ") + cudaGetErrorString(e));
    return GBC_OK;
}

template <class SR>
static int spgemm_entry(gbc_context *ctx, int vt, const gbc_matrix *Am, const gbc_matrix *Bm,
                        const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *st)
{
    if (!ctx || !C) return fail(GBC_EINVAL, "null context or output");
    *C = nullptr;
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    gbc_spgemm_opts opt{GBC_SIZING_EXACT, GBC_SORTED, 1, 0, -1, -1};
    if (opts) opt = *opts;
    if (Am && Bm && Am->ncol != Bm->nrow) return fail(GBC_EINVAL, "inner dimensions do not match");
    Workspace ws(ctx);
    DevMatrix A, B;
    GBC_TRY(upload(ws, Am, vt, &A));
    GBC_TRY(upload(ws, Bm, vt, &B));
    if (opt.sizing == GBC_SIZING_LEARNED) return spgemm_learned<SR>(ctx, A, B, opt, vt, C, st);
    return spgemm_exact<SR>(ctx, A, B, opt, vt, C, st);
}

// --------------------------------------------------------- colstats (API)
int spgemm_colstats(gbc_context *ctx, const gbc_matrix *Am, const gbc_matrix *Bm, int64_t *flop_out,
                    int64_t *nnz_out, int where)
{
    if (!ctx) return fail(GBC_EINVAL, "null context");
    if (Am->ncol != Bm->nrow) return fail(GBC_EINVAL, "inner dimensions do not match");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    DevMatrix A, B;
    GBC_TRY(upload(ws, Am, GBC_F64, &A));
    GBC_TRY(upload(ws, Bm, GBC_F64, &B));
    Plan P;
    GBC_TRY(plan_build(ws, A, B, P));
    int64_t nb = B.nzc;
    int64_t *cnt = nullptr;
    GBC_TRY(ws.alloc_n(&cnt, nb + 1));
    Lists L;
    GBC_TRY(plan_classify(P, s, -1, 0, -1, L, cnt));
    GBC_TRY(run_symbolic(ctx, P, L, cnt));
    cudaMemcpyKind k = where == GBC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (flop_out && nb) GBC_CUDA_TRY(cudaMemcpyAsync(flop_out, P.a().flop, nb * sizeof(int64_t), k, s));
    if (nnz_out && nb) GBC_CUDA_TRY(cudaMemcpyAsync(nnz_out, cnt, nb * sizeof(int64_t), k, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    return GBC_OK;
}

// ------------------------------------------------------- multiway merge
// Sum of K matrices of one shape, entries combined with SR::add in list
// order -- MultiwayMerge (MultiwayMerge.h:428-708) of the SpTuples that
// several SUMMA stages or phases produce for the same block.  It is the
// product [I I ... I] * [L_1; L_2; ...; L_K]: column j of the stacked right
// operand holds L_1(:,j), L_2(:,j) (rows + m), ... in that order, the left
// operand's column k*m + r is e_r with the semiring's multiplicative
// identity, so every output entry is the left fold over the lists in order,
// computed by the SpGEMM kernels.
__global__ void k_stack_counts(int nlists, const int64_t *const *dcp, int64_t n, int64_t *cnt)
{
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int64_t c = 0;
    for (int k = 0; k < nlists; ++k) c += dcp[k][j + 1] - dcp[k][j];
    cnt[j] = c;
}

template <typename V>
__global__ void k_stack_fill(int nlists, const int64_t *const *dcp, const int64_t *const *ir,
                             const void *const *num, V one, int64_t m, int64_t n, const int64_t *bcp, int64_t *bir,
                             V *bnum)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t j = warp; j < n; j += nwarps) {
        int64_t o = bcp[j];
        for (int k = 0; k < nlists; ++k) {
            const int64_t s0 = dcp[k][j], s1 = dcp[k][j + 1];
            const V *v = static_cast<const V *>(num[k]);
            for (int64_t p = s0 + lane; p < s1; p += 32) {
                bir[o + (p - s0)] = ir[k][p] + (int64_t)k * m;
                bnum[o + (p - s0)] = v ? v[p] : one;
            }
            o += s1 - s0;
        }
    }
}

template <typename V>
__global__ void k_identity_stack(int64_t m, int64_t cols, V unit, int64_t *cp, int64_t *ir, V *val)
{
    const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c < cols) {
        cp[c] = c;
        ir[c] = c % m;
        val[c] = unit;
    }
    if (c == cols) cp[c] = cols;
}

template <class SR>
static int multiway_merge(Context *ctx, int vt, int nlists, const gbc_matrix *lists, int64_t m, int64_t n,
                          gbc_result **out, gbc_spgemm_stats *st)
{
    typedef typename SR::V V;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    gbc_spgemm_opts opt{GBC_SIZING_EXACT, GBC_SORTED, 1, 0, -1, -1};
    if (nlists == 0 || m == 0 || n == 0) {  // an empty m x n product
        int64_t *z = nullptr;
        GBC_TRY(ws.alloc_n(&z, (size_t)n + 2));
        GBC_CUDA_TRY(cudaMemsetAsync(z, 0, (n + 2) * sizeof(int64_t), s));
        const DevMatrix A{m, 1, 1, 0, z, nullptr, z, nullptr};
        const DevMatrix B{1, n, n, 0, z, nullptr, z, nullptr};
        return spgemm_exact<SR>(ctx, A, B, opt, vt, out, st);
    }
    std::vector<const int64_t *> hdcp(nlists), hir(nlists);
    std::vector<const void *> hnum(nlists);
    for (int k = 0; k < nlists; ++k) {
        DevMatrix L;
        GBC_TRY(upload(ws, &lists[k], vt, &L));
        const int64_t *dcp = L.cp;
        if (L.jc) {
            int64_t *d = nullptr;
            GBC_TRY(ws.alloc_n(&d, n + 1));
            k_dense_colptr<<<(unsigned)((L.nzc + 1 + 255) / 256), 256, 0, s>>>(n, L.nzc, L.cp, L.jc, d);
            note_launch();
            dcp = d;
        }
        hdcp[k] = dcp;
        hir[k] = L.ir;
        hnum[k] = L.num;
    }
    const int64_t **ddcp = nullptr, **dir = nullptr;
    const void **dnum = nullptr;
    GBC_TRY(ws.alloc_n(&ddcp, nlists));
    GBC_TRY(ws.alloc_n(&dir, nlists));
    GBC_TRY(ws.alloc_n(&dnum, nlists));
    GBC_CUDA_TRY(cudaMemcpyAsync(ddcp, hdcp.data(), nlists * sizeof(void *), cudaMemcpyHostToDevice, s));
    GBC_CUDA_TRY(cudaMemcpyAsync(dir, hir.data(), nlists * sizeof(void *), cudaMemcpyHostToDevice, s));
    GBC_CUDA_TRY(cudaMemcpyAsync(dnum, hnum.data(), nlists * sizeof(void *), cudaMemcpyHostToDevice, s));
    int64_t *cnt = nullptr, *bcp = nullptr;
    GBC_TRY(ws.alloc_n(&cnt, n + 1));
    GBC_TRY(ws.alloc_n(&bcp, n + 1));
    k_stack_counts<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(nlists, ddcp, n, cnt);
    note_launch();
    GBC_TRY(exclusive_scan_i64(ws, cnt, bcp, n, s));
    int64_t total = 0;
    GBC_TRY(read_i64(ctx, bcp + n, &total));
    int64_t *bir = nullptr, *acp = nullptr, *air = nullptr;
    V *bnum = nullptr, *aval = nullptr;
    GBC_TRY(ws.alloc_n(&bir, total + 1));
    GBC_TRY(ws.alloc_n(&bnum, total + 1));
    k_stack_fill<V><<<grid_for(ctx, (n + 7) / 8, 8), 256, 0, s>>>(nlists, ddcp, dir, dnum, SR::one(), m, n, bcp, bir,
                                                                    bnum);
    note_launch();
    const int64_t cols = (int64_t)nlists * m;
    GBC_TRY(ws.alloc_n(&acp, cols + 1));
    GBC_TRY(ws.alloc_n(&air, cols + 1));
    GBC_TRY(ws.alloc_n(&aval, cols + 1));
    k_identity_stack<V><<<(unsigned)((cols + 1 + 255) / 256), 256, 0, s>>>(m, cols, SR::unit(), acp, air, aval);
    note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    const DevMatrix A{m, cols, cols, cols, acp, nullptr, air, aval};
    const DevMatrix B{cols, n, n, total, bcp, nullptr, bir, bnum};
    return spgemm_exact<SR>(ctx, A, B, opt, vt, out, st);
}

}  // namespace gbc

using namespace gbc;

extern "C" {

int gbc_spgemm(gbc_context *ctx, int sr, int vt, const gbc_matrix *A, const gbc_matrix *B,
               const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *st)
{
    switch (sr) {
        case GBC_SR_PLUSTIMES:
            if (vt == GBC_F64) return spgemm_entry<PlusTimes<double>>(ctx, vt, A, B, opts, C, st);
            if (vt == GBC_F32) return spgemm_entry<PlusTimes<float>>(ctx, vt, A, B, opts, C, st);
            if (vt == GBC_I64) return spgemm_entry<PlusTimes<int64_t>>(ctx, vt, A, B, opts, C, st);
            if (vt == GBC_BOOL) return spgemm_entry<BoolOrAnd>(ctx, vt, A, B, opts, C, st);
            break;
        case GBC_SR_BOOL:
            if (vt == GBC_BOOL) return spgemm_entry<BoolOrAnd>(ctx, vt, A, B, opts, C, st);
            break;
        case GBC_SR_MINPLUS:
            if (vt == GBC_F64) return spgemm_entry<MinPlus<double>>(ctx, vt, A, B, opts, C, st);
            if (vt == GBC_I64) return spgemm_entry<MinPlus<int64_t>>(ctx, vt, A, B, opts, C, st);
            break;
        case GBC_SR_SELECT2NDMIN:
            if (vt == GBC_I64) return spgemm_entry<Select2ndMin<int64_t>>(ctx, vt, A, B, opts, C, st);
            break;
        default: break;
    }
    return fail(GBC_EUNSUPPORTED, "semiring/value type combination not instantiated");
}

#define GBC_SPGEMM_INST(NAME, SR, VT)                                                                    \
    int NAME(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B, const gbc_spgemm_opts *opts,   \
             gbc_result **C, gbc_spgemm_stats *st)                                                        \
    {                                                                                                    \
        return gbc_spgemm(ctx, SR, VT, A, B, opts, C, st);                                               \
    }
GBC_SPGEMM_INST(gbc_spgemm_plustimes_f64_i64, GBC_SR_PLUSTIMES, GBC_F64)
GBC_SPGEMM_INST(gbc_spgemm_plustimes_f32_i64, GBC_SR_PLUSTIMES, GBC_F32)
GBC_SPGEMM_INST(gbc_spgemm_plustimes_i64_i64, GBC_SR_PLUSTIMES, GBC_I64)
GBC_SPGEMM_INST(gbc_spgemm_minplus_f64_i64, GBC_SR_MINPLUS, GBC_F64)
GBC_SPGEMM_INST(gbc_spgemm_minplus_i64_i64, GBC_SR_MINPLUS, GBC_I64)
GBC_SPGEMM_INST(gbc_spgemm_select2ndmin_i64_i64, GBC_SR_SELECT2NDMIN, GBC_I64)
GBC_SPGEMM_INST(gbc_spgemm_bool_i64, GBC_SR_BOOL, GBC_BOOL)

int gbc_spgemm_phased(gbc_context *ctx, int sr, int vt, const gbc_matrix *Am, const gbc_matrix *Bm,
                      int64_t max_phase_nnz, int sizing, gbc_phased_stats *st)
{
    if (!ctx) return fail(GBC_EINVAL, "null context");
    if (!Am || !Bm || Am->ncol != Bm->nrow) return fail(GBC_EINVAL, "inner dimensions do not match");
    if (max_phase_nnz <= 0) return fail(GBC_EINVAL, "phase budget must be positive");
    if (sizing != GBC_SIZING_EXACT && sizing != GBC_SIZING_LEARNED) return fail(GBC_EINVAL, "unknown sizing mode");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    Workspace ws(ctx);
    DevMatrix A, B;
    GBC_TRY(upload(ws, Am, vt, &A));
    GBC_TRY(upload(ws, Bm, vt, &B));
    if (sr == GBC_SR_PLUSTIMES && vt == GBC_F64) return spgemm_phased<PlusTimes<double>>(ctx, A, B, max_phase_nnz, sizing, st);
    if (sr == GBC_SR_PLUSTIMES && vt == GBC_F32) return spgemm_phased<PlusTimes<float>>(ctx, A, B, max_phase_nnz, sizing, st);
    if (sr == GBC_SR_SELECT2NDMIN && vt == GBC_I64)
        return spgemm_phased<Select2ndMin<int64_t>>(ctx, A, B, max_phase_nnz, sizing, st);
    return fail(GBC_EUNSUPPORTED, "phased SpGEMM is instantiated for PlusTimes f64/f32 and Select2ndMin i64");
}

struct gbc_batch : gbc::Batch {};

int gbc_batch_destroy(gbc_batch *b)
{
    if (!b) return GBC_OK;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    delete b->ws;
    cudaStreamSynchronize(b->ctx->stream);
    delete b;
    return GBC_OK;
}

int gbc_batch_create(gbc_context *ctx, int sr, int vt, int nprob, const gbc_matrix *A, const gbc_matrix *B,
                     int64_t s1, int64_t s2, gbc_batch **out)
{
    if (!ctx || !A || !B || !out || nprob <= 0) return fail(GBC_EINVAL, "bad argument");
    *out = nullptr;
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    gbc_batch *b = new gbc_batch();
    b->ctx = ctx;
    b->ws = new Workspace(ctx);
    b->sr = sr;
    b->vt = vt;
    b->np = nprob;
    b->vsize = value_size(vt);
    b->P.s1 = s1 >= 0 ? std::min<int64_t>(s1, kSmall1) : kSmall1;
    b->P.s2 = s2 >= 0 ? std::min<int64_t>(std::max(s2, b->P.s1), kSmall2) : GBC_SMALL2;
    b->P.s2_set = s2 >= 0;
    std::vector<DevMatrix> dA(nprob), dB(nprob);
    int rc = GBC_OK;
    for (int p = 0; p < nprob && rc == GBC_OK; ++p) {
        if (A[p].ncol != B[p].nrow) rc = fail(GBC_EINVAL, "inner dimensions do not match in a batch product");
        if (rc == GBC_OK) rc = upload(*b->ws, &A[p], vt, &dA[p]);
        if (rc == GBC_OK) rc = upload(*b->ws, &B[p], vt, &dB[p]);
    }
    if (rc == GBC_OK) {
        if (sr == GBC_SR_PLUSTIMES && vt == GBC_F64)
            rc = batch_build<PlusTimes<double>>(*b, dA, dB);
        else if (sr == GBC_SR_PLUSTIMES && vt == GBC_F32)
            rc = batch_build<PlusTimes<float>>(*b, dA, dB);
        else if (sr == GBC_SR_SELECT2NDMIN && vt == GBC_I64)
            rc = batch_build<Select2ndMin<int64_t>>(*b, dA, dB);
        else if ((sr == GBC_SR_BOOL || sr == GBC_SR_PLUSTIMES) && vt == GBC_BOOL)
            rc = batch_build<BoolOrAnd>(*b, dA, dB);
        else
            rc = fail(GBC_EUNSUPPORTED, "batched SpGEMM: semiring/type not instantiated");
    }
    if (rc != GBC_OK) {
        std::string msg = gbc_last_error();
        gbc_batch_destroy(b);
        return fail(rc, msg);
    }
    *out = b;
    return GBC_OK;
}

// Replay the whole batch (symbolic, scan, numeric of every product) as one
// CUDA graph launch; *ms = device time.
int gbc_batch_run(gbc_batch *b, double *ms)
{
    if (!b) return fail(GBC_EINVAL, "null batch");
    GBC_CUDA_TRY(cudaSetDevice(b->ctx->device));
    cudaStream_t s = b->ctx->stream;
    cudaEventRecord(b->ctx->ev[0], s);
    GBC_CUDA_TRY(cudaGraphLaunch(b->exec, s));
    note_launches(b->graph_kernels);
    cudaEventRecord(b->ctx->ev[1], s);
    GBC_CUDA_TRY(cudaEventSynchronize(b->ctx->ev[1]));
    GBC_TRY(check_err(b->ctx, b->P));
    if (ms) {
        float t = 0;
        cudaEventElapsedTime(&t, b->ctx->ev[0], b->ctx->ev[1]);
        *ms = t;
    }
    return GBC_OK;
}

int gbc_batch_info(const gbc_batch *b, int p, int64_t *nzc, int64_t *nnz, int64_t *flops)
{
    if (!b || p < 0 || p >= b->np) return fail(GBC_EINVAL, "bad batch index");
    const SpgemmArgs &a = b->P.h[p];
    if (nzc) *nzc = a.nb;
    if (nnz) *nnz = b->hccp[a.col_base + a.nb] - b->hccp[a.col_base];
    if (flops) *flops = b->flops[p];
    return GBC_OK;
}

__global__ void k_rebase(int64_t n, const int64_t *src, int64_t base, int64_t *dst)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i <= n) dst[i] = src[i] - base;
}

// Product p of the batch: cp[nzc+1] (one column per stored column of its B),
// ir[nnz], num[nnz], in host or device memory.
int gbc_batch_result(const gbc_batch *b, int p, int64_t *cp, int64_t *ir, void *num, int where)
{
    if (!b || p < 0 || p >= b->np) return fail(GBC_EINVAL, "bad batch index");
    GBC_CUDA_TRY(cudaSetDevice(b->ctx->device));
    cudaStream_t s = b->ctx->stream;
    const SpgemmArgs &a = b->P.h[p];
    const int64_t base = b->hccp[a.col_base], n = b->hccp[a.col_base + a.nb] - base;
    cudaMemcpyKind k = where == GBC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (cp) {
        if (where == GBC_DEVICE) {
            k_rebase<<<(unsigned)((a.nb + 256) / 256), 256, 0, s>>>(a.nb, b->ccp + a.col_base, base, cp);
            note_launch();
        } else {
            for (int64_t j = 0; j <= a.nb; ++j) cp[j] = b->hccp[a.col_base + j] - base;
        }
    }
    if (ir && n) GBC_CUDA_TRY(cudaMemcpyAsync(ir, b->ir + base, n * sizeof(int64_t), k, s));
    if (num && n)
        GBC_CUDA_TRY(cudaMemcpyAsync(num, static_cast<const char *>(b->num) + base * b->vsize, n * b->vsize, k, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    return GBC_OK;
}

int gbc_spgemm_features(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B, float *feat, int64_t *flop,
                        int64_t *nnz, int where)
{
    return spgemm_features(ctx, A, B, feat, flop, nnz, where);
}

int gbc_context_set_mlp(gbc_context *ctx, gbc_mlp *m)
{
    if (!ctx) return fail(GBC_EINVAL, "null context");
    ctx->mlp = m;
    return GBC_OK;
}

int gbc_mcl_expand_f32(gbc_context *ctx, const gbc_matrix *A, float thr, int64_t select, int sizing, gbc_result **out,
                       gbc_spgemm_stats *st)
{
    return mcl_expand(ctx, A, thr, select, 0, 0.0f, sizing, out, st);
}

int gbc_mcl_expand_recover_f32(gbc_context *ctx, const gbc_matrix *A, float thr, int64_t select, int64_t recover_num,
                               float recover_pct, int sizing, gbc_result **out, gbc_spgemm_stats *st)
{
    return mcl_expand(ctx, A, thr, select, recover_num, recover_pct, sizing, out, st);
}

int gbc_spgemm_colstats(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B, int64_t *flop, int64_t *nnz,
                        int where)
{
    return spgemm_colstats(ctx, A, B, flop, nnz, where);
}

int gbc_multiway_merge(gbc_context *ctx, int sr, int vt, int nlists, const gbc_matrix *lists, int64_t nrow,
                       int64_t ncol, gbc_result **C, gbc_spgemm_stats *st)
{
    if (!ctx || !C || (nlists > 0 && !lists) || nlists < 0) return fail(GBC_EINVAL, "null or bad argument");
    *C = nullptr;
    for (int k = 0; k < nlists; ++k)
        if (lists[k].nrow != nrow || lists[k].ncol != ncol)
            return fail(GBC_EINVAL, "dimensions of the merged matrices do not match");
    if ((int64_t)nlists * nrow >= (int64_t(1) << 31)) return fail(GBC_EOVERFLOW, "lists x rows must be below 2^31");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    switch (sr) {
        case GBC_SR_PLUSTIMES:
            if (vt == GBC_F64) return multiway_merge<PlusTimes<double>>(ctx, vt, nlists, lists, nrow, ncol, C, st);
            if (vt == GBC_F32) return multiway_merge<PlusTimes<float>>(ctx, vt, nlists, lists, nrow, ncol, C, st);
            if (vt == GBC_I64) return multiway_merge<PlusTimes<int64_t>>(ctx, vt, nlists, lists, nrow, ncol, C, st);
            if (vt == GBC_BOOL) return multiway_merge<BoolOrAnd>(ctx, vt, nlists, lists, nrow, ncol, C, st);
            break;
        case GBC_SR_BOOL:
            if (vt == GBC_BOOL) return multiway_merge<BoolOrAnd>(ctx, vt, nlists, lists, nrow, ncol, C, st);
            break;
        case GBC_SR_MINPLUS:
            if (vt == GBC_F64) return multiway_merge<MinPlus<double>>(ctx, vt, nlists, lists, nrow, ncol, C, st);
            if (vt == GBC_I64) return multiway_merge<MinPlus<int64_t>>(ctx, vt, nlists, lists, nrow, ncol, C, st);
            break;
        case GBC_SR_SELECT2NDMIN:
            if (vt == GBC_I64)
                return multiway_merge<Select2ndMin<int64_t>>(ctx, vt, nlists, lists, nrow, ncol, C, st);
            break;
        default: break;
    }
    return fail(GBC_EUNSUPPORTED, "semiring/value type combination not instantiated");
}

}  // extern "C"
