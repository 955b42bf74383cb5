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
//                 shared memory, stably partitioned to owner warps (rows are
//                 striped over warps in 32-row groups), and folded by the
//                 owner into a dense shared-memory accumulator in B-entry
//                 order.  Each output entry is therefore the left fold
//                 acc = add(mrhs, acc) over k ascending -- exactly the order
//                 of the reference's hash path (mtSpGEMM.h:385-400) -- so
//                 repeated runs are bit-identical.  Rows come out ascending
//                 (tile order, then bitmap order): no sort is needed.
#include <algorithm>
#include <cstdio>

#include "gbc_internal.cuh"
#include "semiring.cuh"
#include "spgemm_kernels.cuh"

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

// flop[i] = sum over B(:,i) entries k of nnz(A(:,k)).
__global__ void k_flop(int64_t nb, const int64_t *bcp, const int32_t *brow, const int64_t *acp, int64_t *flop)
{
    int lane = threadIdx.x & 31;
    int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp; i < nb; i += nwarps) {
        int64_t f = 0;
        for (int64_t p = bcp[i] + lane; p < bcp[i + 1]; p += 32) {
            int k = brow[p];
            f += acp[k + 1] - acp[k];
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
        if (lane == 0) flop[i] = f;
    }
}

// ---------------------------------------------------------------- symbolic
// One block per column (dynamic work counter).  Bitmap over a super-tile of
// SR rows (a whole number of R-row tiles); products set bits; the column's
// count is the popcount and each R-tile with a set bit is marked in the
// column's tile mask (mask words of 64 tiles).
__global__ void __launch_bounds__(kThreads) k_symbolic(SpgemmArgs a, int64_t *cnt, uint64_t *tmask,
                                                       int sup_rows, unsigned long long *work)
{
    extern __shared__ uint32_t bm[];
    __shared__ ChunkSmem ch;
    __shared__ int64_t s_col;
    __shared__ uint32_t s_tmask[kMaxMaskWords * 2];
    __shared__ int64_t s_red[kThreads / 32];
    const int tid = threadIdx.x;
    const int tiles_per_sup = sup_rows / a.R;
    for (;;) {
        if (tid == 0) s_col = (int64_t)atomicAdd(work, 1ull);
        __syncthreads();
        int64_t i = s_col;
        __syncthreads();
        if (i >= a.nb) break;
        int64_t bs = a.bcp[i], be = a.bcp[i + 1];
        for (int w = tid; w < a.mask_words * 2; w += kThreads) s_tmask[w] = 0;
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
                    int L = load_chunk(a, ch, cb, be, t0, t1, false, nullptr);
                    for (int j = tid; j < L; j += kThreads) {
                        int b = chunk_find(ch, j);
                        int64_t idx = ch.s[b] + (j - ch.off[b]);
                        int r = a.arow[idx] - (int)row0;
                        atomicOr(&bm[r >> 5], 1u << (r & 31));
                    }
                    __syncthreads();
                }
                // count and per-tile occupancy
                int64_t c = 0;
                int wpt = a.R >> 5;  // words per tile
                for (int w = tid; w < words; w += kThreads) {
                    uint32_t x = bm[w];
                    if (x) {
                        c += __popc(x);
                        int t = t0 + w / wpt;
                        atomicOr(&s_tmask[t >> 5], 1u << (t & 31));
                    }
                }
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
            cnt[i] = s;
        }
        for (int w = tid; w < a.mask_words; w += kThreads)
            tmask[i * a.mask_words + w] = (uint64_t)s_tmask[2 * w] | ((uint64_t)s_tmask[2 * w + 1] << 32);
        __syncthreads();
    }
}

// ----------------------------------------------------------------- numeric
// One block per column (dynamic counter); for every row tile t the column
// touches:
//  * dense accumulator acc[R] and touched bitmap in shared memory;
//  * the column's B entries are walked in chunks of kThreads; the chunk's A
//    segments restricted to tile t form a flattened product list, processed
//    in sub-batches of kSub products.  Segment ids of a sub-batch come from a
//    block max-scan over segment-start markers;
//  * staging: all threads load the sub-batch's rows and values with
//    coalesced reads (one load per product), multiply by B(k,j) and store
//    them to shared memory in flattened (k-major) order;
//  * folding: every warp walks every 32-product window of the staged list
//    but folds only the rows of its 32-row stripes (stripe mod kWarps), in
//    window order.  A window inside one A segment has distinct rows; a
//    window spanning segments groups equal rows with __match_any_sync and the
//    lowest lane folds the group in lane order.  Each output entry is thus
//    the left fold acc = add(mrhs, acc) over k ascending.
constexpr int kSub = 4096;
constexpr int kSubPerThread = kSub / kThreads;

// Inclusive max-scan of seg[0..n) (uint8 segment-start markers, 0 where no
// segment starts) seeded with `seed`: seg[j] = id of the segment holding j.
__device__ __forceinline__ void seg_max_scan(uint8_t *seg, int seed)
{
    __shared__ int ws[kWarps];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint8_t loc[kSubPerThread];
    *reinterpret_cast<uint4 *>(loc) = *reinterpret_cast<const uint4 *>(seg + tid * kSubPerThread);
    int run = 0;
#pragma unroll
    for (int u = 0; u < kSubPerThread; ++u) run = max(run, (int)loc[u]);
    int x = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x = max(x, y);
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    int pre = seed;
    for (int w = 0; w < wid; ++w) pre = max(pre, ws[w]);
    int excl = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane > 0) pre = max(pre, excl);
    int cur = pre;
#pragma unroll
    for (int u = 0; u < kSubPerThread; ++u) {
        cur = max(cur, (int)loc[u]);
        loc[u] = (uint8_t)cur;
    }
    *reinterpret_cast<uint4 *>(seg + tid * kSubPerThread) = *reinterpret_cast<const uint4 *>(loc);
    __syncthreads();
}

template <class SR>
__global__ void __launch_bounds__(kThreads, 1) k_numeric(SpgemmArgs a, const void *aval_v, const void *bval_v,
                                                         const uint64_t *tmask, const int64_t *ccp, int64_t *cir,
                                                         void *cval_v, unsigned long long *work)
{
    typedef typename SR::V V;
    extern __shared__ __align__(16) unsigned char smem[];
    V *acc = reinterpret_cast<V *>(smem);                            // [R]
    V *sval = acc + a.R;                                             // [kSub]
    uint32_t *bm = reinterpret_cast<uint32_t *>(sval + kSub);        // [R/32]
    uint16_t *srow = reinterpret_cast<uint16_t *>(bm + (a.R >> 5));  // [kSub]
    uint8_t *seg = reinterpret_cast<uint8_t *>(srow + kSub);         // [kSub]
    __shared__ ChunkSmem ch;
    __shared__ V ch_bv[kThreads];
    __shared__ int32_t s_cnt[kWarps * kSubPerThread * kWarps + 1];  // [owner][round][warp]
    __shared__ int64_t s_col;
    const V *aval = static_cast<const V *>(aval_v);
    const V *bval = static_cast<const V *>(bval_v);
    V *cval = static_cast<V *>(cval_v);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1;
    const int words = a.R >> 5;
    constexpr int NC = kWarps * kSubPerThread * kWarps;

    for (;;) {
        if (tid == 0) s_col = a.col_begin + (int64_t)atomicAdd(work, 1ull);
        __syncthreads();
        const int64_t i = s_col;
        __syncthreads();
        if (i >= a.col_end) break;
        const int64_t bs = a.bcp[i], be = a.bcp[i + 1];
        // ccp is indexed relative to the first column of this pass
        int64_t out = ccp[i - a.col_begin];
        const int64_t lim = ccp[i - a.col_begin + 1];
        for (int mw = 0; mw < a.mask_words; ++mw) {
            uint64_t msk = tmask[i * a.mask_words + mw];
            while (msk) {
                const int t = mw * 64 + __ffsll((long long)msk) - 1;
                msk &= msk - 1;
                const int row0 = t * a.R;
                for (int w = tid; w < words; w += kThreads) bm[w] = 0;
                __syncthreads();
                for (int64_t cb = bs; cb < be; cb += kThreads) {
                    const int L = load_chunk<V>(a, ch, cb, be, t, t + 1, bval, ch_bv, SR::one());
                    const int myoff = ch.off[tid], mylen = ch.off[tid + 1] - myoff;
                    for (int q = 0; q < L; q += kSub) {
                        const int n = min(kSub, L - q);
                        // 1. segment ids of products q .. q+n-1
                        *reinterpret_cast<uint4 *>(seg + tid * kSubPerThread) = make_uint4(0, 0, 0, 0);
                        __syncthreads();
                        if (mylen > 0 && myoff >= q && myoff < q + n) seg[myoff - q] = (uint8_t)tid;
                        __syncthreads();
                        seg_max_scan(seg, chunk_find(ch, q));
                        // 2. load (round-major, all loads in flight), owner = 32-row stripe mod kWarps
                        int o_[kSubPerThread];
                        V v_[kSubPerThread];
#pragma unroll
                        for (int r = 0; r < kSubPerThread; ++r) {
                            const int j = r * kThreads + tid;
                            o_[r] = -1;
                            if (j < n) {
                                const int b = seg[j];
                                const int64_t idx = (int64_t)ch.s[b] + (q + j - ch.off[b]);
                                o_[r] = a.arow[idx] - row0;
                                const V av = aval ? aval[idx] : SR::one();
                                v_[r] = SR::mul(av, ch_bv[b]);
                            }
                        }
                        // 3. stable partition by owner: rank within (round, warp) from 3 ballots
                        int rk_[kSubPerThread];
#pragma unroll
                        for (int r = 0; r < kSubPerThread; ++r) {
                            const bool act = o_[r] >= 0;
                            const int w = (o_[r] >> 5) & (kWarps - 1);
                            const unsigned va = __ballot_sync(0xffffffffu, act);
                            const unsigned b0 = __ballot_sync(0xffffffffu, act && (w & 1));
                            const unsigned b1 = __ballot_sync(0xffffffffu, act && (w & 2));
                            const unsigned b2 = __ballot_sync(0xffffffffu, act && (w & 4));
                            const unsigned same = va & ((w & 1) ? b0 : ~b0) & ((w & 2) ? b1 : ~b1) & ((w & 4) ? b2 : ~b2);
                            rk_[r] = __popc(same & lt);
                            // lanes 0..kWarps-1 publish the size of owner `lane`'s group (0 if absent)
                            if (lane < kWarps) {
                                const unsigned sl = va & ((lane & 1) ? b0 : ~b0) & ((lane & 2) ? b1 : ~b1) &
                                                    ((lane & 4) ? b2 : ~b2);
                                s_cnt[(lane * kSubPerThread + r) * kWarps + warp] = __popc(sl);
                            }
                        }
                        __syncthreads();
                        // 4. exclusive scan of the (owner, round, warp) counts
                        {
                            constexpr int PER = (NC + kThreads - 1) / kThreads;
                            int loc[PER];
                            int sum = 0;
#pragma unroll
                            for (int u = 0; u < PER; ++u) {
                                loc[u] = s_cnt[tid * PER + u];
                                sum += loc[u];
                            }
                            int64_t tot64;
                            int base = (int)block_exclusive_sum64(sum, &tot64);
#pragma unroll
                            for (int u = 0; u < PER; ++u) {
                                s_cnt[tid * PER + u] = base;
                                base += loc[u];
                            }
                            if (tid == 0) s_cnt[NC] = (int)tot64;
                        }
                        __syncthreads();
                        // 5. scatter into owner buckets
#pragma unroll
                        for (int r = 0; r < kSubPerThread; ++r) {
                            if (o_[r] >= 0) {
                                const int w = (o_[r] >> 5) & (kWarps - 1);
                                const int pos = s_cnt[(w * kSubPerThread + r) * kWarps + warp] + rk_[r];
                                srow[pos] = (uint16_t)o_[r];
                                sval[pos] = v_[r];
                            }
                        }
                        __syncthreads();
                        // 6. each warp folds its bucket in staging (= k) order
                        {
                            const int beg = s_cnt[(warp * kSubPerThread) * kWarps];
                            const int end = s_cnt[((warp + 1) * kSubPerThread) * kWarps];
                            for (int p0 = beg; p0 < end; p0 += 32) {
                                const int p = p0 + lane;
                                const bool act = p < end;
                                const int o = act ? (int)srow[p] : (0x10000 + lane);
                                const unsigned grp = __match_any_sync(0xffffffffu, o);
                                if (act && (grp & lt) == 0) {
                                    const uint32_t bit = 1u << (o & 31);
                                    const bool touched = (bm[o >> 5] & bit) != 0;
                                    V cur = touched ? SR::add(sval[p], acc[o]) : sval[p];
                                    unsigned rest = grp & ~(1u << lane);
                                    while (rest) {
                                        const int m = __ffs(rest) - 1;
                                        rest &= rest - 1;
                                        cur = SR::add(sval[p0 + m], cur);
                                    }
                                    acc[o] = cur;
                                    if (!touched) atomicOr(&bm[o >> 5], bit);
                                }
                                __syncwarp();
                            }
                        }
                        __syncthreads();
                    }
                }
                // write the tile's entries in row order: warp-cooperative over
                // 32-word groups so stores stay contiguous
                {
                    int wl = 0;
                    const int wpt = (words + kThreads - 1) / kThreads;
                    const int w0 = min(words, tid * wpt), w1 = min(words, (tid + 1) * wpt);
                    for (int w = w0; w < w1; ++w) wl += __popc(bm[w]);
                    int64_t tot;
                    int64_t pos = out + block_exclusive_sum64(wl, &tot);
                    for (int w = w0; w < w1; ++w) {
                        uint32_t x = bm[w];
                        while (x) {
                            const int bit = __ffs(x) - 1;
                            x &= x - 1;
                            const int o = w * 32 + bit;
                            if (pos < lim) {
                                cir[pos] = (int64_t)row0 + o;
                                cval[pos] = acc[o];
                            } else {
                                atomicOr(a.err, 128);  // count mismatch: never write past the column
                            }
                            ++pos;
                        }
                    }
                    out += tot;
                }
                __syncthreads();
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

int prepare_operands(Workspace &ws, const DevMatrix &A, const DevMatrix &B, SpgemmArgs &a, int64_t **acp_out)
{
    Context *ctx = ws.ctx;
    cudaStream_t s = ctx->stream;
    a.m = A.nrow;
    a.kdim = A.ncol;
    a.n = B.ncol;
    a.nb = B.nzc;
    a.R = std::min<int64_t>(kTileRows, ((A.nrow + kThreads - 1) / kThreads) * kThreads);
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
        k_dense_colptr<<<(unsigned)((A.nzc + 1 + 255) / 256), 256, 0, s>>>(A.ncol, A.nzc, A.cp, A.jc, acp); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    } else {
        acp = const_cast<int64_t *>(A.cp);
    }
    if (A.nzc > 0) {
        k_prep_a<<<grid_for(ctx, (A.nzc + 7) / 8, 8), 256, 0, s>>>(A.ncol, A.nrow, A.cp, A.jc, A.nzc, A.nnz,
                                                                     A.ir, arow, tptr, a.T, a.R, err); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    if (A.ncol > 0) {
        k_fill_empty_tptr<<<(unsigned)((A.ncol + 255) / 256), 256, 0, s>>>(A.ncol, acp, tptr, a.T); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    int32_t *brow = nullptr;
    GBC_TRY(ws.alloc_n(&brow, B.nnz + 1));
    if (B.nzc > 0) {
        k_prep_b<<<grid_for(ctx, (B.nzc + 7) / 8, 8), 256, 0, s>>>(B.nzc, B.nnz, B.cp, B.ir, A.ncol, brow, err); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    int32_t herr[4];
    GBC_CUDA_TRY(cudaMemcpyAsync(herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr[0]) {
        char buf[160];
        snprintf(buf, sizeof buf, "malformed input matrix (code 0x%x): %s%s%s", herr[0],
                 (herr[0] & 0x15) ? "bad column pointers or ids; " : "",
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
    *acp_out = acp;
    return GBC_OK;
}

template <class SR>
static int spgemm_exact(Context *ctx, const DevMatrix &A, const DevMatrix &B, const gbc_spgemm_opts &opt, int vt,
                        gbc_result **Cout, gbc_spgemm_stats *st)
{
    typedef typename SR::V V;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    cudaEventRecord(ctx->ev[0], s);
    SpgemmArgs a{};
    int64_t *acp = nullptr;
    GBC_TRY(prepare_operands(ws, A, B, a, &acp));
    const int64_t nb = B.nzc;
    int64_t *flop = nullptr, *cnt = nullptr, *ccp = nullptr;
    uint64_t *tmask = nullptr;
    unsigned long long *work = nullptr;
    GBC_TRY(ws.alloc_n(&flop, nb + 1));
    GBC_TRY(ws.alloc_n(&cnt, nb + 1));
    GBC_TRY(ws.alloc_n(&tmask, (size_t)nb * a.mask_words + 1));
    GBC_TRY(ws.alloc_n(&work, 8));
    GBC_CUDA_TRY(cudaMemsetAsync(work, 0, 8 * sizeof(unsigned long long), s));
    a.flop = flop;
    a.col_begin = 0;
    a.col_end = nb;
    if (nb > 0) {
        k_flop<<<grid_for(ctx, (nb + 7) / 8, 8), 256, 0, s>>>(nb, B.cp, a.brow, acp, flop); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    // symbolic
    int sup_rows = (int)std::min<int64_t>((int64_t)kSymRows, (int64_t)a.T * a.R);
    sup_rows = (sup_rows / a.R) * a.R;
    size_t sym_smem = (size_t)sup_rows / 8;
    cudaEventRecord(ctx->ev[1], s);
    if (nb > 0) {
        GBC_CUDA_TRY(cudaFuncSetAttribute(k_symbolic, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sym_smem));
        int per_sm = std::max(1, (int)(ctx->smem_optin / (sym_smem + 8192)));
        k_symbolic<<<grid_for(ctx, nb, std::min(per_sm, 8)), kThreads, sym_smem, s>>>(a, cnt, tmask, sup_rows,
                                                                                          work); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    GBC_TRY(device_alloc(ctx, (void **)&ccp, (nb + 1) * sizeof(int64_t)));
    int rc = exclusive_scan_i64(ws, cnt, ccp, nb, s);
    if (rc != GBC_OK) {
        device_free(ctx, ccp);
        return rc;
    }
    int64_t nnzc = 0;
    rc = read_i64(ctx, ccp + nb, &nnzc);
    if (rc != GBC_OK) {
        device_free(ctx, ccp);
        return rc;
    }
    cudaEventRecord(ctx->ev[2], s);
    // numeric
    gbc_result *C = new gbc_result();
    C->ctx = ctx;
    C->nrow = A.nrow;
    C->ncol = B.ncol;
    C->valtype = vt;
    C->nnz = nnzc;
    C->cp = ccp;
    rc = device_alloc(ctx, (void **)&C->ir, (nnzc + 1) * sizeof(int64_t));
    if (rc == GBC_OK) rc = device_alloc(ctx, &C->num, (nnzc + 1) * sizeof(V));
    if (rc != GBC_OK) {
        gbc_result_free(C);
        return rc;
    }
    if (nb > 0 && nnzc > 0) {
        size_t num_smem = numeric_smem_bytes(a.R, sizeof(V));
        GBC_CUDA_TRY(cudaFuncSetAttribute(k_numeric<SR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)num_smem));
        int per_sm = std::max(1, (int)(ctx->smem_optin / (num_smem + 12288)));
        k_numeric<SR><<<grid_for(ctx, nb, std::min(per_sm, 8)), kThreads, num_smem, s>>>(
            a, A.num, B.num, tmask, ccp, C->ir, C->num, work + 2); ::gbc::note_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            gbc_result_free(C);
            return fail(GBC_ECUDA, std::string("k_numeric launch: ") + cudaGetErrorString(e));
        }
    }
    cudaEventRecord(ctx->ev[3], s);
    // column ids / empty-column compaction
    if (opt.keep_empty || nb == 0) {
        C->nzc = nb;
        rc = device_alloc(ctx, (void **)&C->jc, (nb + 1) * sizeof(int64_t));
        if (rc != GBC_OK) {
            gbc_result_free(C);
            return rc;
        }
        if (nb > 0) k_iota_jc<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, B.jc, C->jc); ::gbc::note_launch();
    } else {
        int64_t *flags = nullptr;
        GBC_TRY(ws.alloc_n(&flags, nb + 1));
        k_nonempty_flags<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, cnt, flags); ::gbc::note_launch();
        GBC_TRY(exclusive_scan_i64(ws, flags, flags, nb, s));
        int64_t nzc = 0;
        GBC_TRY(read_i64(ctx, flags + nb, &nzc));
        int64_t *cp2 = nullptr, *jc2 = nullptr;
        rc = device_alloc(ctx, (void **)&cp2, (nzc + 1) * sizeof(int64_t));
        if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&jc2, (nzc + 1) * sizeof(int64_t));
        if (rc != GBC_OK) {
            device_free(ctx, cp2);
            gbc_result_free(C);
            return rc;
        }
        GBC_CUDA_TRY(cudaMemsetAsync(cp2, 0, sizeof(int64_t), s));
        k_compact_cols<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, cnt, flags, ccp, B.jc, cp2, jc2); ::gbc::note_launch();
        device_free(ctx, C->cp);
        C->cp = cp2;
        C->jc = jc2;
        C->nzc = nzc;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        gbc_result_free(C);
        return fail(GBC_ECUDA, std::string("spgemm: ") + cudaGetErrorString(e));
    }
    cudaEventRecord(ctx->ev[4], s);
    {
        int32_t herr = 0;
        GBC_CUDA_TRY(cudaMemcpyAsync(&herr, a.err, sizeof(herr), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
        if (herr) {
            gbc_result_free(C);
            return fail(GBC_ECUDA, "internal error: numeric and symbolic counts disagree");
        }
    }
    if (st) {
        // flop total
        int64_t *fsum = nullptr;
        GBC_TRY(ws.alloc_n(&fsum, nb + 1));
        GBC_TRY(exclusive_scan_i64(ws, flop, fsum, nb, s));
        GBC_TRY(read_i64(ctx, fsum + nb, &st->flops));
        st->nnz = nnzc;
        st->overflow_cols = 0;
        st->alloc_entries = nnzc;
        float t01 = 0, t13 = 0, t04 = 0, t23 = 0;
        cudaEventElapsedTime(&t04, ctx->ev[0], ctx->ev[4]);
        cudaEventElapsedTime(&t01, ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&t23, ctx->ev[2], ctx->ev[3]);
        (void)t13;
        st->ms_total = t04;
        st->ms_symbolic = t01;
        st->ms_numeric = t23;
    }
    *Cout = C;
    return GBC_OK;
}


// ------------------------------------------------------- column phases
// Deterministic checksums of one phase's output: block partial sums over
// contiguous ranges (fixed grid), combined in block order on the host.
template <typename V>
__global__ void k_phase_checksum(const int64_t *ir, const V *num, int64_t nnz, int64_t *rsum, double *vsum)
{
    __shared__ double sv[kWarps];
    __shared__ long long sr[kWarps];
    const int64_t per = (nnz + gridDim.x - 1) / gridDim.x;
    const int64_t b0 = min(nnz, per * blockIdx.x), b1 = min(nnz, b0 + per);
    double v = 0;
    long long r = 0;
    for (int64_t p = b0 + threadIdx.x; p < b1; p += blockDim.x) {
        v += (double)num[p];
        r += ir[p];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, o);
        r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sv[threadIdx.x >> 5] = v;
        sr[threadIdx.x >> 5] = r;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tv = 0;
        long long tr = 0;
        for (int w = 0; w < kWarps; ++w) {
            tv += sv[w];
            tr += sr[w];
        }
        vsum[blockIdx.x] = tv;
        rsum[blockIdx.x] = tr;
    }
}

// C = A*B computed in phases of B's stored columns so that each phase's
// output holds at most max_phase_nnz entries -- the reference's column
// phases of MemEfficientSpGEMM (ParFriends.h:553-556, ColSplit).  Each
// phase's C is written to HBM and reduced to checksums; nothing is kept.
template <class SR>
static int spgemm_phased(Context *ctx, const DevMatrix &A, const DevMatrix &B, int64_t max_phase_nnz,
                         gbc_phased_stats *st)
{
    typedef typename SR::V V;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    cudaEventRecord(ctx->ev[0], s);
    SpgemmArgs a{};
    int64_t *acp = nullptr;
    GBC_TRY(prepare_operands(ws, A, B, a, &acp));
    const int64_t nb = B.nzc;
    int64_t *flop = nullptr, *cnt = nullptr, *fsum = nullptr;
    uint64_t *tmask = nullptr;
    unsigned long long *work = nullptr;
    GBC_TRY(ws.alloc_n(&flop, nb + 1));
    GBC_TRY(ws.alloc_n(&fsum, nb + 1));
    GBC_TRY(ws.alloc_n(&cnt, nb + 1));
    GBC_TRY(ws.alloc_n(&tmask, (size_t)nb * a.mask_words + 1));
    GBC_TRY(ws.alloc_n(&work, 8));
    GBC_CUDA_TRY(cudaMemsetAsync(work, 0, 8 * sizeof(unsigned long long), s));
    a.flop = flop;
    if (nb > 0) {
        k_flop<<<grid_for(ctx, (nb + 7) / 8, 8), 256, 0, s>>>(nb, B.cp, a.brow, acp, flop); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    int sup_rows = (int)std::min<int64_t>((int64_t)kSymRows, (int64_t)a.T * a.R);
    sup_rows = (sup_rows / a.R) * a.R;
    size_t sym_smem = (size_t)sup_rows / 8;
    cudaEventRecord(ctx->ev[1], s);
    if (nb > 0) {
        GBC_CUDA_TRY(cudaFuncSetAttribute(k_symbolic, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sym_smem));
        int per_sm = std::max(1, (int)(ctx->smem_optin / (sym_smem + 8192)));
        k_symbolic<<<grid_for(ctx, nb, std::min(per_sm, 8)), kThreads, sym_smem, s>>>(a, cnt, tmask, sup_rows,
                                                                                          work); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    cudaEventRecord(ctx->ev[2], s);
    std::vector<int64_t> hcnt(nb > 0 ? nb : 1);
    if (nb > 0) GBC_CUDA_TRY(cudaMemcpyAsync(hcnt.data(), cnt, nb * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GBC_TRY(exclusive_scan_i64(ws, flop, fsum, nb, s));
    int64_t flops = 0;
    GBC_TRY(read_i64(ctx, fsum + nb, &flops));
    // phase boundaries (greedy, a column bigger than the budget is alone)
    std::vector<int64_t> bounds{0};
    int64_t acc = 0, maxp = 0, total = 0;
    for (int64_t j = 0; j < nb; ++j) {
        if (acc > 0 && acc + hcnt[j] > max_phase_nnz) {
            bounds.push_back(j);
            maxp = std::max(maxp, acc);
            acc = 0;
        }
        acc += hcnt[j];
        total += hcnt[j];
    }
    maxp = std::max(maxp, acc);
    if (bounds.back() != nb) bounds.push_back(nb);
    int64_t maxcols = 0;
    for (size_t p = 0; p + 1 < bounds.size(); ++p) maxcols = std::max(maxcols, bounds[p + 1] - bounds[p]);
    int64_t *ir = nullptr, *ccp = nullptr, *rsum = nullptr;
    V *num = nullptr;
    double *vsum = nullptr;
    const int csb = ctx->num_sms * 2;
    GBC_TRY(ws.alloc_n(&ir, maxp + 1));
    GBC_TRY(ws.alloc_n(&num, maxp + 1));
    GBC_TRY(ws.alloc_n(&ccp, maxcols + 1));
    GBC_TRY(ws.alloc_n(&rsum, (size_t)csb * (bounds.size() + 1)));
    GBC_TRY(ws.alloc_n(&vsum, (size_t)csb * (bounds.size() + 1)));
    size_t num_smem = numeric_smem_bytes(a.R, sizeof(V));
    GBC_CUDA_TRY(cudaFuncSetAttribute(k_numeric<SR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)num_smem));
    int per_sm = std::max(1, (int)(ctx->smem_optin / (num_smem + 12288)));
    double ms_num = 0;
    const int np = (int)bounds.size() - 1;
    for (int p = 0; p < np; ++p) {
        const int64_t j0 = bounds[p], j1 = bounds[p + 1];
        GBC_TRY(exclusive_scan_i64(ws, cnt + j0, ccp, j1 - j0, s));
        GBC_CUDA_TRY(cudaMemsetAsync(work + 2, 0, sizeof(unsigned long long), s));
        a.col_begin = j0;
        a.col_end = j1;
        cudaEventRecord(ctx->ev[5], s);
        k_numeric<SR><<<grid_for(ctx, j1 - j0, std::min(per_sm, 8)), kThreads, num_smem, s>>>(
            a, A.num, B.num, tmask, ccp, ir, num, work + 2); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
        cudaEventRecord(ctx->ev[6], s);
        int64_t pn = 0;
        for (int64_t j = j0; j < j1; ++j) pn += hcnt[j];
        k_phase_checksum<V><<<csb, kThreads, 0, s>>>(ir, num, pn, rsum + (size_t)p * csb, vsum + (size_t)p * csb); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
        GBC_CUDA_TRY(cudaEventSynchronize(ctx->ev[6]));
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]);
        ms_num += ms;
    }
    cudaEventRecord(ctx->ev[4], s);
    std::vector<int64_t> hr((size_t)csb * np + 1);
    std::vector<double> hv((size_t)csb * np + 1);
    if (np > 0) {
        GBC_CUDA_TRY(cudaMemcpyAsync(hr.data(), rsum, (size_t)csb * np * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(hv.data(), vsum, (size_t)csb * np * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    int32_t herr = 0;
    GBC_CUDA_TRY(cudaMemcpyAsync(&herr, a.err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr) return fail(GBC_ECUDA, "internal error: numeric and symbolic counts disagree");
    if (st) {
        float t04 = 0, t12 = 0;
        cudaEventElapsedTime(&t04, ctx->ev[0], ctx->ev[4]);
        cudaEventElapsedTime(&t12, ctx->ev[1], ctx->ev[2]);
        st->flops = flops;
        st->nnz = total;
        st->phases = np;
        st->ms_total = t04;
        st->ms_symbolic = t12;
        st->ms_numeric = ms_num;
        int64_t rs = 0;
        double vs = 0;
        for (size_t k = 0; k < (size_t)csb * np; ++k) {
            rs += hr[k];
            vs += hv[k];
        }
        st->row_checksum = rs;
        st->val_checksum = vs;
        st->max_phase_nnz = maxp;
    }
    return GBC_OK;
}

template <class SR>
int spgemm_learned(Context *, const DevMatrix &, const DevMatrix &, const gbc_spgemm_opts &, int, gbc_result **,
                   gbc_spgemm_stats *)
{
    return fail(GBC_EUNSUPPORTED, "learned sizing is not built yet");
}

template <class SR>
static int spgemm_entry(gbc_context *ctx, int vt, const gbc_matrix *Am, const gbc_matrix *Bm,
                        const gbc_spgemm_opts *opts, gbc_result **C, gbc_spgemm_stats *st)
{
    if (!ctx || !C) return fail(GBC_EINVAL, "null context or output");
    *C = nullptr;
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    gbc_spgemm_opts opt{GBC_SIZING_EXACT, GBC_SORTED, 1, 0};
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
    SpgemmArgs a{};
    int64_t *acp = nullptr;
    GBC_TRY(prepare_operands(ws, A, B, a, &acp));
    int64_t nb = B.nzc;
    int64_t *flop = nullptr, *cnt = nullptr;
    uint64_t *tmask = nullptr;
    unsigned long long *work = nullptr;
    GBC_TRY(ws.alloc_n(&flop, nb + 1));
    GBC_TRY(ws.alloc_n(&cnt, nb + 1));
    GBC_TRY(ws.alloc_n(&tmask, (size_t)nb * a.mask_words + 1));
    GBC_TRY(ws.alloc_n(&work, 4));
    GBC_CUDA_TRY(cudaMemsetAsync(work, 0, 4 * sizeof(unsigned long long), s));
    a.flop = flop;
    if (nb > 0) {
        k_flop<<<grid_for(ctx, (nb + 7) / 8, 8), 256, 0, s>>>(nb, B.cp, a.brow, acp, flop); ::gbc::note_launch();
        int sup_rows = (int)std::min<int64_t>((int64_t)kSymRows, (int64_t)a.T * a.R);
        sup_rows = (sup_rows / a.R) * a.R;
        size_t sym_smem = (size_t)sup_rows / 8;
        GBC_CUDA_TRY(cudaFuncSetAttribute(k_symbolic, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sym_smem));
        k_symbolic<<<grid_for(ctx, nb, 2), kThreads, sym_smem, s>>>(a, cnt, tmask, sup_rows, work); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    cudaMemcpyKind k = where == GBC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (flop_out && nb) GBC_CUDA_TRY(cudaMemcpyAsync(flop_out, flop, nb * sizeof(int64_t), k, s));
    if (nnz_out && nb) GBC_CUDA_TRY(cudaMemcpyAsync(nnz_out, cnt, nb * sizeof(int64_t), k, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    return GBC_OK;
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
                      int64_t max_phase_nnz, gbc_phased_stats *st)
{
    if (!ctx) return fail(GBC_EINVAL, "null context");
    if (!Am || !Bm || Am->ncol != Bm->nrow) return fail(GBC_EINVAL, "inner dimensions do not match");
    if (max_phase_nnz <= 0) return fail(GBC_EINVAL, "phase budget must be positive");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    Workspace ws(ctx);
    DevMatrix A, B;
    GBC_TRY(upload(ws, Am, vt, &A));
    GBC_TRY(upload(ws, Bm, vt, &B));
    if (sr == GBC_SR_PLUSTIMES && vt == GBC_F64) return spgemm_phased<PlusTimes<double>>(ctx, A, B, max_phase_nnz, st);
    if (sr == GBC_SR_PLUSTIMES && vt == GBC_F32) return spgemm_phased<PlusTimes<float>>(ctx, A, B, max_phase_nnz, st);
    if (sr == GBC_SR_SELECT2NDMIN && vt == GBC_I64)
        return spgemm_phased<Select2ndMin<int64_t>>(ctx, A, B, max_phase_nnz, st);
    return fail(GBC_EUNSUPPORTED, "phased SpGEMM is instantiated for PlusTimes f64/f32 and Select2ndMin i64");
}

int gbc_spgemm_colstats(gbc_context *ctx, const gbc_matrix *A, const gbc_matrix *B, int64_t *flop, int64_t *nnz,
                        int where)
{
    return spgemm_colstats(ctx, A, B, flop, nnz, where);
}

}  // extern "C"
