// Sparse matrix x sparse vector over Select2ndMin / SelectMin and the
// top-down BFS built on it -- the local multiply SpMXSpV_Bucket
// (SpImpl.cpp:389-699) and the BFS_CSC level loop of
// Applications/SpMSpV-IPDPS2017/SpMSpVBench.cpp:128-156.
//
// y(r) = min over x entries (c, v) with A(r,c) != 0 of v, output sorted by r.
// The GPU form: the frontier's columns are walked in chunks of kThreads
// entries whose A segments are flattened across the block; each product does
// an atomicMin into a dense candidate array and marks a touched bitmap.
// Because min is order independent, the result equals the reference's
// bucketed SPA merge bit for bit.  Rows are emitted in ascending order by a
// scan over the touched bitmap (no sort).
//
// BFS fuses the per-level glue: EWiseMult(fringe, parents, exclude=true, -1)
// becomes a visited-bitmap test before the atomicMin, and parents.Set(fringe)
// plus the frontier rebuild is one finalize kernel.  All per-level sizes stay
// on the device, so the level loop is captured once into a CUDA graph and
// replayed per level.
#include <algorithm>
#include <cstring>

#include "gbc_internal.cuh"
#include "spgemm_kernels.cuh"

namespace gbc {

constexpr int32_t kNoCand = INT32_MAX;

struct Graph {
    Context *ctx = nullptr;
    int64_t n = 0, nnz = 0;
    int64_t *cp = nullptr;   // [n+1] (int64 for the caller-facing degree sums)
    uint32_t *cp32 = nullptr;  // [n+1]
    int32_t *row = nullptr;  // [nnz]
    // BFS state (allocated on first use)
    int32_t *cand = nullptr;     // [n] candidate parent, kNoCand when untouched
    uint32_t *visited = nullptr;  // [n/32] parents != -1
    int32_t *front[2] = {nullptr, nullptr};
    uint32_t *fbits[2] = {nullptr, nullptr};  // frontier bitmaps (current / next)
    int64_t *off = nullptr;                   // [n+1] prefix of frontier degrees
    int64_t *tile = nullptr;                  // per-tile sums of that prefix
    int32_t *chunk_f0 = nullptr;              // [nnz / kEdgeChunk + 2] frontier entry holding each chunk's first edge
    int64_t *ctl = nullptr;  // device control block (see CTL_*)
    int64_t *h_ctl = nullptr;  // pinned mirror
    cudaGraphExec_t level_exec = nullptr;
    long long level_kernels = 0;  // kernels one replay of the level graph runs
    cudaGraphExec_t loop_exec = nullptr;  // the whole traversal: a while node around one level
    long long loop_kernels = 0;           // kernels of one trip of its body
    int64_t *g_parents = nullptr, *g_levels = nullptr;  // pointers baked into the graph
    int g_policy = -1;                                   // the direction policy it was captured for
    int64_t *own_parents = nullptr, *own_levels = nullptr;  // device outputs of host-array calls
    bool bfs_ready = false;
    int policy = 0;  // direction policy (see gbc_graph_set_policy)
    // multi-source BFS state, sized for ms_roots roots (allocated on use)
    int64_t ms_roots = 0;
    int32_t *ms_cand = nullptr;       // [roots * n] candidate parent per (root, vertex)
    uint32_t *ms_visited = nullptr;   // [roots * n / 32]
    int64_t *ms_front[2] = {nullptr, nullptr};  // frontier entries (root << 32 | vertex)
    int64_t *ms_ctl = nullptr;        // device control block (MS_*)
    int64_t *ms_rcnt = nullptr, *ms_roff = nullptr;  // root counts / offsets of the frontier sort
    int64_t *h_ms_ctl = nullptr;      // pinned mirror
    cudaGraphExec_t ms_exec = nullptr;
    long long ms_kernels = 0;
    cudaGraphExec_t ms_loop_exec = nullptr;
    long long ms_loop_kernels = 0;
    int64_t *ms_g_parents = nullptr;  // parents pointer baked into ms_exec
};

// control block layout
enum {
    CTL_NF = 0,       // current frontier size
    CTL_NNEXT = 1,    // next frontier size
    CTL_ITER = 2,     // level-loop iterations done
    CTL_WORK = 3,     // work counter of the expand kernels
    CTL_EDGES = 4,    // sum of degrees of reached vertices
    CTL_REACHED = 5,  // reached vertices
    CTL_CUR = 6,      // which frontier buffer is current
    CTL_FE = 7,       // edges of the current frontier (sum of degrees)
    CTL_FE_NEXT = 8,  // edges of the next frontier
    CTL_UE = 9,       // edges of unreached vertices
    CTL_DIR = 10,     // 0 top-down, 1 bottom-up
    CTL_E = 11,       // top-down: total frontier edges of this level (scan result)
    CTL_POLICY = 12,  // 0 choose per level, 1 always top-down, 2 always bottom-up
    CTL_N
};
// frontier pointer table follows the control words
constexpr int kCtlWords = 16;

__global__ void k_graph_prep(int64_t n, int64_t nnz, const int64_t *cp, const int64_t *ir, uint32_t *cp32,
                             int32_t *row, int32_t *err)
{
    int lane = threadIdx.x & 31;
    int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t c = warp; c < n; c += nwarps) {
        int64_t s = cp[c], e = cp[c + 1];
        if (lane == 0) {
            cp32[c] = (uint32_t)s;
            if (c == n - 1) cp32[n] = (uint32_t)e;
        }
        if (e < s || (c == 0 && s != 0) || e > nnz) {
            if (lane == 0) atomicOr(err, 1);
            continue;
        }
        for (int64_t p = s + lane; p < e; p += 32) {
            int64_t r = ir[p];
            if (r < 0 || r >= n) {
                atomicOr(err, 4);
                r = 0;
            }
            row[p] = (int32_t)r;
        }
    }
}

// ------------------------------------------------------------- chunk walk
// kThreads frontier columns per chunk: s = segment start, off = exclusive
// prefix of segment lengths, val = the vector value carried by the column.
struct FrontChunk {
    uint32_t s[kThreads];
    int32_t off[kThreads + 1];
    int64_t val[kThreads];
};

__device__ __forceinline__ int front_find(const FrontChunk &ch, int j)
{
    int lo = 0, hi = kThreads;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (ch.off[mid] <= j)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// --------------------------------------------------------------- SpMSpV
// y = A x (Select2ndMin): atomicMin of the x value into spa[r]; touched
// rows marked in `mark`.
__global__ void __launch_bounds__(kThreads) k_spmspv_expand(const uint32_t *cp32, const int32_t *row,
                                                            const int32_t *xind, const int64_t *xval, int64_t nx,
                                                            int64_t n, unsigned long long *spa, uint32_t *mark,
                                                            unsigned long long *work, int32_t *err)
{
    __shared__ FrontChunk ch;
    __shared__ int64_t s_base;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_base = (int64_t)atomicAdd(work, (unsigned long long)kThreads);
        __syncthreads();
        const int64_t base = s_base;
        __syncthreads();
        if (base >= nx) break;
        const int64_t f = base + tid;
        int len = 0;
        if (f < nx) {
            const int32_t c = xind[f];
            if (c < 0 || c >= n) {
                atomicOr(err, 1);
            } else {
                const uint32_t s = cp32[c];
                ch.s[tid] = s;
                ch.val[tid] = xval[f];
                len = (int)(cp32[c + 1] - s);
            }
        }
        int64_t tot;
        const int off = (int)block_exclusive_sum64(len, &tot);
        ch.off[tid] = off;
        if (tid == kThreads - 1) ch.off[kThreads] = off + len;
        __syncthreads();
        for (int j = tid; j < (int)tot; j += kThreads) {
            const int b = front_find(ch, j);
            const int32_t r = row[ch.s[b] + (j - ch.off[b])];
            // signed min through the order-preserving flip of the sign bit
            atomicMin(&spa[r], (unsigned long long)ch.val[b] ^ 0x8000000000000000ull);
            const uint32_t bit = 1u << (r & 31);
            if (!(mark[r >> 5] & bit)) atomicOr(&mark[r >> 5], bit);
        }
        __syncthreads();
    }
}

// Emit touched rows in ascending order: per 32-row word, popcount prefix.
__global__ void k_mark_counts(const uint32_t *mark, int64_t words, int64_t *cnt)
{
    int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w < words) cnt[w] = __popc(mark[w]);
}

__global__ void k_mark_emit(uint32_t *mark, int64_t words, const int64_t *pos, unsigned long long *spa, int32_t *yind,
                            int64_t *yval)
{
    int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w >= words) return;
    uint32_t x = mark[w];
    int64_t p = pos[w];
    while (x) {
        int b = __ffs(x) - 1;
        x &= x - 1;
        int64_t r = w * 32 + b;
        yind[p] = (int32_t)r;
        yval[p] = (int64_t)(spa[r] ^ 0x8000000000000000ull);
        spa[r] = ~0ull;  // back to "empty" for the next call
        ++p;
    }
    mark[w] = 0;
}

// ------------------------------------------------------------------- BFS
// Level loop of the reference's BFS over SelectMin (parent = smallest
// frontier neighbour), run in either direction per level:
//  * top-down: edge-balanced expansion of the frontier -- frontier degrees
//    are prefix-summed and every block takes fixed chunks of kEdgeChunk edges,
//    so hub vertices are shared by many blocks -- with cand[r] = atomicMin of
//    the frontier ids (EWiseMult(..., exclude) is the visited-bitmap test);
//  * bottom-up: every unreached vertex scans its neighbours in ascending
//    order and takes the first one in the frontier bitmap.  Neighbours are
//    sorted, so that first frontier neighbour IS the minimum, and the result
//    equals the top-down one bit for bit.
// The direction is chosen on the device per level (frontier edges against
// unreached edges, as direction-optimizing BFS does), so one captured graph
// serves every level.
constexpr int kQueue = 4096;
constexpr int kEdgeChunk = 1024;
constexpr int kScanTile = 2048;

__device__ __forceinline__ void queue_flush(int32_t *q, int &s_qn, unsigned long long &s_gbase, int64_t *ctl,
                                            int32_t *next)
{
    const int tid = threadIdx.x;
    const int qn = s_qn;
    if (qn > 0) {
        if (tid == 0) s_gbase = atomicAdd((unsigned long long *)&ctl[CTL_NNEXT], (unsigned long long)qn);
        __syncthreads();
        for (int k = tid; k < qn; k += blockDim.x) next[s_gbase + k] = q[k];
        __syncthreads();
        if (tid == 0) s_qn = 0;
    }
    __syncthreads();
}

// Direction of the level about to run (one thread: the end of the previous
// level, or the traversal's initialisation for the first level).
__device__ void bfs_direction(int64_t *ctl, int64_t n)
{
    const int64_t nf = ctl[CTL_NF];
    if (nf == 0) return;
    int64_t dir = ctl[CTL_DIR];
    if (dir == 0 && ctl[CTL_FE] * 14 > ctl[CTL_UE]) dir = 1;
    else if (dir == 1 && nf * 24 < n) dir = 0;
    if (ctl[CTL_POLICY] == 1) dir = 0;
    if (ctl[CTL_POLICY] == 2) dir = 1;
    ctl[CTL_DIR] = dir;
    ctl[CTL_E] = 0;
}

// Top-down prefix of frontier degrees, in three fixed-size launches so the
// graph can be replayed for any frontier size: tile sums, tile scan (one
// block), rescan.
__global__ void k_bfs_deg_tiles(const uint32_t *cp32, const int64_t *ctl, int32_t *const *fronts, int64_t *tile)
{
    if (ctl[CTL_DIR] != 0) return;
    const int64_t nf = ctl[CTL_NF];
    const int32_t *front = fronts[ctl[CTL_CUR]];
    const int64_t b0 = int64_t(blockIdx.x) * kScanTile;
    if (b0 >= nf) return;
    int64_t sum = 0;
    for (int64_t f = b0 + threadIdx.x; f < min(nf, b0 + kScanTile); f += blockDim.x) {
        const int32_t c = front[f];
        sum += cp32[c + 1] - cp32[c];
    }
    int64_t tot;
    block_exclusive_sum64(sum, &tot);
    if (threadIdx.x == 0) tile[blockIdx.x] = tot;
}

__global__ void k_bfs_deg_scan(int64_t *ctl, int64_t *tile)
{
    if (ctl[CTL_DIR] != 0) return;
    const int64_t nf = ctl[CTL_NF];
    const int64_t nt = (nf + kScanTile - 1) / kScanTile;
    int64_t carry = 0;
    for (int64_t b = 0; b < nt; b += blockDim.x) {
        const int64_t t = b + threadIdx.x;
        const int64_t v = t < nt ? tile[t] : 0;
        int64_t tot;
        const int64_t ex = block_exclusive_sum64(v, &tot);
        if (t < nt) tile[t] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) ctl[CTL_E] = carry;
}

__global__ void k_bfs_deg_rescan(const uint32_t *cp32, const int64_t *ctl, int32_t *const *fronts,
                                 const int64_t *tile, int64_t *off, int32_t *chunk_f0)
{
    if (ctl[CTL_DIR] != 0) return;
    const int64_t nf = ctl[CTL_NF];
    const int32_t *front = fronts[ctl[CTL_CUR]];
    const int64_t b0 = int64_t(blockIdx.x) * kScanTile;
    if (b0 >= nf) return;
    constexpr int PER = kScanTile / kThreads;
    int64_t d[PER], sum = 0;
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int64_t f = b0 + int64_t(threadIdx.x) * PER + u;
        d[u] = 0;
        if (f < nf) {
            const int32_t c = front[f];
            d[u] = cp32[c + 1] - cp32[c];
        }
        sum += d[u];
    }
    int64_t tot;
    int64_t run = tile[blockIdx.x] + block_exclusive_sum64(sum, &tot);
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int64_t f = b0 + int64_t(threadIdx.x) * PER + u;
        if (f < nf) {
            off[f] = run;
            // the edge chunks that start inside this entry's edges
            if (d[u] > 0)
                for (int64_t c = (run + kEdgeChunk - 1) / kEdgeChunk; c <= (run + d[u] - 1) / kEdgeChunk; ++c)
                    chunk_f0[c] = (int32_t)f;
        }
        run += d[u];
    }
    if (b0 + kScanTile >= nf && threadIdx.x == kThreads - 1) off[nf] = run;
}

// Top-down expansion over fixed edge chunks.
__global__ void __launch_bounds__(kThreads) k_bfs_td(const uint32_t *cp32, const int32_t *row,
                                                     const uint32_t *visited, int32_t *cand, int64_t *ctl,
                                                     int32_t *const *fronts, const int64_t *off,
                                                     const int32_t *chunk_f0)
{
    __shared__ int64_t s_off[kEdgeChunk + 2];
    __shared__ uint32_t s_st[kEdgeChunk + 2];
    __shared__ int32_t s_c[kEdgeChunk + 2];
    __shared__ int64_t s_chunk, s_f0;
    __shared__ int s_k;
    __shared__ int32_t q[kQueue];
    __shared__ int s_qn;
    __shared__ unsigned long long s_gbase;
    if (ctl[CTL_DIR] != 0) return;
    const int tid = threadIdx.x, lane = tid & 31;
    const int cur = (int)ctl[CTL_CUR];
    const int32_t *front = fronts[cur];
    int32_t *next = fronts[cur ^ 1];
    const int64_t nf = ctl[CTL_NF];
    const int64_t E = ctl[CTL_E];
    if (tid == 0) s_qn = 0;
    __syncthreads();
    for (;;) {
        if (tid == 0) {
            s_chunk = (int64_t)atomicAdd((unsigned long long *)&ctl[CTL_WORK], 1ull);
            const int64_t e0 = s_chunk * kEdgeChunk;
            if (e0 < E) {
                // first frontier entry of this chunk and of the next one
                // (the last entry holding edges of this chunk is that one or
                // the one before), from the rescan's chunk table
                const int64_t lo = chunk_f0[s_chunk];
                const int64_t lo2 = e0 + kEdgeChunk < E ? chunk_f0[s_chunk + 1] : nf - 1;
                s_f0 = lo;
                s_k = (int)(lo2 - lo + 1);  // <= nf < 2^31
            }
        }
        __syncthreads();
        const int64_t e0 = s_chunk * kEdgeChunk;
        if (e0 >= E) break;
        const int K = s_k;
        const int64_t f0 = s_f0;
        // a chunk spans at most kEdgeChunk non-empty entries; empty entries
        // (columns without entries, in a non-symmetric pattern) between
        // them can make K larger, and such a chunk searches off in memory
        const bool staged = K <= kEdgeChunk + 1;  // block-uniform
        if (staged)
            for (int k = tid; k <= K; k += kThreads) {
                s_off[k] = off[f0 + k];  // off has nf + 1 entries and f0 + K <= nf
                if (k < K) {
                    const int32_t c = front[f0 + k];
                    s_c[k] = c;
                    s_st[k] = cp32[c];
                }
            }
        __syncthreads();
        const int64_t e1 = min(E, e0 + kEdgeChunk);
        for (int64_t e = e0 + tid; e < e0 + kEdgeChunk; e += kThreads) {
            bool fresh = false;
            int32_t r = 0;
            if (e < e1) {
                int lo = 0, hi = K;
                int32_t c;
                if (staged) {
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (s_off[mid] <= e) lo = mid; else hi = mid;
                    }
                    c = s_c[lo];
                    r = row[s_st[lo] + (e - s_off[lo])];
                } else {
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (off[f0 + mid] <= e) lo = mid; else hi = mid;
                    }
                    c = front[f0 + lo];
                    r = row[cp32[c] + (e - off[f0 + lo])];
                }
                if (!(visited[r >> 5] & (1u << (r & 31)))) {
                    if (c < cand[r]) {
                        const int32_t old = atomicMin(&cand[r], c);
                        fresh = old == kNoCand;
                    }
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, fresh);
            if (m) {
                int slot = 0;
                if (lane == __ffs(m) - 1) slot = atomicAdd(&s_qn, __popc(m));
                slot = __shfl_sync(0xffffffffu, slot, __ffs(m) - 1);
                if (fresh) q[slot + __popc(m & ((1u << lane) - 1))] = r;
            }
        }
        __syncthreads();
        if (s_qn > kQueue - kEdgeChunk) queue_flush(q, s_qn, s_gbase, ctl, next);
    }
    queue_flush(q, s_qn, s_gbase, ctl, next);
}

// Top-down finalize: parents.Set(fringe) for the new frontier, plus visited,
// levels, next-frontier bitmap and degree sums.
__global__ void k_bfs_finalize(int32_t *cand, uint32_t *visited, int64_t *parents, int64_t *levels,
                               const int64_t *cp, int64_t *ctl, int32_t *const *fronts, uint32_t *const *fbits)
{
    if (ctl[CTL_NF] == 0 || ctl[CTL_DIR] != 0) return;
    const int cur = (int)ctl[CTL_CUR];
    const int32_t *next = fronts[cur ^ 1];
    uint32_t *nbits = fbits[cur ^ 1];
    const int64_t nn = ctl[CTL_NNEXT];
    const int64_t iter = ctl[CTL_ITER] + 1;
    int64_t deg = 0, reached = 0, fdeg = 0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nn; i += int64_t(gridDim.x) * blockDim.x) {
        const int32_t r = next[i];
        parents[r] = cand[r];
        cand[r] = kNoCand;
        atomicOr(&visited[r >> 5], 1u << (r & 31));
        atomicOr(&nbits[r >> 5], 1u << (r & 31));
        const int64_t d = cp[r + 1] - cp[r];
        fdeg += d;
        if (levels[r] < 0) {
            levels[r] = iter;
            deg += d;
            ++reached;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        deg += __shfl_xor_sync(0xffffffffu, deg, o);
        reached += __shfl_xor_sync(0xffffffffu, reached, o);
        fdeg += __shfl_xor_sync(0xffffffffu, fdeg, o);
    }
    if ((threadIdx.x & 31) == 0 && (fdeg || reached)) {
        atomicAdd((unsigned long long *)&ctl[CTL_EDGES], (unsigned long long)deg);
        atomicAdd((unsigned long long *)&ctl[CTL_REACHED], (unsigned long long)reached);
        atomicAdd((unsigned long long *)&ctl[CTL_FE_NEXT], (unsigned long long)fdeg);
    }
}

// Bottom-up level: every vertex without a parent takes its smallest
// neighbour that is in the current frontier.
__global__ void __launch_bounds__(kThreads) k_bfs_bu(const int64_t *cp, const int32_t *row, uint32_t *visited,
                                                     int64_t *parents, int64_t *levels, int64_t n, int64_t *ctl,
                                                     int32_t *const *fronts, uint32_t *const *fbits)
{
    __shared__ int32_t q[kQueue];
    __shared__ int s_qn;
    __shared__ unsigned long long s_gbase;
    if (ctl[CTL_NF] == 0 || ctl[CTL_DIR] != 1) return;
    const int tid = threadIdx.x, lane = tid & 31;
    const int cur = (int)ctl[CTL_CUR];
    int32_t *next = fronts[cur ^ 1];
    const uint32_t *fb = fbits[cur];
    uint32_t *nb = fbits[cur ^ 1];
    const int64_t iter = ctl[CTL_ITER] + 1;
    if (tid == 0) s_qn = 0;
    __syncthreads();
    int64_t deg = 0, reached = 0, fdeg = 0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t b = int64_t(blockIdx.x) * blockDim.x; b < n; b += stride) {
        const int64_t v = b + tid;
        bool fresh = false;
        if (v < n && !(visited[v >> 5] & (1u << (v & 31)))) {
            const int64_t s = cp[v], e = cp[v + 1];
            for (int64_t p = s; p < e; ++p) {
                const int32_t u = row[p];
                if (fb[u >> 5] & (1u << (u & 31))) {
                    parents[v] = u;
                    fresh = true;
                    break;
                }
            }
            if (fresh) {
                atomicOr(&nb[v >> 5], 1u << (v & 31));
                fdeg += e - s;
                if (levels[v] < 0) {
                    levels[v] = iter;
                    deg += e - s;
                    ++reached;
                }
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, fresh);
        if (m) {
            int slot = 0;
            if (lane == __ffs(m) - 1) slot = atomicAdd(&s_qn, __popc(m));
            slot = __shfl_sync(0xffffffffu, slot, __ffs(m) - 1);
            if (fresh) q[slot + __popc(m & ((1u << lane) - 1))] = (int32_t)v;
        }
        __syncthreads();
        if (s_qn > kQueue - kThreads) queue_flush(q, s_qn, s_gbase, ctl, next);
    }
    queue_flush(q, s_qn, s_gbase, ctl, next);
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        deg += __shfl_xor_sync(0xffffffffu, deg, o);
        reached += __shfl_xor_sync(0xffffffffu, reached, o);
        fdeg += __shfl_xor_sync(0xffffffffu, fdeg, o);
    }
    if (lane == 0 && (fdeg || reached)) {
        atomicAdd((unsigned long long *)&ctl[CTL_EDGES], (unsigned long long)deg);
        atomicAdd((unsigned long long *)&ctl[CTL_REACHED], (unsigned long long)reached);
        atomicAdd((unsigned long long *)&ctl[CTL_FE_NEXT], (unsigned long long)fdeg);
    }
}

// End of a level whose direction may be bottom-up: the current frontier's
// bitmap (read only by the bottom-up kernel) is cleared, so it can collect
// the frontier after next; after a bottom-up level the new vertices are
// marked visited -- after the level, so a vertex found in it is never taken
// as a parent in it (only frontier bits are read there).
__global__ void k_bfs_level_end(uint32_t *visited, const int64_t *ctl, int32_t *const *fronts,
                                uint32_t *const *fbits, int64_t words)
{
    if (ctl[CTL_NF] == 0) return;
    const int cur = (int)ctl[CTL_CUR];
    const int64_t i0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x, stride = int64_t(gridDim.x) * blockDim.x;
    uint32_t *fb = fbits[cur];
    for (int64_t w = i0; w < words; w += stride) fb[w] = 0;
    if (ctl[CTL_DIR] != 1) return;
    const int32_t *next = fronts[cur ^ 1];
    const int64_t nn = ctl[CTL_NNEXT];
    for (int64_t i = i0; i < nn; i += stride) atomicOr(&visited[next[i] >> 5], 1u << (next[i] & 31));
}

// Advance the level (the next frontier becomes current) and choose the next
// level's direction.  Inside a traversal graph (set_cond) it also sets the
// while node's condition: another level while the frontier is nonempty, at
// most `cap` levels (a level loop over n vertices ends within n + 1 levels,
// so the cap never cuts a traversal short).
__global__ void k_bfs_advance(int64_t *ctl, int64_t n, int64_t cap, cudaGraphConditionalHandle h, int set_cond)
{
    if (ctl[CTL_NF] != 0) {  // else finished: later replays change nothing
        ctl[CTL_NF] = ctl[CTL_NNEXT];
        ctl[CTL_NNEXT] = 0;
        ctl[CTL_WORK] = 0;
        ctl[CTL_ITER] += 1;
        ctl[CTL_CUR] ^= 1;
        ctl[CTL_UE] -= ctl[CTL_FE_NEXT];
        ctl[CTL_FE] = ctl[CTL_FE_NEXT];
        ctl[CTL_FE_NEXT] = 0;
        bfs_direction(ctl, n);
    }
    if (set_cond) cudaGraphSetConditional(h, (ctl[CTL_NF] != 0 && ctl[CTL_ITER] < cap) ? 1u : 0u);
}

__global__ void k_bfs_init(int64_t n, int64_t nnz, int32_t *cand, uint32_t *visited, int64_t *parents,
                           int64_t *levels, int64_t source, const int64_t *cp, int64_t *ctl, int32_t *const *fronts,
                           uint32_t *const *fbits)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t v = i; v < n; v += stride) {
        cand[v] = kNoCand;
        parents[v] = -1;
        levels[v] = -1;
    }
    for (int64_t w = i; w < (n + 31) / 32; w += stride) {
        visited[w] = 0;
        fbits[0][w] = 0;
        fbits[1][w] = 0;
    }
}

__global__ void k_bfs_init2(int64_t n, int64_t nnz, int64_t *levels, int64_t source, const int64_t *cp,
                            int64_t *ctl, int32_t *const *fronts, uint32_t *const *fbits, int policy)
{
    ctl[CTL_POLICY] = policy;
    fronts[0][0] = (int32_t)source;
    fbits[0][source >> 5] |= 1u << (source & 31);
    levels[source] = 0;
    const int64_t ds = cp[source + 1] - cp[source];
    ctl[CTL_NF] = 1;
    ctl[CTL_NNEXT] = 0;
    ctl[CTL_ITER] = 0;
    ctl[CTL_WORK] = 0;
    ctl[CTL_EDGES] = ds;
    ctl[CTL_REACHED] = 1;
    ctl[CTL_CUR] = 0;
    ctl[CTL_FE] = ds;
    ctl[CTL_FE_NEXT] = 0;
    ctl[CTL_UE] = nnz;  // the source is still unreached for the reference's loop
    ctl[CTL_DIR] = 0;
    ctl[CTL_E] = 0;
    bfs_direction(ctl, n);  // the first level's
}

// Condition of a traversal's while node: another level while the frontier
// is nonempty, at most `cap` levels (a level loop over n vertices ends
// within n + 1 levels, so the cap never cuts a traversal short).
__global__ void k_loop_cond(const int64_t *nf, const int64_t *level, int64_t cap, cudaGraphConditionalHandle h)
{
    cudaGraphSetConditional(h, (*nf != 0 && *level < cap) ? 1u : 0u);
}

// An executable graph of one while node whose body is what `body(stream,
// handle)` launches on the capturing stream, followed by the condition
// kernel unless the body sets the condition itself (body_sets_cond).  The
// whole traversal then runs from one graph launch with no host round trip.
template <class F>
static int loop_graph(F body, bool body_sets_cond, const int64_t *nf, const int64_t *level, int64_t cap,
                      cudaGraphExec_t *exec, long long *kernels)
{
    cudaGraph_t graph = nullptr;
    GBC_CUDA_TRY(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
    cudaStream_t cs = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    cudaGraph_t bodyg = e == cudaSuccess ? np.conditional.phGraph_out[0] : nullptr;
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(cs, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    int rc = GBC_OK;
    if (e == cudaSuccess) {
        const long long c0 = launch_count();
        rc = body(cs, h);
        if (!body_sets_cond) {
            k_loop_cond<<<1, 1, 0, cs>>>(nf, level, cap, h);
            note_launch();
        }
        *kernels = launch_count() - c0;
        note_launches(-*kernels);  // captured, not run
        e = cudaStreamEndCapture(cs, &bodyg);
    }
    if (cs) cudaStreamDestroy(cs);
    if (e == cudaSuccess && rc == GBC_OK) e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (rc != GBC_OK) return rc;
    if (e != cudaSuccess) {
        *exec = nullptr;
        cudaGetLastError();
        return fail(GBC_ECUDA, std::string("traversal graph: ") + cudaGetErrorString(e));
    }
    return GBC_OK;
}

// -------------------------------------------------------------- host side
static int graph_alloc_bfs(Graph *g)
{
    Context *ctx = g->ctx;
    if (g->bfs_ready) return GBC_OK;
    const int64_t words = (g->n + 31) / 32 + 1;
    GBC_TRY(device_alloc(ctx, (void **)&g->cand, g->n * sizeof(int32_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->visited, words * sizeof(uint32_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->front[0], g->n * sizeof(int32_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->front[1], g->n * sizeof(int32_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->fbits[0], words * sizeof(uint32_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->fbits[1], words * sizeof(uint32_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->off, (g->n + 2) * sizeof(int64_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->tile, ((g->n + kScanTile - 1) / kScanTile + 2) * sizeof(int64_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->chunk_f0, (g->nnz / kEdgeChunk + 2) * sizeof(int32_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->ctl, (kCtlWords + 8) * sizeof(int64_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->own_parents, (g->n + 1) * sizeof(int64_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->own_levels, (g->n + 1) * sizeof(int64_t)));
    GBC_CUDA_TRY(cudaMallocHost(&g->h_ctl, (kCtlWords + 8) * sizeof(int64_t)));
    // pointer tables after the control words: fronts[2], fbits[2]
    void *tab[4] = {g->front[0], g->front[1], g->fbits[0], g->fbits[1]};
    GBC_CUDA_TRY(cudaMemcpyAsync(g->ctl + kCtlWords, tab, sizeof(tab), cudaMemcpyHostToDevice, ctx->stream));
    g->bfs_ready = true;
    return GBC_OK;
}

static int32_t *const *fronts_dev(Graph *g) { return reinterpret_cast<int32_t *const *>(g->ctl + kCtlWords); }
static uint32_t *const *fbits_dev(Graph *g) { return reinterpret_cast<uint32_t *const *>(g->ctl + kCtlWords + 2); }

// A persistent grid of `kernel`: as many blocks as the occupancy query
// allows on every SM (at least one).
static int occ_grid(const Context *ctx, const void *kernel, int threads, size_t smem)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        nb = 4;
    }
    return ctx->num_sms * std::max(nb, 1);
}

// One level.  The policy fixes which kernels can do work: always top-down
// leaves out the bottom-up kernels (the frontier bitmaps are then never
// read), always bottom-up leaves out the top-down ones; "auto" launches
// both sets, the direction flag in the control block enabling one.  In a
// traversal graph (set_cond) the advance kernel sets the while node's
// condition h.
static int launch_level(Graph *g, int64_t *parents, int64_t *levels, cudaStream_t s, cudaGraphConditionalHandle h,
                        int set_cond)
{
    Context *ctx = g->ctx;
    const int grid = ctx->num_sms * 4;
    const int64_t words = (g->n + 31) / 32;
    const unsigned tiles = (unsigned)((g->n + kScanTile - 1) / kScanTile);
    int launched = 1;
    if (g->policy != 2) {
        const int grid_td = occ_grid(ctx, (const void *)k_bfs_td, kThreads, 0);
        k_bfs_deg_tiles<<<tiles, kThreads, 0, s>>>(g->cp32, g->ctl, fronts_dev(g), g->tile);
        k_bfs_deg_scan<<<1, kThreads, 0, s>>>(g->ctl, g->tile);
        k_bfs_deg_rescan<<<tiles, kThreads, 0, s>>>(g->cp32, g->ctl, fronts_dev(g), g->tile, g->off, g->chunk_f0);
        k_bfs_td<<<grid_td, kThreads, 0, s>>>(g->cp32, g->row, g->visited, g->cand, g->ctl, fronts_dev(g), g->off,
                                              g->chunk_f0);
        k_bfs_finalize<<<occ_grid(ctx, (const void *)k_bfs_finalize, 256, 0), 256, 0, s>>>(
            g->cand, g->visited, parents, levels, g->cp, g->ctl, fronts_dev(g), fbits_dev(g));
        launched += 5;
    }
    if (g->policy != 1) {
        const int grid_bu = occ_grid(ctx, (const void *)k_bfs_bu, kThreads, 0);
        k_bfs_bu<<<grid_bu, kThreads, 0, s>>>(g->cp, g->row, g->visited, parents, levels, g->n, g->ctl,
                                              fronts_dev(g), fbits_dev(g));
        k_bfs_level_end<<<grid, 256, 0, s>>>(g->visited, g->ctl, fronts_dev(g), fbits_dev(g), words);
        launched += 2;
    }
    k_bfs_advance<<<1, 1, 0, s>>>(g->ctl, g->n, g->n + 2, h, set_cond);
    note_launches(launched);
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

// Capture one level into a graph once per (graph, output buffers).
static int level_graph(Graph *g, int64_t *parents, int64_t *levels)
{
    if (g->level_exec && g->g_parents == parents && g->g_levels == levels && g->g_policy == g->policy)
        return GBC_OK;
    if (g->level_exec) {
        cudaGraphExecDestroy(g->level_exec);
        g->level_exec = nullptr;
    }
    cudaStream_t cs;
    GBC_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph;
    const long long c0 = launch_count();
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(cs);
        return fail(GBC_ECUDA, std::string("capture: ") + cudaGetErrorString(e));
    }
    int rc = launch_level(g, parents, levels, cs, 0, 0);
    e = cudaStreamEndCapture(cs, &graph);
    g->level_kernels = launch_count() - c0;
    note_launches(-g->level_kernels);  // captured, not run
    cudaStreamDestroy(cs);
    if (rc != GBC_OK) return rc;
    if (e != cudaSuccess) return fail(GBC_ECUDA, std::string("capture end: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&g->level_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(GBC_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    g->g_parents = parents;
    g->g_levels = levels;
    g->g_policy = g->policy;
    if (g->loop_exec) cudaGraphExecDestroy(g->loop_exec);
    g->loop_exec = nullptr;
    // the whole traversal as one while node (replays of the level graph with
    // a host check every few levels remain the path where the CUDA driver cannot
    // build conditional nodes)
    loop_graph([&](cudaStream_t cs, cudaGraphConditionalHandle h) { return launch_level(g, parents, levels, cs, h, 1); },
               true, g->ctl + CTL_NF, g->ctl + CTL_ITER, g->n + 2, &g->loop_exec, &g->loop_kernels);
    return GBC_OK;
}

// One BFS from `source`; parents/levels are device arrays of n entries.
static int bfs_device(Graph *g, int64_t source, int64_t *parents, int64_t *levels, gbc_bfs_stats *st,
                      bool use_graph)
{
    Context *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    GBC_TRY(graph_alloc_bfs(g));
    cudaEventRecord(ctx->ev[5], s);
    k_bfs_init<<<ctx->num_sms * 4, 256, 0, s>>>(g->n, g->nnz, g->cand, g->visited, parents, levels, source, g->cp,
                                                g->ctl, fronts_dev(g), fbits_dev(g));
    k_bfs_init2<<<1, 1, 0, s>>>(g->n, g->nnz, levels, source, g->cp, g->ctl, fronts_dev(g), fbits_dev(g),
                                g->policy);
    note_launches(2);
    GBC_CUDA_TRY(cudaGetLastError());
    if (use_graph) GBC_TRY(level_graph(g, parents, levels));
    if (use_graph && g->loop_exec) {
        GBC_CUDA_TRY(cudaGraphLaunch(g->loop_exec, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(g->h_ctl, g->ctl, kCtlWords * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
        note_launches(g->loop_kernels * std::max<int64_t>(g->h_ctl[CTL_ITER], 1));
    }
    // Otherwise levels are replayed in batches; a finished BFS leaves nf == 0
    // and the remaining replays of the batch are empty launches.
    const int batch = 4;
    int64_t checks = 0;
    for (int64_t lvl = 0; !(use_graph && g->loop_exec) && lvl <= g->n + 1; lvl += batch, ++checks) {
        for (int k = 0; k < batch; ++k) {
            if (use_graph) {
                GBC_CUDA_TRY(cudaGraphLaunch(g->level_exec, s));
                note_launches(g->level_kernels);
            } else {
                GBC_TRY(launch_level(g, parents, levels, s, 0, 0));
            }
        }
        GBC_CUDA_TRY(cudaMemcpyAsync(g->h_ctl, g->ctl, kCtlWords * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
        if (g->h_ctl[CTL_NF] == 0) break;
    }
    cudaEventRecord(ctx->ev[6], s);
    GBC_CUDA_TRY(cudaEventSynchronize(ctx->ev[6]));
    if (st) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]);
        st->iterations = g->h_ctl[CTL_ITER];
        st->reached = g->h_ctl[CTL_REACHED];
        st->edges = g->h_ctl[CTL_EDGES] / 2;
        st->ms = ms;
        st->host_checks = checks;
    }
    return GBC_OK;
}

// ------------------------------------------------------ multi-source BFS
// Many BFS trees at once, the Select2ndMin SpGEMM loop of the reference's
// multi-source traversals (Applications/Ordering/MD.cpp:211-217,
// Applications/BetwCent.cpp:185-186):
//     F_{l+1} = (A * F_l) masked by the complement of visited,
// where column r of F holds root r's frontier with every value equal to its
// own row id, so (A*F)(u, r) = min over frontier neighbours v of v: the
// parent.  Because min is order independent the masked product can go
// straight into a dense per-(root, vertex) accumulator (cand, atomicMin)
// with the visited test in front of it -- no symbolic pass and no output
// sizing -- and every (root, vertex) entering the next frontier is appended
// once (the atomicMin that saw the empty candidate).  F is held as a list
// of (root << 32 | vertex) entries; blocks take fixed chunks of it and
// flatten their edges across the block.
enum {
    MS_NF = 0,       // current frontier entries
    MS_NNEXT = 1,    // next frontier entries
    MS_LEVEL = 2,    // levels done
    MS_WORK = 3,     // chunk counter of the expand kernel
    MS_EDGES = 4,    // sum of degrees of reached (root, vertex) pairs
    MS_REACHED = 5,  // reached (root, vertex) pairs
    MS_CUR = 6,      // which frontier buffer is current
    MS_ROOTS = 7,    // roots of this traversal
    MS_N
};
// Traversals of at most this many roots keep each frontier sorted by root
// (a counting sort after the expansion): the blocks in flight then work on
// a few roots' slices of cand / visited, which stay in L2, instead of
// touching every root's slice at random.
constexpr int64_t kMsSortRoots = 4096;
constexpr int kMsCtlWords = 8;  // then the frontier pointer table [2]

__global__ void __launch_bounds__(kThreads) k_ms_expand(const uint32_t *cp32, const int32_t *row, int64_t n,
                                                        const uint32_t *visited, int32_t *cand, int64_t *ctl,
                                                        int64_t *const *fronts)
{
    __shared__ int32_t s_v[kThreads];
    __shared__ int64_t s_root[kThreads];
    __shared__ int64_t s_base[kThreads];  // root * n
    __shared__ uint32_t s_st[kThreads];
    __shared__ int32_t s_off[kThreads + 1];
    __shared__ int64_t q[kQueue];
    __shared__ int s_qn;
    __shared__ unsigned long long s_gbase;
    __shared__ int64_t s_chunk;
    const int tid = threadIdx.x, lane = tid & 31;
    const int cur = (int)ctl[MS_CUR];
    const int64_t *front = fronts[cur];
    int64_t *next = fronts[cur ^ 1];
    const int64_t nf = ctl[MS_NF];
    if (tid == 0) s_qn = 0;
    __syncthreads();
    for (;;) {
        if (tid == 0) s_chunk = (int64_t)atomicAdd((unsigned long long *)&ctl[MS_WORK], 1ull);
        __syncthreads();
        const int64_t f = s_chunk * kThreads + tid;
        if (s_chunk * kThreads >= nf) break;
        int len = 0;
        if (f < nf) {
            const int64_t x = front[f];
            const int32_t v = (int32_t)(x & 0xffffffff);
            s_v[tid] = v;
            s_root[tid] = x >> 32;
            s_base[tid] = (x >> 32) * n;
            s_st[tid] = cp32[v];
            len = (int)(cp32[v + 1] - cp32[v]);
        }
        int64_t tot;
        const int off = (int)block_exclusive_sum64(len, &tot);
        s_off[tid] = off;
        if (tid == kThreads - 1) s_off[kThreads] = off + len;
        __syncthreads();
        const int L = (int)tot;
        for (int e0 = 0; e0 < L; e0 += kThreads) {
            const int e = e0 + tid;
            bool fresh = false;
            int64_t entry = 0;
            if (e < L) {
                int lo = 0, hi = kThreads;
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (s_off[mid] <= e) lo = mid; else hi = mid;
                }
                const int32_t u = row[s_st[lo] + (e - s_off[lo])];
                const int64_t idx = s_base[lo] + u;
                if (!(visited[idx >> 5] & (1u << (idx & 31)))) {
                    const int32_t v = s_v[lo];
                    if (v < cand[idx]) {
                        const int32_t old = atomicMin(&cand[idx], v);
                        fresh = old == kNoCand;
                        entry = (s_root[lo] << 32) | (uint32_t)u;
                    }
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, fresh);
            if (m) {
                int slot = 0;
                if (lane == __ffs(m) - 1) slot = atomicAdd(&s_qn, __popc(m));
                slot = __shfl_sync(0xffffffffu, slot, __ffs(m) - 1);
                if (fresh) q[slot + __popc(m & ((1u << lane) - 1))] = entry;
            }
            __syncthreads();
            if (s_qn > kQueue - kThreads) {
                if (tid == 0) s_gbase = atomicAdd((unsigned long long *)&ctl[MS_NNEXT], (unsigned long long)s_qn);
                __syncthreads();
                for (int k = tid; k < s_qn; k += kThreads) next[s_gbase + k] = q[k];
                __syncthreads();
                if (tid == 0) s_qn = 0;
                __syncthreads();
            }
        }
        __syncthreads();
    }
    if (s_qn > 0) {
        if (tid == 0) s_gbase = atomicAdd((unsigned long long *)&ctl[MS_NNEXT], (unsigned long long)s_qn);
        __syncthreads();
        for (int k = tid; k < s_qn; k += kThreads) next[s_gbase + k] = q[k];
    }
}

// Counting sort of the next frontier by root into the current buffer (its
// entries are consumed): the root counts of contiguous slices (one per
// block, counted in shared memory) are added up, scanned, and every block
// reserves its range of each root once and scatters into it.  The order
// inside one root is arbitrary (the product is a min, order-free).
__global__ void __launch_bounds__(256) k_ms_rhist(const int64_t *ctl, int64_t *const *fronts, int64_t *rcnt)
{
    extern __shared__ int32_t s_hist[];  // [roots]
    const int64_t R = ctl[MS_ROOTS], nn = ctl[MS_NNEXT];
    const int64_t *next = fronts[ctl[MS_CUR] ^ 1];
    for (int64_t r = threadIdx.x; r < R; r += blockDim.x) s_hist[r] = 0;
    __syncthreads();
    const int64_t per = (nn + gridDim.x - 1) / gridDim.x;
    const int64_t i0 = int64_t(blockIdx.x) * per, i1 = min(nn, i0 + per);
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) atomicAdd(&s_hist[next[i] >> 32], 1);
    __syncthreads();
    for (int64_t r = threadIdx.x; r < R; r += blockDim.x)
        if (s_hist[r]) atomicAdd((unsigned long long *)&rcnt[r], (unsigned long long)s_hist[r]);
}

__global__ void k_ms_rscan(const int64_t *ctl, int64_t *rcnt, int64_t *roff)
{
    const int64_t R = ctl[MS_ROOTS];
    int64_t carry = 0;
    for (int64_t b = 0; b < R; b += kThreads) {
        const int64_t r = b + threadIdx.x;
        const int64_t v = r < R ? rcnt[r] : 0;
        int64_t tot;
        const int64_t ex = block_exclusive_sum64(v, &tot);
        if (r < R) {
            roff[r] = carry + ex;
            rcnt[r] = 0;  // ready for the next level
        }
        carry += tot;
    }
}

__global__ void __launch_bounds__(256) k_ms_rscatter(const int64_t *ctl, int64_t *const *fronts, int64_t *roff)
{
    extern __shared__ int64_t s_base[];  // [roots] then int32 counts [roots]
    const int64_t R = ctl[MS_ROOTS], nn = ctl[MS_NNEXT];
    int32_t *s_cnt = reinterpret_cast<int32_t *>(s_base + R);
    const int cur = (int)ctl[MS_CUR];
    const int64_t *next = fronts[cur ^ 1];
    int64_t *out = fronts[cur];
    for (int64_t r = threadIdx.x; r < R; r += blockDim.x) s_cnt[r] = 0;
    __syncthreads();
    const int64_t per = (nn + gridDim.x - 1) / gridDim.x;
    const int64_t i0 = int64_t(blockIdx.x) * per, i1 = min(nn, i0 + per);
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) atomicAdd(&s_cnt[next[i] >> 32], 1);
    __syncthreads();
    for (int64_t r = threadIdx.x; r < R; r += blockDim.x) {
        const int c = s_cnt[r];
        if (c) s_base[r] = (int64_t)atomicAdd((unsigned long long *)&roff[r], (unsigned long long)c);
        s_cnt[r] = 0;
    }
    __syncthreads();
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int64_t x = next[i];
        const int64_t r = x >> 32;
        out[s_base[r] + atomicAdd(&s_cnt[r], 1)] = x;
    }
}

// parents.Set(fringe) for the new frontier entries, visited update and the
// reached-edge sums.  `sorted`: the entries were sorted into the current
// buffer.
__global__ void k_ms_finalize(int32_t *cand, uint32_t *visited, int64_t *parents, const uint32_t *cp32, int64_t n,
                              int64_t *ctl, int64_t *const *fronts, int sorted)
{
    const int64_t *next = fronts[ctl[MS_CUR] ^ (sorted ? 0 : 1)];
    const int64_t nn = ctl[MS_NNEXT];
    int64_t deg = 0, reached = 0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nn; i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t x = next[i];
        const int32_t u = (int32_t)(x & 0xffffffff);
        const int64_t idx = (x >> 32) * n + u;
        parents[idx] = cand[idx];
        cand[idx] = kNoCand;
        atomicOr(&visited[idx >> 5], 1u << (idx & 31));
        deg += cp32[u + 1] - cp32[u];
        ++reached;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        deg += __shfl_xor_sync(0xffffffffu, deg, o);
        reached += __shfl_xor_sync(0xffffffffu, reached, o);
    }
    if ((threadIdx.x & 31) == 0 && reached) {
        atomicAdd((unsigned long long *)&ctl[MS_EDGES], (unsigned long long)deg);
        atomicAdd((unsigned long long *)&ctl[MS_REACHED], (unsigned long long)reached);
    }
}

__global__ void k_ms_advance(int64_t *ctl, int sorted)
{
    if (ctl[MS_NF] == 0) return;
    ctl[MS_NF] = ctl[MS_NNEXT];
    ctl[MS_NNEXT] = 0;
    ctl[MS_WORK] = 0;
    if (!sorted) ctl[MS_CUR] ^= 1;  // a sorted frontier is already in the current buffer
    ctl[MS_LEVEL] += 1;
}

// Roots: frontier entries, visited bits, parents[root] = root (as the
// reference's visited matrix starts with the sources), degree sums.
__global__ void k_ms_init(const int64_t *roots, int64_t nroots, int64_t n, const uint32_t *cp32, uint32_t *visited,
                          int64_t *parents, int64_t *ctl, int64_t *const *fronts)
{
    const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= nroots) return;
    const int64_t v = roots[r];
    const int64_t idx = r * n + v;
    fronts[0][r] = (r << 32) | v;
    parents[idx] = v;
    atomicOr(&visited[idx >> 5], 1u << (idx & 31));
    atomicAdd((unsigned long long *)&ctl[MS_EDGES], (unsigned long long)(cp32[v + 1] - cp32[v]));
    atomicAdd((unsigned long long *)&ctl[MS_REACHED], 1ull);
}

__global__ void k_fill_i32(int32_t *p, int64_t n, int32_t v)
{
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        p[i] = v;
}

static int64_t *const *ms_fronts_dev(Graph *g) { return reinterpret_cast<int64_t *const *>(g->ms_ctl + kMsCtlWords); }

static void ms_free(Graph *g)
{
    Context *c = g->ctx;
    if (g->ms_exec) cudaGraphExecDestroy(g->ms_exec);
    g->ms_exec = nullptr;
    if (g->ms_loop_exec) cudaGraphExecDestroy(g->ms_loop_exec);
    g->ms_loop_exec = nullptr;
    device_free(c, g->ms_cand);
    device_free(c, g->ms_visited);
    device_free(c, g->ms_front[0]);
    device_free(c, g->ms_front[1]);
    device_free(c, g->ms_ctl);
    device_free(c, g->ms_rcnt);
    device_free(c, g->ms_roff);
    g->ms_rcnt = g->ms_roff = nullptr;
    if (g->h_ms_ctl) cudaFreeHost(g->h_ms_ctl);
    g->ms_cand = nullptr;
    g->ms_visited = nullptr;
    g->ms_front[0] = g->ms_front[1] = nullptr;
    g->ms_ctl = nullptr;
    g->h_ms_ctl = nullptr;
    g->ms_roots = 0;
}

static int ms_alloc(Graph *g, int64_t nroots)
{
    if (g->ms_roots >= nroots) return GBC_OK;
    cudaStreamSynchronize(g->ctx->stream);
    ms_free(g);
    Context *ctx = g->ctx;
    const int64_t cells = nroots * g->n;
    GBC_TRY(device_alloc(ctx, (void **)&g->ms_cand, cells * sizeof(int32_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->ms_visited, ((cells + 31) / 32 + 1) * sizeof(uint32_t)));
    // a (root, vertex) pair enters a frontier at most once
    GBC_TRY(device_alloc(ctx, (void **)&g->ms_front[0], cells * sizeof(int64_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->ms_front[1], cells * sizeof(int64_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->ms_ctl, (kMsCtlWords + 4) * sizeof(int64_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->ms_rcnt, (nroots + 1) * sizeof(int64_t)));
    GBC_TRY(device_alloc(ctx, (void **)&g->ms_roff, (nroots + 1) * sizeof(int64_t)));
    GBC_CUDA_TRY(cudaMemsetAsync(g->ms_rcnt, 0, (nroots + 1) * sizeof(int64_t), ctx->stream));
    GBC_CUDA_TRY(cudaMallocHost(&g->h_ms_ctl, (kMsCtlWords + 4) * sizeof(int64_t)));
    void *tab[2] = {g->ms_front[0], g->ms_front[1]};
    GBC_CUDA_TRY(cudaMemcpyAsync(g->ms_ctl + kMsCtlWords, tab, sizeof(tab), cudaMemcpyHostToDevice, ctx->stream));
    k_fill_i32<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(g->ms_cand, cells, kNoCand);
    note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    g->ms_roots = nroots;
    return GBC_OK;
}

static int ms_launch_level(Graph *g, int64_t *parents, cudaStream_t s)
{
    const int grid = g->ctx->num_sms * 4;
    const int sorted = g->ms_roots <= kMsSortRoots ? 1 : 0;
    k_ms_expand<<<occ_grid(g->ctx, (const void *)k_ms_expand, kThreads, 0), kThreads, 0, s>>>(g->cp32, g->row, g->n, g->ms_visited, g->ms_cand, g->ms_ctl,
                                          ms_fronts_dev(g));
    note_launch();
    if (sorted) {
        k_ms_rhist<<<grid, 256, g->ms_roots * sizeof(int32_t), s>>>(g->ms_ctl, ms_fronts_dev(g), g->ms_rcnt);
        k_ms_rscan<<<1, kThreads, 0, s>>>(g->ms_ctl, g->ms_rcnt, g->ms_roff);
        k_ms_rscatter<<<grid, 256, g->ms_roots * (sizeof(int64_t) + sizeof(int32_t)), s>>>(
            g->ms_ctl, ms_fronts_dev(g), g->ms_roff);
        note_launches(3);
    }
    k_ms_finalize<<<occ_grid(g->ctx, (const void *)k_ms_finalize, 256, 0), 256, 0, s>>>(
        g->ms_cand, g->ms_visited, parents, g->cp32, g->n, g->ms_ctl,
                                       ms_fronts_dev(g), sorted);
    k_ms_advance<<<1, 1, 0, s>>>(g->ms_ctl, sorted);
    note_launches(2);
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

static int ms_level_graph(Graph *g, int64_t *parents)
{
    if (g->ms_exec && g->ms_g_parents == parents) return GBC_OK;
    if (g->ms_exec) {
        cudaGraphExecDestroy(g->ms_exec);
        g->ms_exec = nullptr;
    }
    cudaStream_t cs;
    GBC_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph;
    const long long c0 = launch_count();
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(cs);
        return fail(GBC_ECUDA, std::string("capture: ") + cudaGetErrorString(e));
    }
    int rc = ms_launch_level(g, parents, cs);
    e = cudaStreamEndCapture(cs, &graph);
    g->ms_kernels = launch_count() - c0;
    note_launches(-g->ms_kernels);
    cudaStreamDestroy(cs);
    if (rc != GBC_OK) return rc;
    if (e != cudaSuccess) return fail(GBC_ECUDA, std::string("capture end: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&g->ms_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(GBC_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    g->ms_g_parents = parents;
    if (g->ms_loop_exec) cudaGraphExecDestroy(g->ms_loop_exec);
    g->ms_loop_exec = nullptr;
    loop_graph([&](cudaStream_t cs, cudaGraphConditionalHandle) { return ms_launch_level(g, parents, cs); }, false,
               g->ms_ctl + MS_NF, g->ms_ctl + MS_LEVEL, g->n + 2, &g->ms_loop_exec, &g->ms_loop_kernels);
    return GBC_OK;
}

// parents: device [nroots * n], root-major.
static int msbfs_device(Graph *g, const int64_t *d_roots, int64_t nroots, int64_t *parents, gbc_msbfs_stats *st)
{
    Context *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    GBC_TRY(ms_alloc(g, nroots));
    const int64_t cells = nroots * g->n;
    cudaEventRecord(ctx->ev[5], s);
    GBC_CUDA_TRY(cudaMemsetAsync(parents, 0xff, cells * sizeof(int64_t), s));  // -1: unreached
    GBC_CUDA_TRY(cudaMemsetAsync(g->ms_visited, 0, ((cells + 31) / 32 + 1) * sizeof(uint32_t), s));
    GBC_CUDA_TRY(cudaMemsetAsync(g->ms_ctl, 0, kMsCtlWords * sizeof(int64_t), s));
    k_ms_init<<<(unsigned)((nroots + 255) / 256), 256, 0, s>>>(d_roots, nroots, g->n, g->cp32, g->ms_visited,
                                                                parents, g->ms_ctl, ms_fronts_dev(g));
    note_launch();
    int64_t nf = nroots;
    GBC_CUDA_TRY(cudaMemcpyAsync(g->ms_ctl + MS_NF, &nf, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    GBC_CUDA_TRY(cudaMemcpyAsync(g->ms_ctl + MS_ROOTS, &nf, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    GBC_CUDA_TRY(cudaGetLastError());
    GBC_TRY(ms_level_graph(g, parents));
    if (g->ms_loop_exec) {
        GBC_CUDA_TRY(cudaGraphLaunch(g->ms_loop_exec, s));
        GBC_CUDA_TRY(
            cudaMemcpyAsync(g->h_ms_ctl, g->ms_ctl, kMsCtlWords * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
        note_launches(g->ms_loop_kernels * std::max<int64_t>(g->h_ms_ctl[MS_LEVEL], 1));
    }
    const int batch = 2;
    int64_t checks = 0;
    for (int64_t lvl = 0; !g->ms_loop_exec && lvl <= g->n + 1; lvl += batch, ++checks) {
        for (int k = 0; k < batch; ++k) {
            GBC_CUDA_TRY(cudaGraphLaunch(g->ms_exec, s));
            note_launches(g->ms_kernels);
        }
        GBC_CUDA_TRY(
            cudaMemcpyAsync(g->h_ms_ctl, g->ms_ctl, kMsCtlWords * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
        if (g->h_ms_ctl[MS_NF] == 0) break;
    }
    cudaEventRecord(ctx->ev[6], s);
    GBC_CUDA_TRY(cudaEventSynchronize(ctx->ev[6]));
    if (st) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]);
        st->levels = g->h_ms_ctl[MS_LEVEL];
        st->reached = g->h_ms_ctl[MS_REACHED];
        st->edges = g->h_ms_ctl[MS_EDGES] / 2;
        st->ms = ms;
        st->host_checks = checks;
    }
    return GBC_OK;
}

}  // namespace gbc

using namespace gbc;

struct gbc_graph : gbc::Graph {};

extern "C" {

int gbc_graph_create(gbc_context *ctx, const gbc_matrix *Am, gbc_graph **out)
{
    if (!ctx || !Am || !out) return fail(GBC_EINVAL, "null argument");
    *out = nullptr;
    if (Am->nrow != Am->ncol) return fail(GBC_EINVAL, "graph matrix must be square");
    if (Am->jc) return fail(GBC_EINVAL, "graph matrix must be CSC (jc == NULL)");
    if (Am->nnz >= (int64_t(1) << 32)) return fail(GBC_EOVERFLOW, "nnz must be below 2^32");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    Workspace ws(ctx);
    DevMatrix A;
    GBC_TRY(upload(ws, Am, GBC_BOOL, &A));
    gbc_graph *g = new gbc_graph();
    g->ctx = ctx;
    g->n = A.ncol;
    g->nnz = A.nnz;
    int rc = device_alloc(ctx, (void **)&g->cp, (g->n + 1) * sizeof(int64_t));
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&g->cp32, (g->n + 1) * sizeof(uint32_t));
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&g->row, (g->nnz + 1) * sizeof(int32_t));
    int32_t *err = nullptr;
    if (rc == GBC_OK) rc = ws.alloc_n(&err, 1);
    if (rc != GBC_OK) {
        gbc_graph_destroy(g);
        return rc;
    }
    cudaStream_t s = ctx->stream;
    cudaMemsetAsync(err, 0, sizeof(int32_t), s);
    cudaMemcpyAsync(g->cp, A.cp, (g->n + 1) * sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
    if (g->n > 0)
        k_graph_prep<<<ctx->num_sms * 8, 256, 0, s>>>(g->n, g->nnz, A.cp, A.ir, g->cp32, g->row, err); ::gbc::note_launch();
    int32_t herr = 0;
    cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess || herr) {
        gbc_graph_destroy(g);
        return e != cudaSuccess ? fail(GBC_ECUDA, cudaGetErrorString(e))
                                : fail(GBC_EINVAL, "malformed graph matrix (column pointers or row ids)");
    }
    *out = g;
    return GBC_OK;
}

int gbc_graph_destroy(gbc_graph *g)
{
    if (!g) return GBC_OK;
    Context *c = g->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (g->level_exec) cudaGraphExecDestroy(g->level_exec);
    if (g->loop_exec) cudaGraphExecDestroy(g->loop_exec);
    ms_free(g);
    device_free(c, g->cp);
    device_free(c, g->cp32);
    device_free(c, g->row);
    device_free(c, g->cand);
    device_free(c, g->visited);
    device_free(c, g->front[0]);
    device_free(c, g->front[1]);
    device_free(c, g->fbits[0]);
    device_free(c, g->fbits[1]);
    device_free(c, g->off);
    device_free(c, g->tile);
    device_free(c, g->chunk_f0);
    device_free(c, g->ctl);
    device_free(c, g->own_parents);
    device_free(c, g->own_levels);
    if (g->h_ctl) cudaFreeHost(g->h_ctl);
    cudaStreamSynchronize(c->stream);
    delete g;
    return GBC_OK;
}

int gbc_graph_set_policy(gbc_graph *g, int policy)
{
    if (!g || policy < 0 || policy > 2) return fail(GBC_EINVAL, "bad graph or policy");
    g->policy = policy;
    return GBC_OK;
}

int gbc_spmspv_select2ndmin_i64(gbc_context *ctx, gbc_graph *g, const int32_t *indx, const int64_t *numx,
                                int32_t veclen, int32_t *indy, int64_t *numy, int32_t *nnzy, int where)
{
    if (!ctx || !g || !nnzy) return fail(GBC_EINVAL, "null argument");
    if (veclen < 0) return fail(GBC_EINVAL, "negative vector length");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    const int32_t *dx = indx;
    const int64_t *dv = numx;
    if (where == GBC_HOST && veclen > 0) {
        int32_t *a = nullptr;
        int64_t *b = nullptr;
        GBC_TRY(ws.alloc_n(&a, veclen));
        GBC_TRY(ws.alloc_n(&b, veclen));
        GBC_CUDA_TRY(cudaMemcpyAsync(a, indx, veclen * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(b, numx, veclen * sizeof(int64_t), cudaMemcpyHostToDevice, s));
        dx = a;
        dv = b;
    }
    const int64_t words = (g->n + 31) / 32;
    unsigned long long *spa = nullptr;
    uint32_t *mark = nullptr;
    int64_t *pos = nullptr;
    unsigned long long *work = nullptr;
    int32_t *err = nullptr;
    GBC_TRY(ws.alloc_n(&err, 1));
    GBC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int32_t), s));
    GBC_TRY(ws.alloc_n(&spa, g->n + 1));
    GBC_TRY(ws.alloc_n(&mark, words + 1));
    GBC_TRY(ws.alloc_n(&pos, words + 1));
    GBC_TRY(ws.alloc_n(&work, 1));
    GBC_CUDA_TRY(cudaMemsetAsync(spa, 0xff, g->n * sizeof(unsigned long long), s));
    GBC_CUDA_TRY(cudaMemsetAsync(mark, 0, words * sizeof(uint32_t), s));
    GBC_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(unsigned long long), s));
    // indices must address columns of A
    if (veclen > 0) {
        k_spmspv_expand<<<std::min<int64_t>(ctx->num_sms * 4, (veclen + kThreads - 1) / kThreads), kThreads, 0, s>>>(
            g->cp32, g->row, dx, dv, veclen, g->n, spa, mark, work, err); ::gbc::note_launch();
        int32_t herr = 0;
        GBC_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
        if (herr) return fail(GBC_EINVAL, "vector index out of range");
    }
    if (words > 0) {
        k_mark_counts<<<(unsigned)((words + 255) / 256), 256, 0, s>>>(mark, words, pos); ::gbc::note_launch();
        GBC_TRY(exclusive_scan_i64(ws, pos, pos, words, s));
    }
    int64_t ny = 0;
    if (words > 0) GBC_TRY(read_i64(ctx, pos + words, &ny));
    int32_t *yi = indy;
    int64_t *yv = numy;
    if (where == GBC_HOST) {
        GBC_TRY(ws.alloc_n(&yi, ny + 1));
        GBC_TRY(ws.alloc_n(&yv, ny + 1));
    }
    if (words > 0) k_mark_emit<<<(unsigned)((words + 255) / 256), 256, 0, s>>>(mark, words, pos, spa, yi, yv); ::gbc::note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    if (where == GBC_HOST && ny > 0) {
        GBC_CUDA_TRY(cudaMemcpyAsync(indy, yi, ny * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(numy, yv, ny * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    }
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    *nnzy = (int32_t)ny;
    return GBC_OK;
}

int gbc_bfs(gbc_context *ctx, gbc_graph *g, int64_t source, int64_t *parents, int64_t *levels,
            gbc_bfs_stats *st, int where)
{
    if (!ctx || !g) return fail(GBC_EINVAL, "null argument");
    if (source < 0 || source >= g->n) return fail(GBC_EINVAL, "source out of range");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    g->ctx = ctx;
    GBC_TRY(graph_alloc_bfs(g));
    int64_t *dp = parents, *dl = levels;
    if (where == GBC_HOST || !parents || !levels) {
        // the graph's own device outputs: the captured traversal is reused
        dp = g->own_parents;
        dl = g->own_levels;
    }
    GBC_TRY(bfs_device(g, source, dp, dl, st, true));
    if (where == GBC_HOST) {
        if (parents) GBC_CUDA_TRY(cudaMemcpyAsync(parents, dp, g->n * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        if (levels) GBC_CUDA_TRY(cudaMemcpyAsync(levels, dl, g->n * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return GBC_OK;
}

int gbc_msbfs(gbc_context *ctx, gbc_graph *g, const int64_t *roots, int64_t nroots, int64_t *parents, int where,
              gbc_msbfs_stats *st)
{
    if (!ctx || !g || !roots || !parents) return fail(GBC_EINVAL, "null argument");
    if (nroots <= 0 || nroots >= (int64_t(1) << 31)) return fail(GBC_EINVAL, "root count out of range");
    if (where != GBC_HOST && where != GBC_DEVICE) return fail(GBC_EINVAL, "bad memory location");
    if (g->n >= (int64_t(1) << 31) || nroots > (int64_t(1) << 62) / std::max<int64_t>(g->n, 1))
        return fail(GBC_EOVERFLOW, "roots x vertices too large");
    for (int64_t r = 0; r < nroots; ++r)
        if (roots[r] < 0 || roots[r] >= g->n) return fail(GBC_EINVAL, "root out of range");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    g->ctx = ctx;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    int64_t *d_roots = nullptr;
    GBC_TRY(ws.alloc_n(&d_roots, nroots));
    GBC_CUDA_TRY(cudaMemcpyAsync(d_roots, roots, nroots * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    const int64_t cells = nroots * g->n;
    int64_t *dp = parents;
    if (where == GBC_HOST) GBC_TRY(ws.alloc_n(&dp, cells));
    GBC_TRY(msbfs_device(g, d_roots, nroots, dp, st));
    if (where == GBC_HOST) {
        GBC_CUDA_TRY(cudaMemcpyAsync(parents, dp, cells * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return GBC_OK;
}

}  // extern "C"
