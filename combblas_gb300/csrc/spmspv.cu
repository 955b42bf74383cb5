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
    int64_t *ctl = nullptr;  // device control block (see CTL_*)
    int64_t *h_ctl = nullptr;  // pinned mirror
    cudaGraphExec_t level_exec = nullptr;
    long long level_kernels = 0;  // kernels one replay of the level graph runs
    int64_t *g_parents = nullptr, *g_levels = nullptr;  // pointers baked into the graph
    bool bfs_ready = false;
};

// control block layout
enum { CTL_NF = 0, CTL_NNEXT = 1, CTL_ITER = 2, CTL_WORK = 3, CTL_EDGES = 4, CTL_REACHED = 5, CTL_CUR = 6, CTL_N };

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

// Warp-aggregated append of `r` (where `want`) to list[*count].
__device__ __forceinline__ void warp_append(bool want, int32_t r, int32_t *list, int64_t *count)
{
    unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd((unsigned long long *)count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (want) list[base + __popc(m & ((1u << lane) - 1))] = r;
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
// Expand one level: for every column c of the frontier (value c, as after
// setNumToInd) and every row r of A(:,c) not yet visited, cand[r] = min(c);
// a row touched for the first time joins the next frontier.  New frontier
// rows are gathered in a block-local queue and flushed with one global
// atomic per kQueue entries (a single global counter per warp would
// serialise on hot levels).
constexpr int kQueue = 4096;

__global__ void __launch_bounds__(kThreads) k_bfs_expand(const uint32_t *cp32, const int32_t *row,
                                                         const uint32_t *visited, int32_t *cand, int64_t *ctl,
                                                         int32_t *const *fronts)
{
    __shared__ FrontChunk ch;
    __shared__ int64_t s_base;
    __shared__ int32_t q[kQueue];
    __shared__ int s_qn;
    __shared__ unsigned long long s_gbase;
    const int tid = threadIdx.x, lane = tid & 31;
    const int cur = (int)ctl[CTL_CUR];
    const int32_t *front = fronts[cur];
    int32_t *next = fronts[cur ^ 1];
    const int64_t nf = ctl[CTL_NF];
    if (tid == 0) s_qn = 0;
    __syncthreads();
    auto flush = [&]() {
        // all threads: move the queue to the global frontier
        const int qn = s_qn;
        if (qn > 0) {
            if (tid == 0) s_gbase = atomicAdd((unsigned long long *)&ctl[CTL_NNEXT], (unsigned long long)qn);
            __syncthreads();
            for (int k = tid; k < qn; k += kThreads) next[s_gbase + k] = q[k];
            __syncthreads();
            if (tid == 0) s_qn = 0;
        }
        __syncthreads();
    };
    for (;;) {
        if (tid == 0) s_base = (int64_t)atomicAdd((unsigned long long *)&ctl[CTL_WORK], (unsigned long long)kThreads);
        __syncthreads();
        const int64_t base = s_base;
        __syncthreads();
        if (base >= nf) break;
        const int64_t f = base + tid;
        int len = 0;
        if (f < nf) {
            const int32_t c = front[f];
            const uint32_t s = cp32[c];
            ch.s[tid] = s;
            ch.val[tid] = c;
            len = (int)(cp32[c + 1] - s);
        }
        int64_t tot;
        const int off = (int)block_exclusive_sum64(len, &tot);
        ch.off[tid] = off;
        if (tid == kThreads - 1) ch.off[kThreads] = off + len;
        __syncthreads();
        const int iters = ((int)tot + kThreads - 1) / kThreads;
        for (int it = 0; it < iters; ++it) {
            const int j = it * kThreads + tid;
            bool fresh = false;
            int32_t r = 0;
            if (j < (int)tot) {
                const int b = front_find(ch, j);
                r = row[ch.s[b] + (j - ch.off[b])];
                if (!(visited[r >> 5] & (1u << (r & 31)))) {
                    const int32_t c = (int32_t)ch.val[b];
                    // skip the atomic when the stored candidate is already smaller
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
            __syncthreads();
            if (s_qn > kQueue - kThreads) flush();
        }
        __syncthreads();
    }
    flush();
}

// parents.Set(fringe) for the new frontier; visited/levels/degree sums.
__global__ void k_bfs_finalize(int32_t *cand, uint32_t *visited, int64_t *parents, int64_t *levels,
                               const int64_t *cp, int64_t *ctl, int32_t *const *fronts)
{
    const int cur = (int)ctl[CTL_CUR];
    const int32_t *next = fronts[cur ^ 1];
    const int64_t nn = ctl[CTL_NNEXT];
    const int64_t iter = ctl[CTL_ITER] + 1;
    int64_t deg = 0, reached = 0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nn; i += int64_t(gridDim.x) * blockDim.x) {
        const int32_t r = next[i];
        parents[r] = cand[r];
        cand[r] = kNoCand;
        atomicOr(&visited[r >> 5], 1u << (r & 31));
        if (levels[r] < 0) {
            levels[r] = iter;
            deg += cp[r + 1] - cp[r];
            ++reached;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        deg += __shfl_xor_sync(0xffffffffu, deg, o);
        reached += __shfl_xor_sync(0xffffffffu, reached, o);
    }
    if ((threadIdx.x & 31) == 0 && (deg || reached)) {
        atomicAdd((unsigned long long *)&ctl[CTL_EDGES], (unsigned long long)deg);
        atomicAdd((unsigned long long *)&ctl[CTL_REACHED], (unsigned long long)reached);
    }
}

// Advance the level: next frontier becomes current.
__global__ void k_bfs_advance(int64_t *ctl)
{
    if (ctl[CTL_NF] == 0) return;  // finished: later replays change nothing
    ctl[CTL_NF] = ctl[CTL_NNEXT];
    ctl[CTL_NNEXT] = 0;
    ctl[CTL_WORK] = 0;
    ctl[CTL_ITER] += 1;
    ctl[CTL_CUR] ^= 1;
}

__global__ void k_bfs_init(int64_t n, int32_t *cand, uint32_t *visited, int64_t *parents, int64_t *levels,
                           int64_t source, const int64_t *cp, int64_t *ctl, int32_t *const *fronts)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t v = i; v < n; v += stride) {
        cand[v] = kNoCand;
        parents[v] = -1;
        levels[v] = -1;
    }
    for (int64_t w = i; w < (n + 31) / 32; w += stride) visited[w] = 0;
    if (i == 0) {
        fronts[0][0] = (int32_t)source;
        ctl[CTL_NF] = 1;
        ctl[CTL_NNEXT] = 0;
        ctl[CTL_ITER] = 0;
        ctl[CTL_WORK] = 0;
        ctl[CTL_EDGES] = cp[source + 1] - cp[source];
        ctl[CTL_REACHED] = 1;
        ctl[CTL_CUR] = 0;
    }
}

__global__ void k_set_source_level(int64_t *levels, int64_t source) { levels[source] = 0; }

// -------------------------------------------------------------- host side
static int graph_alloc_bfs(Graph *g)
{
    Context *ctx = g->ctx;
    if (g->bfs_ready) return GBC_OK;
    GBC_TRY(device_alloc(ctx, (void **)&g->cand, g->n * sizeof(int32_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->visited, ((g->n + 31) / 32) * sizeof(uint32_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->front[0], g->n * sizeof(int32_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->front[1], g->n * sizeof(int32_t) + 16));
    GBC_TRY(device_alloc(ctx, (void **)&g->ctl, 16 * sizeof(int64_t)));
    GBC_CUDA_TRY(cudaMallocHost(&g->h_ctl, 16 * sizeof(int64_t)));
    g->bfs_ready = true;
    return GBC_OK;
}

static int32_t *const *fronts_dev(Graph *g)
{
    // the two frontier pointers, stored right after the control block
    return reinterpret_cast<int32_t *const *>(g->ctl + 8);
}

static int launch_level(Graph *g, int64_t *parents, int64_t *levels, cudaStream_t s)
{
    Context *ctx = g->ctx;
    int grid = ctx->num_sms * 4;
    k_bfs_expand<<<grid, kThreads, 0, s>>>(g->cp32, g->row, g->visited, g->cand, g->ctl, fronts_dev(g)); ::gbc::note_launch();
    k_bfs_finalize<<<ctx->num_sms * 4, 256, 0, s>>>(g->cand, g->visited, parents, levels, g->cp, g->ctl,
                                                    fronts_dev(g)); ::gbc::note_launch();
    k_bfs_advance<<<1, 1, 0, s>>>(g->ctl); ::gbc::note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

// Capture one level into a graph once per (graph, output buffers).
static int level_graph(Graph *g, int64_t *parents, int64_t *levels)
{
    if (g->level_exec && g->g_parents == parents && g->g_levels == levels) return GBC_OK;
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
    int rc = launch_level(g, parents, levels, cs);
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
    return GBC_OK;
}

// One BFS from `source`; parents/levels are device arrays of n entries.
static int bfs_device(Graph *g, int64_t source, int64_t *parents, int64_t *levels, gbc_bfs_stats *st,
                      bool use_graph)
{
    Context *ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    GBC_TRY(graph_alloc_bfs(g));
    // frontier pointer table lives after the control words
    int32_t *fp[2] = {g->front[0], g->front[1]};
    GBC_CUDA_TRY(cudaMemcpyAsync(g->ctl + 8, fp, sizeof(fp), cudaMemcpyHostToDevice, s));
    cudaEventRecord(ctx->ev[5], s);
    k_bfs_init<<<ctx->num_sms * 4, 256, 0, s>>>(g->n, g->cand, g->visited, parents, levels, source, g->cp, g->ctl,
                                                fronts_dev(g)); ::gbc::note_launch();
    k_set_source_level<<<1, 1, 0, s>>>(levels, source); ::gbc::note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    if (use_graph) GBC_TRY(level_graph(g, parents, levels));
    // Levels are replayed in batches; a finished BFS leaves nf == 0 and the
    // remaining replays of the batch are empty launches.
    const int batch = 4;
    for (int64_t lvl = 0; lvl <= g->n + 1; lvl += batch) {
        for (int k = 0; k < batch; ++k) {
            if (use_graph) {
                GBC_CUDA_TRY(cudaGraphLaunch(g->level_exec, s));
                note_launches(g->level_kernels);
            } else {
                GBC_TRY(launch_level(g, parents, levels, s));
            }
        }
        GBC_CUDA_TRY(cudaMemcpyAsync(g->h_ctl, g->ctl, 8 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
        if (g->h_ctl[CTL_NF] == 0) break;
    }
    cudaEventRecord(ctx->ev[6], s);
    GBC_CUDA_TRY(cudaEventSynchronize(ctx->ev[6]));
    if (st) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]);
        // iterations of the reference loop: the last level that produced a
        // nonempty fringe, plus the final (empty) one
        st->iterations = g->h_ctl[CTL_ITER];
        st->reached = g->h_ctl[CTL_REACHED];
        st->edges = g->h_ctl[CTL_EDGES] / 2;
        st->ms = ms;
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
    device_free(c, g->cp);
    device_free(c, g->cp32);
    device_free(c, g->row);
    device_free(c, g->cand);
    device_free(c, g->visited);
    device_free(c, g->front[0]);
    device_free(c, g->front[1]);
    device_free(c, g->ctl);
    if (g->h_ctl) cudaFreeHost(g->h_ctl);
    cudaStreamSynchronize(c->stream);
    delete g;
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
    int64_t *dp = parents, *dl = levels;
    Workspace ws(ctx);
    if (where == GBC_HOST || !parents) GBC_TRY(ws.alloc_n(&dp, g->n));
    if (where == GBC_HOST || !levels) GBC_TRY(ws.alloc_n(&dl, g->n));
    GBC_TRY(bfs_device(g, source, dp, dl, st, where == GBC_DEVICE && parents && levels));
    if (where == GBC_HOST) {
        if (parents) GBC_CUDA_TRY(cudaMemcpyAsync(parents, dp, g->n * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        if (levels) GBC_CUDA_TRY(cudaMemcpyAsync(levels, dl, g->n * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return GBC_OK;
}

}  // extern "C"
