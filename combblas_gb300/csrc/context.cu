// Context, memory, results, uploads and device-wide scans of libgbcomb.
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>

#include "gbc_internal.cuh"

namespace gbc {

static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(); }

void set_error(const std::string &msg) { g_err = msg; }

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

size_t value_size(int vt)
{
    switch (vt) {
        case GBC_F64: return 8;
        case GBC_F32: return 4;
        case GBC_I64: return 8;
        case GBC_BOOL: return 1;
        default: return 0;
    }
}

int device_alloc(Context *ctx, void **p, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(GBC_ENOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed: " +
                                    cudaGetErrorString(e));
    }
    return GBC_OK;
}

void device_free(Context *ctx, void *p)
{
    if (p) cudaFreeAsync(p, ctx->stream);
}

Workspace::~Workspace()
{
    for (void *p : ptrs) device_free(ctx, p);
}

int Workspace::alloc(void **p, size_t bytes)
{
    GBC_TRY(device_alloc(ctx, p, bytes));
    ptrs.push_back(*p);
    return GBC_OK;
}

int read_i64(Context *ctx, const int64_t *dptr, int64_t *out)
{
    int64_t *h = static_cast<int64_t *>(ctx->pinned);
    GBC_CUDA_TRY(cudaMemcpyAsync(h, dptr, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    GBC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *out = *h;
    return GBC_OK;
}

// ------------------------------------------------------------------ upload
template <typename T>
static int put(Workspace &ws, const T *src, size_t n, int where, const T **dst)
{
    if (where == GBC_DEVICE || n == 0) {
        *dst = src;
        return GBC_OK;
    }
    T *d = nullptr;
    GBC_TRY(ws.alloc_n(&d, n));
    GBC_CUDA_TRY(cudaMemcpyAsync(d, src, n * sizeof(T), cudaMemcpyHostToDevice, ws.ctx->stream));
    *dst = d;
    return GBC_OK;
}

int upload(Workspace &ws, const gbc_matrix *M, int vt, DevMatrix *out)
{
    if (!M) return fail(GBC_EINVAL, "null matrix");
    if (M->nrow < 0 || M->ncol < 0 || M->nnz < 0 || M->nzc < 0)
        return fail(GBC_EINVAL, "negative matrix dimension");
    if (!M->jc && M->nzc != M->ncol) return fail(GBC_EINVAL, "CSC matrix needs nzc == ncol");
    if (M->nzc > M->ncol) return fail(GBC_EINVAL, "nzc exceeds ncol");
    if (M->nrow >= (int64_t(1) << 31) || M->ncol >= (int64_t(1) << 31))
        return fail(GBC_EOVERFLOW, "matrix dimensions must be below 2^31");
    if (M->where != GBC_HOST && M->where != GBC_DEVICE) return fail(GBC_EINVAL, "bad `where`");
    if (M->nzc > 0 && !M->cp) return fail(GBC_EINVAL, "missing column pointers");
    if (M->nnz > 0 && !M->ir) return fail(GBC_EINVAL, "missing row ids");
    out->nrow = M->nrow;
    out->ncol = M->ncol;
    out->nzc = M->nzc;
    out->nnz = M->nnz;
    GBC_TRY(put(ws, M->cp, M->nzc + 1, M->where, &out->cp));
    GBC_TRY(put(ws, M->jc, M->jc ? M->nzc : 0, M->where, &out->jc));
    if (!M->jc) out->jc = nullptr;
    GBC_TRY(put(ws, M->ir, M->nnz, M->where, &out->ir));
    if (M->num) {
        size_t vs = value_size(vt);
        const char *d = nullptr;
        GBC_TRY(put(ws, static_cast<const char *>(M->num), M->nnz * vs, M->where, &d));
        out->num = d;
    } else {
        out->num = nullptr;
    }
    return GBC_OK;
}

// ------------------------------------------------------------------- scans
// Exclusive scan in three launches: per-tile sums, a scan of the tile sums
// (recursively), and the per-tile rescan that adds the tile offset.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int64_t block_exclusive_sum(int64_t v, int64_t *total)
{
    __shared__ int64_t warp_sums[SCAN_THREADS / 32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int64_t s = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < SCAN_THREADS / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    int64_t base = wid ? warp_sums[wid - 1] : 0;
    if (total) *total = warp_sums[SCAN_THREADS / 32 - 1];
    __syncthreads();
    return base + x - v;
}

__global__ void k_tile_sums(const int64_t *in, int64_t n, int64_t *sums)
{
    int64_t base = int64_t(blockIdx.x) * SCAN_TILE;
    int64_t s = 0;
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        int64_t idx = base + int64_t(i) * SCAN_THREADS + threadIdx.x;
        if (idx < n) s += in[idx];
    }
    int64_t tot;
    block_exclusive_sum(s, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_tile_scan(const int64_t *in, int64_t *out, int64_t n, const int64_t *offsets)
{
    int64_t base = int64_t(blockIdx.x) * SCAN_TILE;
    int64_t v[SCAN_ITEMS];
    int64_t s = 0;
    // thread owns a contiguous run of SCAN_ITEMS elements
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        int64_t idx = base + int64_t(threadIdx.x) * SCAN_ITEMS + i;
        v[i] = idx < n ? in[idx] : 0;
        s += v[i];
    }
    int64_t tot;
    int64_t run = block_exclusive_sum(s, &tot) + (offsets ? offsets[blockIdx.x] : 0);
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        int64_t idx = base + int64_t(threadIdx.x) * SCAN_ITEMS + i;
        int64_t x = v[i];
        if (idx < n) out[idx] = run;
        run += x;
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_THREADS - 1) out[n] = run;
}

int exclusive_scan_i64(Workspace &ws, const int64_t *in, int64_t *out, int64_t n, cudaStream_t s)
{
    if (n <= 0) {
        GBC_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int64_t), s));
        return GBC_OK;
    }
    int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        k_tile_scan<<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr); ::gbc::note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
        return GBC_OK;
    }
    int64_t *sums = nullptr;
    GBC_TRY(ws.alloc_n(&sums, tiles + 1));
    k_tile_sums<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, sums); ::gbc::note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    GBC_TRY(exclusive_scan_i64(ws, sums, sums, tiles, s));
    k_tile_scan<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, out, n, sums); ::gbc::note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

int64_t scan_tmp_elems(int64_t n)
{
    int64_t t = 0;
    while (n > SCAN_TILE) {
        const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
        t += tiles + 1;
        n = tiles;
    }
    return t + 1;
}

// Same scan with caller-provided temporary storage (scan_tmp_elems(n)
// int64s): no allocation, so it can be captured into a CUDA graph.
int exclusive_scan_i64_tmp(const int64_t *in, int64_t *out, int64_t n, int64_t *tmp, cudaStream_t s)
{
    if (n <= 0) {
        GBC_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int64_t), s));
        return GBC_OK;
    }
    const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        k_tile_scan<<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr);
        note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
        return GBC_OK;
    }
    int64_t *sums = tmp;
    k_tile_sums<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, sums);
    note_launch();
    GBC_TRY(exclusive_scan_i64_tmp(sums, sums, tiles, tmp + tiles + 1, s));
    k_tile_scan<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, out, n, sums);
    note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

}  // namespace gbc

using namespace gbc;

// ===================================================================== C ABI
extern "C" {

const char *gbc_last_error(void) { return g_err.c_str(); }

int gbc_version(void) { return 1; }

int64_t gbc_launch_count(void) { return (int64_t)g_launches.load(); }

int gbc_context_create(gbc_context **out, int device)
{
    if (!out) return fail(GBC_EINVAL, "null output pointer");
    *out = nullptr;
    int ndev = 0;
    GBC_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(GBC_EINVAL, "no such CUDA device");
    GBC_CUDA_TRY(cudaSetDevice(device));
    gbc_context *c = new gbc_context();
    c->device = device;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        delete c;
        return fail(GBC_ECUDA, "cudaGetDeviceProperties failed");
    }
    c->num_sms = prop.multiProcessorCount;
    c->smem_optin = prop.sharedMemPerBlockOptin;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(GBC_ECUDA, "cudaStreamCreate failed");
    }
    c->own_stream = true;
    for (auto &e : c->ev) cudaEventCreate(&e);
    // keep freed pool memory cached across calls
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if (cudaMalloc(&c->d_flag, 8 * sizeof(int32_t)) != cudaSuccess ||
        cudaMallocHost(&c->pinned, 4096) != cudaSuccess) {
        cudaGetLastError();
        gbc_context_destroy(c);
        return fail(GBC_ENOMEM, "context allocation failed");
    }
    cudaMemset(c->d_flag, 0, 8 * sizeof(int32_t));
    *out = c;
    return GBC_OK;
}

int gbc_context_destroy(gbc_context *c)
{
    if (!c) return GBC_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->d_flag) cudaFree(c->d_flag);
    if (c->pinned) cudaFreeHost(c->pinned);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return GBC_OK;
}

int gbc_context_set_fold(gbc_context *c, int fold)
{
    if (!c) return fail(GBC_EINVAL, "null context");
    if (fold != GBC_FOLD_EXACT && fold != GBC_FOLD_ORDERED)
        return fail(GBC_EINVAL, "fold must be GBC_FOLD_EXACT or GBC_FOLD_ORDERED");
    c->fold = fold;
    return GBC_OK;
}

int gbc_context_set_stream(gbc_context *c, void *stream)
{
    if (!c) return fail(GBC_EINVAL, "null context");
    GBC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (stream) {
        if (c->own_stream) cudaStreamDestroy(c->stream);
        c->stream = static_cast<cudaStream_t>(stream);
        c->own_stream = false;
    } else if (!c->own_stream) {
        GBC_CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    return GBC_OK;
}

int gbc_context_synchronize(gbc_context *c)
{
    if (!c) return fail(GBC_EINVAL, "null context");
    GBC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return GBC_OK;
}

int gbc_result_info(const gbc_result *r, int64_t *nrow, int64_t *ncol, int64_t *nzc, int64_t *nnz, int *vt)
{
    if (!r) return fail(GBC_EINVAL, "null result");
    if (nrow) *nrow = r->nrow;
    if (ncol) *ncol = r->ncol;
    if (nzc) *nzc = r->nzc;
    if (nnz) *nnz = r->nnz;
    if (vt) *vt = r->valtype;
    return GBC_OK;
}

int gbc_result_copy(const gbc_result *r, int64_t *cp, int64_t *jc, int64_t *ir, void *num, int where)
{
    if (!r) return fail(GBC_EINVAL, "null result");
    cudaMemcpyKind k = where == GBC_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaStream_t s = r->ctx->stream;
    if (cp) GBC_CUDA_TRY(cudaMemcpyAsync(cp, r->cp, (r->nzc + 1) * sizeof(int64_t), k, s));
    if (jc && r->nzc && r->jc) GBC_CUDA_TRY(cudaMemcpyAsync(jc, r->jc, r->nzc * sizeof(int64_t), k, s));
    if (jc && r->nzc && !r->jc) {  // a CSC result: stored column i is column i
        if (where == GBC_DEVICE) return fail(GBC_EINVAL, "the result has no column ids (CSC form)");
        for (int64_t i = 0; i < r->nzc; ++i) jc[i] = i;
    }
    if (ir && r->nnz) GBC_CUDA_TRY(cudaMemcpyAsync(ir, r->ir, r->nnz * sizeof(int64_t), k, s));
    if (num && r->nnz) GBC_CUDA_TRY(cudaMemcpyAsync(num, r->num, r->nnz * value_size(r->valtype), k, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    return GBC_OK;
}

int gbc_result_device_ptrs(const gbc_result *r, const int64_t **cp, const int64_t **jc, const int64_t **ir,
                           const void **num)
{
    if (!r) return fail(GBC_EINVAL, "null result");
    if (cp) *cp = r->cp;
    if (jc) *jc = r->jc;
    if (ir) *ir = r->ir;
    if (num) *num = r->num;
    return GBC_OK;
}

int gbc_result_free(gbc_result *r)
{
    if (!r) return GBC_OK;
    Context *c = r->ctx;
    device_free(c, r->cp);
    device_free(c, r->jc);
    device_free(c, r->ir);
    device_free(c, r->num);
    delete r;
    return GBC_OK;
}

}  // extern "C"
