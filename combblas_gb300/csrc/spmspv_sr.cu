// Sparse matrix x sparse vector over the semirings of the reference's other
// SpMXSpV instantiations (the overload set of SpImpl.h:49-142):
//   Select2ndMin / SelectMin  y(r) = min of the x values whose column hits r
//                             (SpMXSpV_Bucket, SpImpl.cpp:389-699);
//   Select2nd (bool A)        y(r) = the x value of the LAST column, in
//                             ascending column order, that hits r -- add keeps
//                             its second argument (Semirings.h:144-163) and the
//                             boolean SPA loops of SpImpl.cpp:167-328 visit the
//                             columns in ascending order; TopDownBFS reaches it
//                             through BFSFriends.h:198-207;
//   SelectMax (bool A)        y(r) = max of the x values (Semirings.h:192-210);
//   PlusTimes (f64/f32/i64)   y(r) = sum over hitting columns c of A(r,c)*x(c),
//                             folded left in ascending column order: the
//                             first product is stored, later ones are added,
//                             as the SPA of SpMXSpV_Bucket does (bit-exact).
// A plan holds A on the device once (CSC, and for PlusTimes also row-major),
// with its scratch, so repeated multiplies by one matrix copy only vectors.
//
// GPU form.  The order-independent semirings push: blocks take the vector's
// columns in chunks, flatten their row segments and do one 64-bit atomicMax
// per product into a per-row key (min through the complemented order-
// preserving flip, Select2nd through (column << 32 | vector position)),
// marking a touched-row bitmap.  Rows come out ascending from a popcount
// scan of the bitmap.  PlusTimes pushes only the marks, then each touched
// row is pulled by one warp over its row-major entries (ascending column):
// lanes test 32 entries against a dense column -> vector position map and
// form the products, and the products that hit are folded in lane order.
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "gbc_internal.cuh"
#include "spgemm_kernels.cuh"
#include "spmv_plan.cuh"

namespace gbc {

enum { SX_SELECT2NDMIN = 0, SX_SELECT2ND = 1, SX_SELECTMAX = 2, SX_PLUSTIMES = 3 };

constexpr int kSxThreads = 256;
constexpr unsigned long long kSign = 0x8000000000000000ull;

struct SpmspvPlan {
    Context *ctx = nullptr;
    int64_t m = 0, n = 0, nnz = 0;
    int vt = 0;
    int64_t *cp = nullptr;   // [n+1] dense column pointers
    int32_t *row = nullptr;  // [nnz]
    SpmvPlan rm;             // row-major form (numeric value types only)
    bool have_rm = false;
    // scratch kept between calls: every call leaves it as it found it
    unsigned long long *spa = nullptr;  // [m] per-row key, 0 when untouched
    uint32_t *mark = nullptr;           // [words] touched rows
    int64_t *pos = nullptr;             // [words + 1] output offsets
    int32_t *xpos = nullptr;            // [n] 1 + vector position of a column, 0 when absent
    int32_t *err = nullptr;
    unsigned long long *work = nullptr;
    int64_t words = 0;
};

// Per stored column: dense column counts, checks, int32 rows.
__global__ void k_sx_prep(int64_t nzc, int64_t m, int64_t n, int64_t nnz, const int64_t *cp, const int64_t *jc,
                          const int64_t *ir, int64_t *cnt, int32_t *row, int32_t *err)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp; i < nzc; i += nwarps) {
        const int64_t s = cp[i], e = cp[i + 1];
        const int64_t c = jc ? jc[i] : i;
        const bool bad = e < s || s < 0 || e > nnz || (i == 0 && s != 0) || (i == nzc - 1 && e != nnz) || c < 0 ||
                         c >= n || (jc && i > 0 && jc[i - 1] >= c);
        if (bad) {
            if (lane == 0) atomicOr(err, 1);
            continue;
        }
        if (lane == 0) cnt[c] = e - s;
        for (int64_t p = s + lane; p < e; p += 32) {
            int64_t r = ir[p];
            if (r < 0 || r >= m) {
                atomicOr(err, 2);
                r = 0;
            }
            row[p] = (int32_t)r;
        }
    }
}

// Vector positions of the columns; flags columns out of range (1) and
// repeated columns (2).
__global__ void k_sx_xpos(int64_t nx, const int32_t *xind, int64_t n, int32_t *xpos, int32_t *err)
{
    const int64_t f = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= nx) return;
    const int32_t c = xind[f];
    if (c < 0 || c >= n) {
        atomicOr(err, 1);
        return;
    }
    if (atomicExch(&xpos[c], (int32_t)(f + 1)) != 0) atomicOr(err, 2);
}

__global__ void k_sx_xpos_clear(int64_t nx, const int32_t *xind, int64_t n, int32_t *xpos)
{
    const int64_t f = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= nx) return;
    const int32_t c = xind[f];
    if (c >= 0 && c < n) xpos[c] = 0;
}

template <int SX>
__device__ __forceinline__ unsigned long long sx_key(int64_t x, int32_t c, int64_t f)
{
    if (SX == SX_SELECT2NDMIN) return ~((unsigned long long)x ^ kSign);
    if (SX == SX_SELECTMAX) return (unsigned long long)x ^ kSign;
    return ((unsigned long long)(uint32_t)c << 32) | (uint32_t)f;  // SX_SELECT2ND
}

// Push: per product one atomicMax of the column's key into spa[r] (not for
// PlusTimes) and the touched mark.
template <int SX>
__global__ void __launch_bounds__(kSxThreads) k_sx_expand(const int64_t *cp, const int32_t *row, const int32_t *xind,
                                                          const int64_t *xval, int64_t nx, int64_t n,
                                                          unsigned long long *spa, uint32_t *mark,
                                                          unsigned long long *work)
{
    __shared__ int64_t s_seg[kSxThreads];
    __shared__ int64_t s_off[kSxThreads + 1];
    __shared__ unsigned long long s_key[kSxThreads];
    __shared__ int64_t s_base;
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_base = (int64_t)atomicAdd(work, (unsigned long long)kSxThreads);
        __syncthreads();
        const int64_t base = s_base;
        __syncthreads();
        if (base >= nx) break;
        const int64_t f = base + tid;
        int64_t len = 0;
        if (f < nx) {
            const int32_t c = xind[f];
            if (c >= 0 && c < n) {
                const int64_t s = cp[c];
                len = cp[c + 1] - s;
                s_seg[tid] = s;
                if (SX != SX_PLUSTIMES) s_key[tid] = sx_key<SX>(xval[f], c, f);
            }
        }
        int64_t tot;
        const int64_t off = block_exclusive_sum64<kSxThreads>(len, &tot);
        s_off[tid] = off;
        if (tid == kSxThreads - 1) s_off[kSxThreads] = off + len;
        __syncthreads();
        for (int64_t j = tid; j < tot; j += kSxThreads) {
            int lo = 0, hi = kSxThreads;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (s_off[mid] <= j)
                    lo = mid;
                else
                    hi = mid;
            }
            const int32_t r = row[s_seg[lo] + (j - s_off[lo])];
            if (SX != SX_PLUSTIMES) atomicMax(&spa[r], s_key[lo]);
            const uint32_t bit = 1u << (r & 31);
            if (!(mark[r >> 5] & bit)) atomicOr(&mark[r >> 5], bit);
        }
        __syncthreads();
    }
}

__global__ void k_sx_counts(const uint32_t *mark, int64_t words, int64_t *cnt)
{
    const int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w < words) cnt[w] = __popc(mark[w]);
}

// Touched rows in ascending order with their values (select semirings);
// clears the marks and keys.
template <int SX>
__global__ void k_sx_emit(uint32_t *mark, int64_t words, const int64_t *pos, unsigned long long *spa,
                          const int64_t *xval, int32_t *yind, int64_t *yval)
{
    const int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w >= words) return;
    uint32_t bits = mark[w];
    int64_t p = pos[w];
    while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1;
        const int64_t r = w * 32 + b;
        yind[p] = (int32_t)r;
        if (SX != SX_PLUSTIMES) {
            const unsigned long long k = spa[r];
            spa[r] = 0;
            int64_t v;
            if (SX == SX_SELECT2NDMIN)
                v = (int64_t)(~k ^ kSign);
            else if (SX == SX_SELECTMAX)
                v = (int64_t)(k ^ kSign);
            else
                v = xval[(uint32_t)(k & 0xffffffffu)];
            yval[p] = v;
        }
        ++p;
    }
    mark[w] = 0;
}

template <typename V>
__device__ __forceinline__ V sx_mul(V a, V b)
{
    if constexpr (std::is_same<V, double>::value) return __dmul_rn(a, b);
    else if constexpr (std::is_same<V, float>::value) return __fmul_rn(a, b);
    else return a * b;
}

template <typename V>
__device__ __forceinline__ V sx_add(V a, V b)
{
    if constexpr (std::is_same<V, double>::value) return __dadd_rn(a, b);
    else if constexpr (std::is_same<V, float>::value) return __fadd_rn(a, b);
    else return a + b;
}

// PlusTimes pull: one warp per touched row, entries in ascending column
// order, hits folded left in that order.
template <typename V>
__global__ void __launch_bounds__(256) k_sx_pull(int64_t ny, const int32_t *yind, const int64_t *rowptr,
                                                 const int32_t *col, const V *aval, const int32_t *xpos,
                                                 const V *xval, V *yval)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp; i < ny; i += nwarps) {
        const int32_t r = yind[i];
        const int64_t b = rowptr[r], e = rowptr[r + 1];
        V acc = V(0);
        bool have = false;
        for (int64_t base = b; base < e; base += 32) {
            const int64_t idx = base + lane;
            V prod = V(0);
            bool hit = false;
            if (idx < e) {
                const int32_t fx = xpos[col[idx]];
                if (fx) {
                    prod = sx_mul<V>(aval[idx], xval[fx - 1]);
                    hit = true;
                }
            }
            unsigned bal = __ballot_sync(0xffffffffu, hit);
            while (bal) {
                const int l = __ffs(bal) - 1;
                bal &= bal - 1;
                const V pv = __shfl_sync(0xffffffffu, prod, l);
                acc = have ? sx_add<V>(acc, pv) : pv;
                have = true;
            }
        }
        if (lane == 0) yval[i] = acc;
    }
}

static void plan_release(SpmspvPlan *p)
{
    if (!p->ctx) return;
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->ctx->stream);
    if (p->have_rm) spmv_plan_release(&p->rm);
    device_free(p->ctx, p->cp);
    device_free(p->ctx, p->row);
    device_free(p->ctx, p->spa);
    device_free(p->ctx, p->mark);
    device_free(p->ctx, p->pos);
    device_free(p->ctx, p->xpos);
    device_free(p->ctx, p->err);
    device_free(p->ctx, p->work);
    cudaStreamSynchronize(p->ctx->stream);
}

static int plan_build(SpmspvPlan *p, const gbc_matrix *Am)
{
    Context *ctx = p->ctx;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    DevMatrix A;
    GBC_TRY(upload(ws, Am, p->vt, &A));
    p->m = A.nrow;
    p->n = A.ncol;
    p->nnz = A.nnz;
    if (A.nrow >= (int64_t(1) << 31) || A.ncol >= (int64_t(1) << 31))
        return fail(GBC_EOVERFLOW, "SpMSpV plan: dimensions must be below 2^31");
    p->words = (p->m + 31) / 32;
    int64_t *cnt = nullptr;
    GBC_TRY(ws.alloc_n(&cnt, p->n + 1));
    GBC_TRY(device_alloc(ctx, (void **)&p->cp, (p->n + 1) * sizeof(int64_t)));
    GBC_TRY(device_alloc(ctx, (void **)&p->row, (p->nnz + 1) * sizeof(int32_t)));
    GBC_TRY(device_alloc(ctx, (void **)&p->spa, (p->m + 1) * sizeof(unsigned long long)));
    GBC_TRY(device_alloc(ctx, (void **)&p->mark, (p->words + 1) * sizeof(uint32_t)));
    GBC_TRY(device_alloc(ctx, (void **)&p->pos, (p->words + 1) * sizeof(int64_t)));
    GBC_TRY(device_alloc(ctx, (void **)&p->xpos, (p->n + 1) * sizeof(int32_t)));
    GBC_TRY(device_alloc(ctx, (void **)&p->err, sizeof(int32_t)));
    GBC_TRY(device_alloc(ctx, (void **)&p->work, sizeof(unsigned long long)));
    GBC_CUDA_TRY(cudaMemsetAsync(cnt, 0, (p->n + 1) * sizeof(int64_t), s));
    GBC_CUDA_TRY(cudaMemsetAsync(p->spa, 0, (p->m + 1) * sizeof(unsigned long long), s));
    GBC_CUDA_TRY(cudaMemsetAsync(p->mark, 0, (p->words + 1) * sizeof(uint32_t), s));
    GBC_CUDA_TRY(cudaMemsetAsync(p->xpos, 0, (p->n + 1) * sizeof(int32_t), s));
    GBC_CUDA_TRY(cudaMemsetAsync(p->err, 0, sizeof(int32_t), s));
    if (A.nzc > 0) {
        const int grid = (int)std::min<int64_t>((A.nzc + 7) / 8, (int64_t)ctx->num_sms * 16);
        k_sx_prep<<<grid, 256, 0, s>>>(A.nzc, p->m, p->n, p->nnz, A.cp, A.jc, A.ir, cnt, p->row, p->err);
        note_launch();
    }
    GBC_TRY(exclusive_scan_i64(ws, cnt, p->cp, p->n, s));
    int32_t herr = 0;
    GBC_CUDA_TRY(cudaMemcpyAsync(&herr, p->err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr & 1) return fail(GBC_EINVAL, "SpMSpV plan: malformed column pointers or column ids");
    if (herr & 2) return fail(GBC_EINVAL, "SpMSpV plan: row id out of range");
    if (p->vt == GBC_F64 || p->vt == GBC_F32 || p->vt == GBC_I64) {
        p->rm.ctx = ctx;
        p->rm.vt = p->vt;
        p->have_rm = true;
        GBC_TRY(spmv_plan_build(&p->rm, Am));
    }
    return GBC_OK;
}

template <int SX, typename V>
static int sx_run(SpmspvPlan *p, Workspace &ws, const int32_t *dx, const void *dv, int64_t nx, int32_t **yi,
                  void **yv, int64_t *ny, bool host_out)
{
    Context *ctx = p->ctx;
    cudaStream_t s = ctx->stream;
    GBC_CUDA_TRY(cudaMemsetAsync(p->err, 0, sizeof(int32_t), s));
    GBC_CUDA_TRY(cudaMemsetAsync(p->work, 0, sizeof(unsigned long long), s));
    if (nx > 0) {
        k_sx_xpos<<<(unsigned)((nx + 255) / 256), 256, 0, s>>>(nx, dx, p->n, p->xpos, p->err);
        const int grid = (int)std::min<int64_t>((int64_t)ctx->num_sms * 4, (nx + kSxThreads - 1) / kSxThreads);
        k_sx_expand<SX><<<grid, kSxThreads, 0, s>>>(p->cp, p->row, dx, static_cast<const int64_t *>(dv), nx, p->n,
                                                    p->spa, p->mark, p->work);
        note_launches(2);
    }
    int64_t *cnt = nullptr;
    GBC_TRY(ws.alloc_n(&cnt, p->words + 1));
    if (p->words > 0) {
        k_sx_counts<<<(unsigned)((p->words + 255) / 256), 256, 0, s>>>(p->mark, p->words, cnt);
        note_launch();
    }
    GBC_TRY(exclusive_scan_i64(ws, cnt, p->pos, p->words, s));
    GBC_TRY(read_i64(ctx, p->pos + p->words, ny));
    if (host_out) {
        GBC_TRY(ws.alloc_n(yi, *ny + 1));
        void *b = nullptr;
        GBC_TRY(ws.alloc(&b, (*ny + 1) * sizeof(V)));
        *yv = b;
    }
    if (p->words > 0) {
        k_sx_emit<SX><<<(unsigned)((p->words + 255) / 256), 256, 0, s>>>(
            p->mark, p->words, p->pos, p->spa, static_cast<const int64_t *>(dv), *yi,
            SX == SX_PLUSTIMES ? nullptr : static_cast<int64_t *>(*yv));
        note_launch();
    }
    if (SX == SX_PLUSTIMES && *ny > 0) {
        const int grid = (int)std::min<int64_t>((*ny + 7) / 8, (int64_t)ctx->num_sms * 16);
        k_sx_pull<V><<<grid, 256, 0, s>>>(*ny, *yi, p->rm.rowptr, p->rm.col, static_cast<const V *>(p->rm.val),
                                          p->xpos, static_cast<const V *>(dv), static_cast<V *>(*yv));
        note_launch();
    }
    if (nx > 0) {
        k_sx_xpos_clear<<<(unsigned)((nx + 255) / 256), 256, 0, s>>>(nx, dx, p->n, p->xpos);
        note_launch();
    }
    GBC_CUDA_TRY(cudaGetLastError());
    int32_t herr = 0;
    GBC_CUDA_TRY(cudaMemcpyAsync(&herr, p->err, sizeof(herr), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr & 1) return fail(GBC_EINVAL, "vector index out of range");
    if (herr & 2) return fail(GBC_EINVAL, "repeated vector index");
    return GBC_OK;
}

}  // namespace gbc

using namespace gbc;

struct gbc_spmspv_plan : gbc::SpmspvPlan {};

extern "C" {

int gbc_spmspv_plan_create(gbc_context *ctx, int vt, const gbc_matrix *A, gbc_spmspv_plan **out)
{
    if (!ctx || !A || !out) return fail(GBC_EINVAL, "null argument");
    *out = nullptr;
    if (vt != GBC_F64 && vt != GBC_F32 && vt != GBC_I64 && vt != GBC_BOOL) return fail(GBC_EINVAL, "bad value type");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    gbc_spmspv_plan *p = new gbc_spmspv_plan();
    p->ctx = ctx;
    p->vt = vt;
    const int rc = plan_build(p, A);
    if (rc != GBC_OK) {
        gbc_spmspv_plan_destroy(p);
        return rc;
    }
    *out = p;
    return GBC_OK;
}

int gbc_spmspv_plan_destroy(gbc_spmspv_plan *p)
{
    if (!p) return GBC_OK;
    plan_release(p);
    delete p;
    return GBC_OK;
}

int gbc_spmspv(gbc_context *ctx, gbc_spmspv_plan *p, int sr, const int32_t *indx, const void *numx, int32_t veclen,
               int32_t *indy, void *numy, int32_t *nnzy, int where)
{
    if (!ctx || !p || !nnzy) return fail(GBC_EINVAL, "null argument");
    if (veclen < 0) return fail(GBC_EINVAL, "negative vector length");
    if (veclen > 0 && (!indx || !numx)) return fail(GBC_EINVAL, "null vector");
    if (where != GBC_HOST && where != GBC_DEVICE) return fail(GBC_EINVAL, "bad memory location");
    int sx = -1;
    size_t xs = 8;
    switch (sr) {
        case GBC_SR_SELECT2NDMIN: sx = SX_SELECT2NDMIN; break;
        case GBC_SR_SELECT2ND: sx = SX_SELECT2ND; break;
        case GBC_SR_SELECTMAX: sx = SX_SELECTMAX; break;
        case GBC_SR_PLUSTIMES:
            if (p->vt == GBC_BOOL) return fail(GBC_EUNSUPPORTED, "PlusTimes SpMSpV needs a numeric matrix");
            sx = SX_PLUSTIMES;
            xs = value_size(p->vt);
            break;
        default: return fail(GBC_EUNSUPPORTED, "semiring not instantiated for SpMSpV");
    }
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    p->ctx = ctx;
    p->rm.ctx = ctx;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    const int32_t *dx = indx;
    const void *dv = numx;
    if (where == GBC_HOST && veclen > 0) {
        int32_t *a = nullptr;
        void *b = nullptr;
        GBC_TRY(ws.alloc_n(&a, veclen));
        GBC_TRY(ws.alloc(&b, veclen * xs));
        GBC_CUDA_TRY(cudaMemcpyAsync(a, indx, veclen * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(b, numx, veclen * xs, cudaMemcpyHostToDevice, s));
        dx = a;
        dv = b;
    }
    int32_t *yi = indy;
    void *yv = numy;
    int64_t ny = 0;
    const bool host_out = where == GBC_HOST;
    int rc;
    switch (sx) {
        case SX_SELECT2NDMIN: rc = sx_run<SX_SELECT2NDMIN, int64_t>(p, ws, dx, dv, veclen, &yi, &yv, &ny, host_out); break;
        case SX_SELECT2ND: rc = sx_run<SX_SELECT2ND, int64_t>(p, ws, dx, dv, veclen, &yi, &yv, &ny, host_out); break;
        case SX_SELECTMAX: rc = sx_run<SX_SELECTMAX, int64_t>(p, ws, dx, dv, veclen, &yi, &yv, &ny, host_out); break;
        default:
            if (p->vt == GBC_F64)
                rc = sx_run<SX_PLUSTIMES, double>(p, ws, dx, dv, veclen, &yi, &yv, &ny, host_out);
            else if (p->vt == GBC_F32)
                rc = sx_run<SX_PLUSTIMES, float>(p, ws, dx, dv, veclen, &yi, &yv, &ny, host_out);
            else
                rc = sx_run<SX_PLUSTIMES, int64_t>(p, ws, dx, dv, veclen, &yi, &yv, &ny, host_out);
    }
    if (rc != GBC_OK) return rc;
    const size_t ys = sx == SX_PLUSTIMES ? xs : 8;
    if (host_out && ny > 0) {
        GBC_CUDA_TRY(cudaMemcpyAsync(indy, yi, ny * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(numy, yv, ny * ys, cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
    }
    *nnzy = (int32_t)ny;
    return GBC_OK;
}

int gbc_spmspv_plan_info(const gbc_spmspv_plan *p, int64_t *nrow, int64_t *ncol, int64_t *nnz)
{
    if (!p) return fail(GBC_EINVAL, "null argument");
    if (nrow) *nrow = p->m;
    if (ncol) *ncol = p->n;
    if (nnz) *nnz = p->nnz;
    return GBC_OK;
}

}  // extern "C"
