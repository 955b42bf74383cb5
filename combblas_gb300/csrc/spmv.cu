// Sparse matrix x dense vector over a semiring, y <- y (+) A x: the local
// multiply of dcsc_gespmv / dcsc_gespmv_threaded (Friends.h:63-175), whose
// per-row update is SR::axpy(a, x[col], y[row]) over A's columns in order.
//
// GPU form: a plan holds A row-major (rows ascending, each row's entries in
// ascending column order) built once on the device by a stable LSD radix
// sort of the column-major entries by row.  Rows of at most 64 entries are
// taken by eight lanes each (four rows per warp); longer rows are cut into
// chunks of at most 256 entries, a warp per chunk.  Lanes fold their share
// of a row or chunk in column order, a fixed shuffle tree combines the
// lanes, and rows of several chunks fold their chunk results in order before
// y is folded in.
// The order is fixed, so repeated runs are bit-identical; for min-type,
// boolean and integer semirings every order gives the reference's result
// exactly, and for PlusTimes on floating values the sum differs from the
// reference's column-order sum only by rounding.
#include <algorithm>

#include "gbc_internal.cuh"
#include "semiring.cuh"
#include "spmv_plan.cuh"

namespace gbc {

constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsRounds = 8;
constexpr int kRsTile = kRsThreads * kRsRounds;  // items per block and pass
constexpr int kRsRadix = 256;

// per-entry column ids of a CSC/DCSC
__global__ void k_entry_cols(int64_t nzc, const int64_t *cp, const int64_t *jc, int32_t *col)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp; i < nzc; i += nwarps) {
        const int32_t c = (int32_t)(jc ? jc[i] : i);
        for (int64_t p = cp[i] + lane; p < cp[i + 1]; p += 32) col[p] = c;
    }
}

__global__ void k_row_keys(int64_t n, const int64_t *ir, int64_t m, uint32_t *key, int32_t *idx, int64_t *rowcnt,
                           int32_t *err)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t r = ir[i];
    if (r < 0 || r >= m) {
        atomicOr(err, 1);
        r = 0;
    }
    key[i] = (uint32_t)r;
    idx[i] = (int32_t)i;
    atomicAdd((unsigned long long *)&rowcnt[r], 1ull);
}

// Digit counts of one tile of kRsTile items.
__global__ void __launch_bounds__(kRsThreads) k_rs_count(const uint32_t *key, int64_t n, int shift, int64_t *hist)
{
    __shared__ int cnt[kRsRadix];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int64_t t0 = int64_t(blockIdx.x) * kRsTile;
    for (int i = threadIdx.x; i < kRsTile; i += kRsThreads) {
        const int64_t it = t0 + i;
        if (it < n) atomicAdd(&cnt[(key[it] >> shift) & (kRsRadix - 1)], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter of one tile: items keep their order within a digit.
// off[d * nblocks + b] is the first output slot of digit d for tile b.
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint32_t *key_in, const int32_t *val_in, int64_t n,
                                                           int shift, const int64_t *off, uint32_t *key_out,
                                                           int32_t *val_out)
{
    __shared__ int64_t base[kRsWarps][kRsRadix];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1;
    for (int d = threadIdx.x; d < kRsWarps * kRsRadix; d += kRsThreads) base[d / kRsRadix][d % kRsRadix] = 0;
    __syncthreads();
    // warp w owns items [t0 + w*256, t0 + (w+1)*256) in 8 rounds of 32
    const int64_t w0 = int64_t(blockIdx.x) * kRsTile + (int64_t)w * (kRsTile / kRsWarps);
    for (int r = 0; r < kRsRounds; ++r) {
        const int64_t it = w0 + r * 32 + lane;
        if (it < n) atomicAdd((unsigned long long *)&base[w][(key_in[it] >> shift) & (kRsRadix - 1)], 1ull);
    }
    __syncthreads();
    {
        const int d = threadIdx.x;  // kRsThreads == kRsRadix
        int64_t run = off[(int64_t)d * gridDim.x + blockIdx.x];
        for (int u = 0; u < kRsWarps; ++u) {
            const int64_t c = base[u][d];
            base[u][d] = run;
            run += c;
        }
    }
    __syncthreads();
    for (int r = 0; r < kRsRounds; ++r) {
        const int64_t it = w0 + r * 32 + lane;
        const bool act = it < n;
        const uint32_t k = act ? key_in[it] : 0;
        const int d = act ? (int)((k >> shift) & (kRsRadix - 1)) : 0;
        // lanes holding the same digit, from eight ballots
        unsigned peers = __ballot_sync(0xffffffffu, act);
#pragma unroll
        for (int bit = 0; bit < 8; ++bit) {
            const unsigned bb = __ballot_sync(0xffffffffu, act && ((d >> bit) & 1));
            peers &= ((d >> bit) & 1) ? bb : ~bb;
        }
        if (act) {
            const int64_t dst = base[w][d] + __popc(peers & lt);
            key_out[dst] = k;
            val_out[dst] = val_in[it];
        }
        __syncwarp();
        if (act && (peers & lt) == 0) base[w][d] += __popc(peers);
        __syncwarp();
    }
}

template <typename V>
__global__ void k_gather_rowmajor(int64_t n, const int32_t *perm, const int32_t *col_cm, const V *val_cm, V one,
                                  int32_t *col, V *val)
{
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int32_t e = perm[p];
    col[p] = col_cm[e];
    val[p] = val_cm ? val_cm[e] : one;
}

// Rows are cut into chunks of at most kChunk entries (fixed at plan time).
// A warp takes one chunk: lane l folds entries l, l+32, ... (up to 8, loads
// issued together), then a fixed shuffle tree combines the lanes.  A row of
// one chunk updates y directly; longer rows leave their chunk partials for
// k_spmv_rows, which folds them in chunk order.
constexpr int kChunk = 256;

template <class SR>
__global__ void __launch_bounds__(256) k_spmv_chunks(int64_t nchunks, const int64_t *chunk_start,
                                                     const int64_t *chunk_end, const int32_t *chunk_row,
                                                     const int8_t *partial_slot,
                                                     const int32_t *col, const typename SR::V *val,
                                                     const typename SR::V *x, typename SR::V *y,
                                                     typename SR::V *partial)
{
    typedef typename SR::V V;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t c = warp; c < nchunks; c += nwarps) {
        const int32_t r = chunk_row[c];
        const int64_t s = chunk_start[c];
        const int64_t e = chunk_end[c];
        V t[kChunk / 32];
        int cnt = 0;
#pragma unroll
        for (int k = 0; k < kChunk / 32; ++k) {
            const int64_t p = s + k * 32 + lane;
            if (p < e) {
                t[k] = SR::mul(val[p], x[col[p]]);
                cnt = k + 1;
            }
        }
        bool have = cnt > 0;
        V acc = t[0];
#pragma unroll
        for (int k = 1; k < kChunk / 32; ++k)
            if (k < cnt) acc = SR::add(acc, t[k]);
        // fixed tree: lane l takes lane l + o's partial, if that lane has one
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            const V other = __shfl_down_sync(0xffffffffu, acc, o);
            const bool ho = __shfl_down_sync(0xffffffffu, (int)have, o) != 0;
            if (lane + o < 32 && ho) {
                acc = have ? SR::add(acc, other) : other;
                have = true;
            }
        }
        if (lane == 0) {
            if (partial_slot[c] < 0)
                y[r] = SR::add(y[r], acc);  // the row is this one chunk
            else
                partial[c] = acc;
        }
    }
}

// Rows of at most kShort entries: eight lanes per row, four rows per warp;
// lane g of a row folds entries g, g+8, ... in column order, then a fixed
// three-step shuffle tree over the eight lanes.
constexpr int kShort = 64;

template <class SR>
__global__ void __launch_bounds__(256) k_spmv_short(int64_t nshort, const int32_t *short_rows,
                                                    const int64_t *rowptr, const int32_t *col,
                                                    const typename SR::V *val, const typename SR::V *x,
                                                    typename SR::V *y)
{
    typedef typename SR::V V;
    const int lane = threadIdx.x & 31, gl = lane & 7;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t b = warp * 4; b < nshort; b += nwarps * 4) {
        const int64_t i = b + (lane >> 3);
        const bool act = i < nshort;
        const int32_t r = act ? short_rows[i] : 0;
        const int64_t s = act ? rowptr[r] : 0, e = act ? rowptr[r + 1] : 0;
        V t[kShort / 8];
        int cnt = 0;
#pragma unroll
        for (int k = 0; k < kShort / 8; ++k) {
            const int64_t p = s + k * 8 + gl;
            if (p < e) {
                t[k] = SR::mul(val[p], x[col[p]]);
                cnt = k + 1;
            }
        }
        bool have = cnt > 0;
        V acc = t[0];
#pragma unroll
        for (int k = 1; k < kShort / 8; ++k)
            if (k < cnt) acc = SR::add(acc, t[k]);
#pragma unroll
        for (int o = 4; o; o >>= 1) {
            const V other = __shfl_down_sync(0xffffffffu, acc, o, 8);
            const bool ho = __shfl_down_sync(0xffffffffu, (int)have, o, 8) != 0;
            if (gl + o < 8 && ho) {
                acc = have ? SR::add(acc, other) : other;
                have = true;
            }
        }
        if (act && gl == 0 && have) y[r] = SR::add(y[r], acc);
    }
}

template <class SR>
__global__ void k_spmv_rows(int64_t nlong, const int32_t *long_row, const int64_t *long_first,
                            const int64_t *long_end, const typename SR::V *partial, typename SR::V *y)
{
    typedef typename SR::V V;
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nlong) return;
    const int64_t c0 = long_first[i], c1 = long_end[i];
    V acc = partial[c0];
    for (int64_t c = c0 + 1; c < c1; ++c) acc = SR::add(acc, partial[c]);
    const int32_t r = long_row[i];
    y[r] = SR::add(y[r], acc);
}

// chunks per row (0 for an empty row)
__global__ void k_row_chunks(int64_t m, const int64_t *rowptr, int64_t *nch, int64_t *islong, int64_t *isshort)
{
    const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const int64_t len = rowptr[r + 1] - rowptr[r];
    const bool sh = len > 0 && len <= kShort;
    nch[r] = sh ? 0 : (len + kChunk - 1) / kChunk;
    islong[r] = len > kChunk;
    isshort[r] = sh;
}

__global__ void k_fill_chunks(int64_t m, const int64_t *rowptr, const int64_t *cfirst, const int64_t *lpos,
                              const int64_t *spos, int64_t *chunk_start, int64_t *chunk_end, int32_t *chunk_row,
                              int8_t *partial_slot, int32_t *short_rows, int32_t *long_row, int64_t *long_first,
                              int64_t *long_end)
{
    const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= m) return;
    const int64_t s = rowptr[r], e = rowptr[r + 1];
    if (e > s && e - s <= kShort) {
        short_rows[spos[r]] = (int32_t)r;
        return;
    }
    int64_t c = cfirst[r];
    const int8_t slot = (e - s > kChunk) ? 1 : -1;
    for (int64_t p = s; p < e; p += kChunk, ++c) {
        chunk_start[c] = p;
        chunk_end[c] = min(e, p + kChunk);
        chunk_row[c] = (int32_t)r;
        partial_slot[c] = slot;
    }
    if (e - s > kChunk) {
        const int64_t q = lpos[r];
        long_row[q] = (int32_t)r;
        long_first[q] = cfirst[r];
        long_end[q] = c;
    }
}


template <typename V>
static int plan_values(SpmvPlan *p, Workspace &ws, const DevMatrix &A, const int32_t *perm, const int32_t *col_cm)
{
    GBC_TRY(device_alloc(p->ctx, &p->val, (p->nnz + 1) * sizeof(V)));
    if (p->nnz > 0) {
        k_gather_rowmajor<V><<<(unsigned)((p->nnz + 255) / 256), 256, 0, p->ctx->stream>>>(
            p->nnz, perm, col_cm, static_cast<const V *>(A.num), (V)1, p->col, static_cast<V *>(p->val));
        note_launch();
    }
    return GBC_OK;
}

int spmv_plan_build(SpmvPlan *p, const gbc_matrix *Am)
{
    Context *ctx = p->ctx;
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    DevMatrix A;
    GBC_TRY(upload(ws, Am, p->vt, &A));
    p->m = A.nrow;
    p->n = A.ncol;
    p->nnz = A.nnz;
    if (A.nnz >= (int64_t(1) << 31) || A.ncol >= (int64_t(1) << 31) || A.nrow >= (int64_t(1) << 32))
        return fail(GBC_EOVERFLOW, "SpMV plan: nnz and columns must be below 2^31, rows below 2^32");
    const int64_t n = A.nnz;
    int32_t *err = nullptr, *col_cm = nullptr, *idx[2] = {nullptr, nullptr};
    uint32_t *key[2] = {nullptr, nullptr};
    int64_t *rowcnt = nullptr;
    GBC_TRY(ws.alloc_n(&err, 4));
    GBC_CUDA_TRY(cudaMemsetAsync(err, 0, 4 * sizeof(int32_t), s));
    GBC_TRY(ws.alloc_n(&col_cm, n + 1));
    GBC_TRY(ws.alloc_n(&key[0], n + 1));
    GBC_TRY(ws.alloc_n(&key[1], n + 1));
    GBC_TRY(ws.alloc_n(&idx[0], n + 1));
    GBC_TRY(ws.alloc_n(&idx[1], n + 1));
    GBC_TRY(ws.alloc_n(&rowcnt, p->m + 1));
    GBC_CUDA_TRY(cudaMemsetAsync(rowcnt, 0, (p->m + 1) * sizeof(int64_t), s));
    GBC_TRY(device_alloc(ctx, (void **)&p->rowptr, (p->m + 1) * sizeof(int64_t)));
    GBC_TRY(device_alloc(ctx, (void **)&p->col, (n + 1) * sizeof(int32_t)));
    if (A.nzc > 0) {
        k_entry_cols<<<(unsigned)std::min<int64_t>((A.nzc + 7) / 8, (int64_t)ctx->num_sms * 16), 256, 0, s>>>(
            A.nzc, A.cp, A.jc, col_cm);
        note_launch();
    }
    if (n > 0) {
        k_row_keys<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, A.ir, p->m, key[0], idx[0], rowcnt, err);
        note_launch();
    }
    GBC_TRY(exclusive_scan_i64(ws, rowcnt, p->rowptr, p->m, s));
    // stable LSD radix sort of the entries by row (8-bit digits)
    int cur = 0;
    if (n > 0) {
        int bits = 0;
        while (bits < 32 && (uint64_t(1) << bits) < (uint64_t)p->m) ++bits;
        const int64_t nblocks = (n + kRsTile - 1) / kRsTile;
        int64_t *hist = nullptr;
        GBC_TRY(ws.alloc_n(&hist, (size_t)kRsRadix * nblocks + 1));
        for (int shift = 0; shift < bits; shift += 8) {
            k_rs_count<<<(unsigned)nblocks, kRsThreads, 0, s>>>(key[cur], n, shift, hist);
            GBC_TRY(exclusive_scan_i64(ws, hist, hist, kRsRadix * nblocks, s));
            k_rs_scatter<<<(unsigned)nblocks, kRsThreads, 0, s>>>(key[cur], idx[cur], n, shift, hist, key[cur ^ 1],
                                                                   idx[cur ^ 1]);
            note_launches(2);
            cur ^= 1;
        }
    }
    // row chunks
    {
        int64_t *nch = nullptr, *cfirst = nullptr, *islong = nullptr, *lpos = nullptr, *isshort = nullptr,
                *spos = nullptr;
        GBC_TRY(ws.alloc_n(&nch, p->m + 1));
        GBC_TRY(ws.alloc_n(&cfirst, p->m + 1));
        GBC_TRY(ws.alloc_n(&islong, p->m + 1));
        GBC_TRY(ws.alloc_n(&lpos, p->m + 1));
        GBC_TRY(ws.alloc_n(&isshort, p->m + 1));
        GBC_TRY(ws.alloc_n(&spos, p->m + 1));
        const unsigned rg = (unsigned)((p->m + 255) / 256);
        if (p->m > 0) {
            k_row_chunks<<<rg, 256, 0, s>>>(p->m, p->rowptr, nch, islong, isshort);
            note_launch();
        }
        GBC_TRY(exclusive_scan_i64(ws, nch, cfirst, p->m, s));
        GBC_TRY(exclusive_scan_i64(ws, islong, lpos, p->m, s));
        GBC_TRY(exclusive_scan_i64(ws, isshort, spos, p->m, s));
        GBC_TRY(read_i64(ctx, cfirst + p->m, &p->nchunks));
        GBC_TRY(read_i64(ctx, lpos + p->m, &p->nlong));
        GBC_TRY(read_i64(ctx, spos + p->m, &p->nshort));
        GBC_TRY(device_alloc(ctx, (void **)&p->short_rows, (p->nshort + 1) * sizeof(int32_t)));
        GBC_TRY(device_alloc(ctx, (void **)&p->chunk_end, (p->nchunks + 1) * sizeof(int64_t)));
        GBC_TRY(device_alloc(ctx, (void **)&p->chunk_start, (p->nchunks + 1) * sizeof(int64_t)));
        GBC_TRY(device_alloc(ctx, (void **)&p->chunk_row, (p->nchunks + 1) * sizeof(int32_t)));
        GBC_TRY(device_alloc(ctx, (void **)&p->partial_slot, (p->nchunks + 1) * sizeof(int8_t)));
        GBC_TRY(device_alloc(ctx, (void **)&p->long_row, (p->nlong + 1) * sizeof(int32_t)));
        GBC_TRY(device_alloc(ctx, (void **)&p->long_first, (p->nlong + 1) * sizeof(int64_t)));
        GBC_TRY(device_alloc(ctx, (void **)&p->long_end, (p->nlong + 1) * sizeof(int64_t)));
        GBC_TRY(device_alloc(ctx, &p->partial, (p->nchunks + 1) * sizeof(int64_t)));  // widest value type
        if (p->m > 0) {
            k_fill_chunks<<<rg, 256, 0, s>>>(p->m, p->rowptr, cfirst, lpos, spos, p->chunk_start, p->chunk_end,
                                             p->chunk_row, p->partial_slot, p->short_rows, p->long_row,
                                             p->long_first, p->long_end);
            note_launch();
        }
    }
    switch (p->vt) {
        case GBC_F64: GBC_TRY(plan_values<double>(p, ws, A, idx[cur], col_cm)); break;
        case GBC_F32: GBC_TRY(plan_values<float>(p, ws, A, idx[cur], col_cm)); break;
        case GBC_I64: GBC_TRY(plan_values<int64_t>(p, ws, A, idx[cur], col_cm)); break;
        case GBC_BOOL: GBC_TRY(plan_values<uint8_t>(p, ws, A, idx[cur], col_cm)); break;
        default: return fail(GBC_EINVAL, "unknown value type");
    }
    GBC_CUDA_TRY(cudaGetLastError());
    int32_t herr = 0;
    GBC_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr) return fail(GBC_EINVAL, "SpMV plan: row id out of range");
    return GBC_OK;
}

template <class SR>
static int spmv_run(SpmvPlan *p, const void *x, void *y)
{
    typedef typename SR::V V;
    cudaStream_t s = p->ctx->stream;
    if (p->nshort > 0) {
        const int sg = (int)std::min<int64_t>((p->nshort + 31) / 32, (int64_t)p->ctx->num_sms * 16);
        k_spmv_short<SR><<<sg, 256, 0, s>>>(p->nshort, p->short_rows, p->rowptr, p->col,
                                            static_cast<const V *>(p->val), static_cast<const V *>(x),
                                            static_cast<V *>(y));
        note_launch();
    }
    if (p->nchunks == 0) return GBC_OK;
    const int grid = (int)std::min<int64_t>((p->nchunks + 7) / 8, (int64_t)p->ctx->num_sms * 16);
    k_spmv_chunks<SR><<<grid, 256, 0, s>>>(p->nchunks, p->chunk_start, p->chunk_end, p->chunk_row,
                                           p->partial_slot, p->col,
                                           static_cast<const V *>(p->val), static_cast<const V *>(x),
                                           static_cast<V *>(y), static_cast<V *>(p->partial));
    note_launch();
    if (p->nlong > 0) {
        k_spmv_rows<SR><<<(unsigned)((p->nlong + 127) / 128), 128, 0, s>>>(
            p->nlong, p->long_row, p->long_first, p->long_end, static_cast<const V *>(p->partial),
            static_cast<V *>(y));
        note_launch();
    }
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

void spmv_plan_release(SpmvPlan *p)
{
    if (!p->ctx) return;
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->ctx->stream);
    device_free(p->ctx, p->rowptr);
    device_free(p->ctx, p->col);
    device_free(p->ctx, p->val);
    device_free(p->ctx, p->chunk_start);
    device_free(p->ctx, p->chunk_row);
    device_free(p->ctx, p->partial_slot);
    device_free(p->ctx, p->chunk_end);
    device_free(p->ctx, p->short_rows);
    device_free(p->ctx, p->long_row);
    device_free(p->ctx, p->long_first);
    device_free(p->ctx, p->long_end);
    device_free(p->ctx, p->partial);
    cudaStreamSynchronize(p->ctx->stream);
}

}  // namespace gbc

using namespace gbc;

struct gbc_spmv_plan : gbc::SpmvPlan {};

extern "C" {

int gbc_spmv_plan_create(gbc_context *ctx, int vt, const gbc_matrix *A, gbc_spmv_plan **out)
{
    if (!ctx || !A || !out) return fail(GBC_EINVAL, "null argument");
    *out = nullptr;
    if (vt != GBC_F64 && vt != GBC_F32 && vt != GBC_I64 && vt != GBC_BOOL) return fail(GBC_EINVAL, "bad value type");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    gbc_spmv_plan *p = new gbc_spmv_plan();
    p->ctx = ctx;
    p->vt = vt;
    const int rc = spmv_plan_build(p, A);
    if (rc != GBC_OK) {
        gbc_spmv_plan_destroy(p);
        return rc;
    }
    *out = p;
    return GBC_OK;
}

int gbc_spmv_plan_destroy(gbc_spmv_plan *p)
{
    if (!p) return GBC_OK;
    spmv_plan_release(p);
    delete p;
    return GBC_OK;
}

int gbc_spmv(gbc_context *ctx, const gbc_spmv_plan *p, int sr, const void *x, void *y, int where)
{
    if (!ctx || !p || !x || !y) return fail(GBC_EINVAL, "null argument");
    if (where != GBC_HOST && where != GBC_DEVICE) return fail(GBC_EINVAL, "bad memory location");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    SpmvPlan *q = const_cast<gbc_spmv_plan *>(p);
    q->ctx = ctx;
    cudaStream_t s = ctx->stream;
    const size_t vs = value_size(p->vt);
    Workspace ws(ctx);
    const void *dx = x;
    void *dy = y;
    if (where == GBC_HOST) {
        void *bx = nullptr, *by = nullptr;
        GBC_TRY(ws.alloc(&bx, p->n * vs + 16));
        GBC_TRY(ws.alloc(&by, p->m * vs + 16));
        GBC_CUDA_TRY(cudaMemcpyAsync(bx, x, p->n * vs, cudaMemcpyHostToDevice, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(by, y, p->m * vs, cudaMemcpyHostToDevice, s));
        dx = bx;
        dy = by;
    }
    int rc = fail(GBC_EUNSUPPORTED, "semiring/value type combination not instantiated");
    switch (sr) {
        case GBC_SR_PLUSTIMES:
            if (p->vt == GBC_F64) rc = spmv_run<PlusTimes<double>>(q, dx, dy);
            if (p->vt == GBC_F32) rc = spmv_run<PlusTimes<float>>(q, dx, dy);
            if (p->vt == GBC_I64) rc = spmv_run<PlusTimes<int64_t>>(q, dx, dy);
            if (p->vt == GBC_BOOL) rc = spmv_run<BoolOrAnd>(q, dx, dy);
            break;
        case GBC_SR_BOOL:
            if (p->vt == GBC_BOOL) rc = spmv_run<BoolOrAnd>(q, dx, dy);
            break;
        case GBC_SR_MINPLUS:
            if (p->vt == GBC_F64) rc = spmv_run<MinPlus<double>>(q, dx, dy);
            if (p->vt == GBC_I64) rc = spmv_run<MinPlus<int64_t>>(q, dx, dy);
            break;
        case GBC_SR_SELECT2NDMIN:
            if (p->vt == GBC_I64) rc = spmv_run<Select2ndMin<int64_t>>(q, dx, dy);
            break;
        default: break;
    }
    if (rc != GBC_OK) return rc;
    if (where == GBC_HOST) GBC_CUDA_TRY(cudaMemcpyAsync(y, dy, p->m * vs, cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    return GBC_OK;
}

}  // extern "C"
