// MCL prune / select / recovery of one expansion step on the GPU, with the
// semantics of MCLPruneRecoverySelect (ParFriends.h:185-354) and Kselect1
// (SpParMat.cpp:1191-1300, 1411-1690); recovery is described at k_mcl_cut.
// Without recovery:
//   * statistics on the column pruned "val <= hardThreshold" (ParFriends.h:196);
//   * a column is selected when its pruned nnz > selectNum (:257-260); its
//     cut is the selectNum-th largest value of the UNPRUNED column (Kselect1
//     partial_sort with std::greater);
//   * PruneColumn(pruneCols, std::less) removes val < cut: cut = kth for
//     selected columns (ties kept), cut = hardThreshold for the others
//     (:283, :339).
// The k-th largest is found with an MSB-first radix select over an
// order-preserving 32-bit transform of the float values (one warp per
// column, 8 bits per pass).  Entries keep their order within the column.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "gbc_internal.cuh"
#undef GBC_XPROF  // the phase clocks belong to the SpGEMM unit
#include "spgemm_exact.cuh"

namespace gbc {

__device__ __forceinline__ uint32_t f2key(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float key2f(uint32_t k)
{
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

// Where column j's entries live: region 1 (beg1/ir1/v1) when flag[j] is set,
// else region 0; [b, b + cnt[j]) or, without cnt, [beg0[j], beg0[j+1]).
struct Src {
    const int64_t *cnt;
    const int32_t *flag;
    const int64_t *beg0, *ir0;
    const float *v0;
    const int64_t *beg1, *ir1;
    const float *v1;
};

__device__ __forceinline__ void col_src(const Src &S, int64_t j, int64_t &b, int64_t &e, const int64_t *&ir,
                                        const float *&v)
{
    const bool o = S.flag && S.flag[j];
    b = o ? S.beg1[j] : S.beg0[j];
    e = S.cnt ? b + S.cnt[j] : S.beg0[j + 1];
    ir = o ? S.ir1 : S.ir0;
    v = o ? S.v1 : S.v0;
}

// Warp-wide k-th largest value of v[b, e) (k <= e - b): MSB-first radix
// select over the order-preserving keys, 8 bits per pass.
__device__ float warp_kth_largest(const float *v, int64_t b, int64_t e, int64_t k, int32_t *hist)
{
    const int lane = threadIdx.x & 31;
    uint32_t prefix = 0, pmask = 0;
    int64_t kk = k;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int d = lane; d < 256; d += 32) hist[d] = 0;
        __syncwarp();
        for (int64_t p = b + lane; p < e; p += 32) {
            const uint32_t u = f2key(v[p]);
            if ((u & pmask) == prefix) atomicAdd(&hist[(u >> shift) & 255], 1);
        }
        __syncwarp();
        // suffix sums from the top digit: lane owns digits 255-8*lane .. 248-8*lane
        int loc[8], sum = 0;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            loc[u] = hist[255 - (lane * 8 + u)];
            sum += loc[u];
        }
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        int above = incl - sum;  // entries with a larger digit than this lane's first
        int chosen = -1;
        int64_t before = 0;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (chosen < 0 && above + loc[u] >= kk && above < kk) {
                chosen = 255 - (lane * 8 + u);
                before = above;
            }
            above += loc[u];
        }
        const unsigned hit = __ballot_sync(0xffffffffu, chosen >= 0);
        const int src = __ffs(hit) - 1;
        chosen = __shfl_sync(0xffffffffu, chosen, src);
        before = __shfl_sync(0xffffffffu, before, src);
        kk -= before;
        prefix |= (uint32_t)chosen << shift;
        pmask |= 255u << shift;
        __syncwarp();
    }
    return key2f(prefix);
}

// Kselect1 over a sparse column list (SpParMat.cpp:1411-1690): the k-th
// largest value of the column, its smallest when it holds fewer than k
// entries, numeric_limits<float>::min() when it is empty.
__device__ float warp_kselect(const float *v, int64_t b, int64_t e, int64_t k, int32_t *hist)
{
    if (e == b) return 1.17549435e-38f;
    if (e - b >= k) return warp_kth_largest(v, b, e, k, hist);
    float m = 3.4028235e38f;
    for (int64_t p = b + (threadIdx.x & 31); p < e; p += 32) m = fminf(m, v[p]);
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

// Column sum of the values of v[b, e) with v > thr (mode 0), v >= thr
// (mode 1), or of every value squared (mode 2, each square rounded to
// float as the reference's pow(val, 2) is): the exact sum of their parts (with 2^emax the largest value's
// exponent among them, parts below 2^(emax - 72) are truncated), rounded to
// double and then to float -- independent of the column's storage order.
__device__ float warp_colsum(const float *v, int64_t b, int64_t e, float thr, int mode)
{
    const int lane = threadIdx.x & 31;
    int emax = -1000;
    for (int64_t p = b + lane; p < e; p += 32) {
        const float x = mode == 2 ? __fmul_rn(v[p], v[p]) : v[p];
        if (mode == 0 ? !(x > thr) : mode == 1 ? (x < thr) : false) continue;
        const uint32_t u = __float_as_uint(x);
        if ((u << 1) == 0) continue;
        int ex = (int)((u >> 23) & 0xff);
        if (ex == 0) ex = 1;
        emax = max(emax, ex);
    }
    emax = __reduce_max_sync(0xffffffffu, emax);
    if (emax == -1000) return 0.0f;
    const int unit = emax - 150 - 72;  // the accumulator's lowest bit is 2^unit
    uint64_t hi = 0, lo = 0;
    for (int64_t p = b + lane; p < e; p += 32) {
        const float x = mode == 2 ? __fmul_rn(v[p], v[p]) : v[p];
        if (mode == 0 ? !(x > thr) : mode == 1 ? (x < thr) : false) continue;
        const uint32_t u = __float_as_uint(x);
        int ex = (int)((u >> 23) & 0xff);
        uint32_t m = u & 0x7fffff;
        if (ex) m |= 0x800000; else ex = 1;
        const int sh = ex - 150 - unit;  // m * 2^(ex - 150) = (m << sh) * 2^unit, sh <= 72
        uint64_t tl, th;
        if (sh >= 64) {
            tl = 0;
            th = (uint64_t)m << (sh - 64);
        } else if (sh > 0) {
            tl = (uint64_t)m << sh;
            th = (uint64_t)m >> (64 - sh);
        } else {
            tl = (uint64_t)(m >> min(-sh, 31));
            th = 0;
        }
        if (u >> 31) {
            const uint64_t old = lo;
            lo -= tl;
            hi -= th + (old < tl ? 1ull : 0ull);
        } else {
            lo += tl;
            hi += th + (lo < tl ? 1ull : 0ull);
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const uint64_t l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        lo += l2;
        hi += h2 + (lo < l2 ? 1ull : 0ull);
    }
    return (float)x_round(hi, lo, 2, unit + 1075);
}

// Pass 1: per column, the cut value and the number of kept entries
// (MCLPruneRecoverySelect, ParFriends.h:185-354):
//   nnzP / sumP over the entries with val > thr (the "val <= thr" prune);
//   recovered when recover_num > 0, nnzP < recover_num, nnz > nnzP and sumP <
//     recover_pct: cut = Kselect(recover_num);
//   else selected when select > 0 and nnzP > select: cut = Kselect(select),
//     then recovered after the selection when recover_num > 0 and the kept
//     entries (val >= cut) number fewer than recover_num and sum below
//     recover_pct: cut = Kselect(recover_num);
//   else cut = thr; kept entries: !(val < cut).
__global__ void __launch_bounds__(256) k_mcl_cut(int64_t n, Src S, float thr, int64_t select, int64_t rnum,
                                                 float rpct, float *cut, int64_t *keep)
{
    __shared__ int32_t hist_all[8][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t *hist = hist_all[w];
    for (int64_t j = int64_t(blockIdx.x) * 8 + w; j < n; j += int64_t(gridDim.x) * 8) {
        int64_t b, e;
        const int64_t *ir;
        const float *v;
        col_src(S, j, b, e, ir, v);
        int64_t npr = 0;
        for (int64_t p = b + lane; p < e; p += 32) npr += !(v[p] <= thr);
#pragma unroll
        for (int o = 16; o; o >>= 1) npr += __shfl_xor_sync(0xffffffffu, npr, o);
        float c = thr;
        const bool recover = rnum > 0 && npr < rnum && (e - b) > npr && warp_colsum(v, b, e, thr, 0) < rpct;
        if (recover) {
            c = warp_kselect(v, b, e, rnum, hist);
        } else if (select > 0 && npr > select) {
            c = warp_kselect(v, b, e, select, hist);
            if (rnum > 0) {
                int64_t n1 = 0;
                for (int64_t p = b + lane; p < e; p += 32) n1 += !(v[p] < c);
#pragma unroll
                for (int o = 16; o; o >>= 1) n1 += __shfl_xor_sync(0xffffffffu, n1, o);
                if (n1 < rnum && warp_colsum(v, b, e, c, 1) < rpct) c = warp_kselect(v, b, e, rnum, hist);
            }
        }
        int64_t kept = 0;
        for (int64_t p = b + lane; p < e; p += 32) kept += !(v[p] < c);
#pragma unroll
        for (int o = 16; o; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
        if (lane == 0) {
            cut[j] = c;
            keep[j] = kept;
        }
    }
}

// Pass 2: copy the kept entries (order preserved) to their new positions.
__global__ void __launch_bounds__(256) k_mcl_write(int64_t n, Src S, const float *cut, const int64_t *pos,
                                                   int64_t *oir, float *ov)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t j = int64_t(blockIdx.x) * 8 + w; j < n; j += int64_t(gridDim.x) * 8) {
        int64_t b, e;
        const int64_t *ir;
        const float *v;
        col_src(S, j, b, e, ir, v);
        const float c = cut[j];
        int64_t o = pos[j];
        for (int64_t p0 = b; p0 < e; p0 += 32) {
            const int64_t p = p0 + lane;
            const bool k = p < e && !(v[p] < c);
            const unsigned m = __ballot_sync(0xffffffffu, k);
            if (k) {
                const int64_t d = o + __popc(m & ((1u << lane) - 1));
                oir[d] = ir[p];
                ov[d] = v[p];
            }
            o += __popc(m);
        }
    }
}

// MakeColStochastic (Applications/MCL.cpp:389-394): every column scaled by
// 1 / (its sum), safemultinv giving FLT_MAX for a zero sum.  One warp per
// column, sums as warp_colsum (mode 1 over all values).
__global__ void __launch_bounds__(256) k_mcl_colscale(int64_t n, const int64_t *cp, float *v)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t j = int64_t(blockIdx.x) * 8 + w; j < n; j += int64_t(gridDim.x) * 8) {
        const int64_t b = cp[j], e = cp[j + 1];
        const float sum = warp_colsum(v, b, e, -3.4028235e38f, 1);
        const float inv = sum == 0.0f ? 3.4028235e38f : __fdiv_rn(1.0f, sum);
        for (int64_t p = b + lane; p < e; p += 32) v[p] = __fmul_rn(v[p], inv);
    }
}

// Inflate (MCL.cpp:446-450): every value raised to `power` (in double, then
// rounded to float).
__global__ void k_mcl_inflate(int64_t nnz, float *v, double power)
{
    for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < nnz; p += int64_t(gridDim.x) * blockDim.x)
        v[p] = power == 2.0 ? __fmul_rn(v[p], v[p]) : (float)pow((double)v[p], power);
}

// Chaos (MCL.cpp:407-421): max over columns of (column max - sum of squares)
// * nnz, max taken with identity 0 (the entries are non-negative).
__global__ void __launch_bounds__(256) k_mcl_chaos(int64_t n, const int64_t *cp, const float *v, unsigned *out)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float best = 0.0f;
    for (int64_t j = int64_t(blockIdx.x) * 8 + w; j < n; j += int64_t(gridDim.x) * 8) {
        const int64_t b = cp[j], e = cp[j + 1];
        float mx = 0.0f;
        for (int64_t p = b + lane; p < e; p += 32) mx = fmaxf(mx, v[p]);
#pragma unroll
        for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const float sq = warp_colsum(v, b, e, 0.0f, 2);
        const float c = __fmul_rn(__fsub_rn(mx, sq), (float)(e - b));
        best = fmaxf(best, c);
    }
    if (lane == 0 && best > 0.0f) atomicMax(out, __float_as_uint(best));  // non-negative floats order as integers
}

int mcl_colscale(Context *ctx, gbc_result *A)
{
    if (A->nzc > 0) {
        const int grid = (int)std::min<int64_t>((int64_t)ctx->num_sms * 8, (A->nzc + 7) / 8 + 1);
        k_mcl_colscale<<<grid, 256, 0, ctx->stream>>>(A->nzc, A->cp, static_cast<float *>(A->num));
        note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    return GBC_OK;
}

int mcl_inflate(Context *ctx, gbc_result *A, double power)
{
    if (A->nnz > 0) {
        const int grid = (int)std::min<int64_t>((int64_t)ctx->num_sms * 8, (A->nnz + 255) / 256);
        k_mcl_inflate<<<grid, 256, 0, ctx->stream>>>(A->nnz, static_cast<float *>(A->num), power);
        note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    return GBC_OK;
}

int mcl_chaos(Context *ctx, const gbc_result *A, float *chaos)
{
    Workspace ws(ctx);
    unsigned *d = nullptr;
    GBC_TRY(ws.alloc_n(&d, 1));
    GBC_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(unsigned), ctx->stream));
    if (A->nzc > 0) {
        const int grid = (int)std::min<int64_t>((int64_t)ctx->num_sms * 8, (A->nzc + 7) / 8 + 1);
        k_mcl_chaos<<<grid, 256, 0, ctx->stream>>>(A->nzc, A->cp, static_cast<const float *>(A->num), d);
        note_launch();
        GBC_CUDA_TRY(cudaGetLastError());
    }
    unsigned h = 0;
    GBC_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    GBC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    memcpy(chaos, &h, sizeof(float));
    return GBC_OK;
}

// Prune/select a device CSC (n columns; column j = [beg[j], beg[j]+cnt[j]) or
// [beg[j], beg[j+1]) when cnt is null) into a new gbc_result.
int mcl_select_device2(Context *ctx, int64_t nrow, int64_t n, const int64_t *cnt, const int32_t *flag,
                       const int64_t *beg0, const int64_t *ir0, const float *v0, const int64_t *beg1,
                       const int64_t *ir1, const float *v1, float thr, int64_t select, int64_t rnum, float rpct,
                       const int64_t *jc_src, gbc_result **out)
{
    const Src S{cnt, flag, beg0, ir0, v0, beg1, ir1, v1};
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    float *cut = nullptr;
    int64_t *keep = nullptr, *pos = nullptr;
    GBC_TRY(ws.alloc_n(&cut, n + 1));
    GBC_TRY(ws.alloc_n(&keep, n + 1));
    GBC_TRY(device_alloc(ctx, (void **)&pos, (n + 1) * sizeof(int64_t)));
    const int grid = (int)std::min<int64_t>((int64_t)ctx->num_sms * 8, (n + 7) / 8 + 1);
    if (n > 0) {
        k_mcl_cut<<<grid, 256, 0, s>>>(n, S, thr, select, rnum, rpct, cut, keep);
        note_launch();
    }
    int rc = exclusive_scan_i64(ws, keep, pos, n, s);
    int64_t total = 0;
    if (rc == GBC_OK) rc = read_i64(ctx, pos + n, &total);
    gbc_result *R = new gbc_result();
    R->ctx = ctx;
    R->nrow = nrow;
    R->ncol = n;
    R->valtype = GBC_F32;
    R->cp = pos;
    R->nzc = n;
    R->nnz = total;
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&R->ir, (total + 1) * sizeof(int64_t));
    if (rc == GBC_OK) rc = device_alloc(ctx, &R->num, (total + 1) * sizeof(float));
    if (rc == GBC_OK && jc_src) rc = device_alloc(ctx, (void **)&R->jc, (n + 1) * sizeof(int64_t));
    if (rc == GBC_OK && n > 0) {
        k_mcl_write<<<grid, 256, 0, s>>>(n, S, cut, pos, R->ir, static_cast<float *>(R->num));
        note_launch();
        if (jc_src)
            rc = cudaMemcpyAsync(R->jc, jc_src, n * sizeof(int64_t), cudaMemcpyDeviceToDevice, s) == cudaSuccess
                     ? GBC_OK
                     : fail(GBC_ECUDA, "copy of column ids failed");
    }
    if (rc == GBC_OK && cudaGetLastError() != cudaSuccess) rc = fail(GBC_ECUDA, "mcl select launch failed");
    if (rc == GBC_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = fail(GBC_ECUDA, "mcl select failed");
    if (rc != GBC_OK) {
        gbc_result_free(R);
        return rc;
    }
    *out = R;
    return GBC_OK;
}

// A device-resident fp32 copy of M (host or device), same storage form.
int mcl_result_copy(Context *ctx, const gbc_matrix *M, gbc_result **out)
{
    Workspace ws(ctx);
    DevMatrix D;
    GBC_TRY(upload(ws, M, GBC_F32, &D));
    if (!D.num) return fail(GBC_EINVAL, "MCL needs matrix values");
    gbc_result *R = new gbc_result();
    R->ctx = ctx;
    R->nrow = D.nrow;
    R->ncol = D.ncol;
    R->nzc = D.nzc;
    R->nnz = D.nnz;
    R->valtype = GBC_F32;
    cudaStream_t s = ctx->stream;
    int rc = device_alloc(ctx, (void **)&R->cp, (D.nzc + 1) * sizeof(int64_t));
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&R->ir, (D.nnz + 1) * sizeof(int64_t));
    if (rc == GBC_OK) rc = device_alloc(ctx, &R->num, (D.nnz + 1) * sizeof(float));
    if (rc == GBC_OK && D.jc) rc = device_alloc(ctx, (void **)&R->jc, (D.nzc + 1) * sizeof(int64_t));
    if (rc == GBC_OK) {
        bool ok = cudaMemcpyAsync(R->cp, D.cp, (D.nzc + 1) * sizeof(int64_t), cudaMemcpyDeviceToDevice, s) ==
                  cudaSuccess;
        if (D.nnz > 0) {
            ok = ok && cudaMemcpyAsync(R->ir, D.ir, D.nnz * sizeof(int64_t), cudaMemcpyDeviceToDevice, s) == cudaSuccess;
            ok = ok && cudaMemcpyAsync(R->num, D.num, D.nnz * sizeof(float), cudaMemcpyDeviceToDevice, s) == cudaSuccess;
        }
        if (D.jc && D.nzc > 0)
            ok = ok && cudaMemcpyAsync(R->jc, D.jc, D.nzc * sizeof(int64_t), cudaMemcpyDeviceToDevice, s) == cudaSuccess;
        if (ok) ok = cudaStreamSynchronize(s) == cudaSuccess;
        if (!ok) rc = fail(GBC_ECUDA, "copy of the MCL input failed");
    }
    if (rc != GBC_OK) {
        gbc_result_free(R);
        return rc;
    }
    *out = R;
    return GBC_OK;
}

int mcl_expand(gbc_context *ctx, const gbc_matrix *Am, float thr, int64_t select, int64_t rnum, float rpct,
               int sizing, gbc_result **out, gbc_spgemm_stats *st);

// The HipMCL loop (Applications/MCL.cpp:526-626, layers == 1) from the
// loop-adjusted matrix on: MakeColStochastic; the prune/select/recovery
// before the first iteration when nnz / n > max(select, recover_num)
// (:534-543); then while chaos > EPS (0.0001, :55): expansion with
// prune/select/recovery (:573), MakeColStochastic, Chaos, Inflate,
// MakeColStochastic.  The matrix stays on the device; each iteration reads
// back the one chaos value that decides the loop.
int mcl_iterate(gbc_context *ctx, const gbc_matrix *Am, double inflation, float thr, int64_t select, int64_t rnum,
                float rpct, int sizing, int64_t max_iter, gbc_result **out, int64_t *iterations, float *chaos_out)
{
    gbc_result *A = nullptr;
    GBC_TRY(mcl_result_copy(ctx, Am, &A));
    int rc = mcl_colscale(ctx, A);
    const int64_t avg = A->nrow > 0 ? A->nnz / A->nrow : 0;
    if (rc == GBC_OK && avg > std::max(select, rnum)) {
        gbc_result *P = nullptr;
        rc = mcl_select_device2(ctx, A->nrow, A->nzc, nullptr, nullptr, A->cp, A->ir,
                                static_cast<const float *>(A->num), nullptr, nullptr, nullptr, thr, select, rnum, rpct,
                                A->jc, &P);
        if (rc == GBC_OK) {
            gbc_result_free(A);
            A = P;
        }
    }
    float chaos = 1.0f;
    int64_t it = 0;
    while (rc == GBC_OK && (double)chaos > 0.0001 && (max_iter <= 0 || it < max_iter)) {
        const gbc_matrix view{A->nrow, A->ncol, A->nzc, A->nnz, A->cp, A->jc, A->ir, A->num, GBC_DEVICE};
        gbc_result *N = nullptr;
        rc = mcl_expand(ctx, &view, thr, select, rnum, rpct, sizing, &N, nullptr);
        if (rc != GBC_OK) break;
        gbc_result_free(A);
        A = N;
        rc = mcl_colscale(ctx, A);
        if (rc == GBC_OK) rc = mcl_chaos(ctx, A, &chaos);
        if (rc == GBC_OK) rc = mcl_inflate(ctx, A, inflation);
        if (rc == GBC_OK) rc = mcl_colscale(ctx, A);
        ++it;
    }
    if (rc == GBC_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = fail(GBC_ECUDA, "MCL iteration failed");
    if (rc != GBC_OK) {
        gbc_result_free(A);
        return rc;
    }
    *out = A;
    if (iterations) *iterations = it;
    if (chaos_out) *chaos_out = chaos;
    return GBC_OK;
}

}  // namespace gbc

using namespace gbc;

extern "C" {

int gbc_mcl_prune_select_recover_f32(gbc_context *ctx, const gbc_result *C, float thr, int64_t select,
                                     int64_t recover_num, float recover_pct, gbc_result **out)
{
    if (!ctx || !C || !out) return fail(GBC_EINVAL, "null argument");
    if (C->valtype != GBC_F32) return fail(GBC_EINVAL, "MCL prune/select expects fp32 values");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    return mcl_select_device2(ctx, C->nrow, C->nzc, nullptr, nullptr, C->cp, C->ir, static_cast<const float *>(C->num),
                              nullptr, nullptr, nullptr, thr, select, recover_num, recover_pct, C->jc, out);
}

int gbc_mcl_prune_select_f32(gbc_context *ctx, const gbc_result *C, float thr, int64_t select, gbc_result **out)
{
    return gbc_mcl_prune_select_recover_f32(ctx, C, thr, select, 0, 0.0f, out);
}

static int check_f32(const gbc_context *ctx, const gbc_result *A)
{
    if (!ctx || !A) return fail(GBC_EINVAL, "null argument");
    if (A->valtype != GBC_F32) return fail(GBC_EINVAL, "MCL steps expect fp32 values");
    return GBC_OK;
}

int gbc_mcl_make_col_stochastic_f32(gbc_context *ctx, gbc_result *A)
{
    GBC_TRY(check_f32(ctx, A));
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    return mcl_colscale(ctx, A);
}

int gbc_mcl_inflate_f32(gbc_context *ctx, gbc_result *A, double power)
{
    GBC_TRY(check_f32(ctx, A));
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    return mcl_inflate(ctx, A, power);
}

int gbc_mcl_chaos_f32(gbc_context *ctx, const gbc_result *A, float *chaos)
{
    GBC_TRY(check_f32(ctx, A));
    if (!chaos) return fail(GBC_EINVAL, "null argument");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    return mcl_chaos(ctx, A, chaos);
}

int gbc_mcl_iterate_f32(gbc_context *ctx, const gbc_matrix *A, double inflation, float thr, int64_t select,
                        int64_t recover_num, float recover_pct, int sizing, int64_t max_iter, gbc_result **out,
                        int64_t *iterations, float *chaos)
{
    if (!ctx || !A || !out) return fail(GBC_EINVAL, "null argument");
    if (A->nrow != A->ncol) return fail(GBC_EINVAL, "MCL needs a square matrix");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    return mcl_iterate(ctx, A, inflation, thr, select, recover_num, recover_pct, sizing, max_iter, out, iterations,
                       chaos);
}

}  // extern "C"
