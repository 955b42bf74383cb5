// MCL prune / select of one expansion step on the GPU, with the semantics of
// MCLPruneRecoverySelect for recoverNum == 0 (ParFriends.h:185-354) and
// Kselect1 (SpParMat.cpp:1191-1300):
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
#include <cstdio>

#include "gbc_internal.cuh"

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

// Pass 1: per column, the cut value and the number of kept entries.
__global__ void __launch_bounds__(256) k_mcl_cut(int64_t n, Src S, float thr, int64_t select, float *cut,
                                                 int64_t *keep)
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
        if (select > 0 && npr > select) {
            // k-th largest (k = select) of all entries of the column
            uint32_t prefix = 0, pmask = 0;
            int64_t kk = select;
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
            c = key2f(prefix);
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

// Prune/select a device CSC (n columns; column j = [beg[j], beg[j]+cnt[j]) or
// [beg[j], beg[j+1]) when cnt is null) into a new gbc_result.
int mcl_select_device2(Context *ctx, int64_t nrow, int64_t n, const int64_t *cnt, const int32_t *flag,
                       const int64_t *beg0, const int64_t *ir0, const float *v0, const int64_t *beg1,
                       const int64_t *ir1, const float *v1, float thr, int64_t select, const int64_t *jc_src,
                       gbc_result **out)
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
        k_mcl_cut<<<grid, 256, 0, s>>>(n, S, thr, select, cut, keep);
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
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&R->jc, (n + 1) * sizeof(int64_t));
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

}  // namespace gbc

using namespace gbc;

extern "C" {

int gbc_mcl_prune_select_f32(gbc_context *ctx, const gbc_result *C, float thr, int64_t select, gbc_result **out)
{
    if (!ctx || !C || !out) return fail(GBC_EINVAL, "null argument");
    if (C->valtype != GBC_F32) return fail(GBC_EINVAL, "MCL prune/select expects fp32 values");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    return mcl_select_device2(ctx, C->nrow, C->nzc, nullptr, nullptr, C->cp, C->ir, static_cast<const float *>(C->num),
                              nullptr, nullptr, nullptr, thr, select, C->jc, out);
}

}  // extern "C"
