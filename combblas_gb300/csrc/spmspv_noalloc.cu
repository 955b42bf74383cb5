// Allocation-free variant of the Select2ndMin sparse-matrix x sparse-vector
// product (gbc_spmspv_select2ndmin_noalloc).
//
// Why it exists: some callers cannot call cudaMalloc at the point where they
// need this product -- for example code that runs while another component
// (a caching allocator, a communication runtime) has already reserved the
// device's free memory, code on latency-critical paths that cannot afford
// the implicit device-wide synchronisation of cudaMalloc/cudaFree, or code
// whose environment forbids driver allocations after start-up.  This entry
// point therefore takes every input and output as caller-provided device
// memory and keeps its working storage in one file-scope __device__ array.
// The CUDA runtime reserves that array when it loads this file's device
// code on a device; with lazy module loading (the runtime's default) that
// happens at the first use on each device, i.e. inside the first call of
// this entry point, which then needs the array's ~8.4 MB to be free.
// Callers should therefore make one warm-up call per device at start-up
// (nrow = 0 and veclen = 0 is enough), while memory is still available.
//
// Limits and rules (also stated in include/gbcomb.h):
//  * the matrix may have at most kNoAllocMaxRows rows; larger inputs are
//    rejected with GBC_EOVERFLOW before anything runs;
//  * the array is reserved on every GPU that loads the library and is held
//    until the process exits (about 8.4 MB);
//  * every call shares the array and it keeps the previous call's contents;
//    each call clears what must start empty.  Calls whose work overlaps on
//    the GPU (different streams, or host threads racing) corrupt each other
//    and must be serialised by the caller;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it.  If
//    the lookup reports an error the cache entry stays empty and the next
//    call tries again;
//  * every call reads its error flag and output count back to the host and
//    waits for `stream` to finish before it returns, so no call can be
//    captured into a CUDA graph.
#include <mutex>

#include "gbc_internal.cuh"

namespace gbc {
namespace {

constexpr int64_t kNoAllocMaxRows = int64_t(1) << 20;
constexpr int64_t kNoAllocWords = kNoAllocMaxRows / 32;
constexpr int kNaThreads = 256;
constexpr int kMaxDevices = 64;

// Working storage: spa[rows] (min candidate, sign-flipped so that unsigned
// min is signed min; all ones = empty), mark[rows/32] (touched rows),
// pos[rows/32 + 1] (output offset of each 32-row word), and a few counters.
struct NoAllocScratch {
    unsigned long long spa[kNoAllocMaxRows];
    uint32_t mark[kNoAllocWords];
    int64_t pos[kNoAllocWords + 1];
    unsigned long long work;
    int32_t err;
    int32_t pad;
};

__device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_addr_mu;
NoAllocScratch *g_addr[kMaxDevices] = {};

int scratch_address(int device, NoAllocScratch **out)
{
    if (device < 0 || device >= kMaxDevices) return fail(GBC_EINVAL, "device id out of range");
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();  // nothing is cached: the next call looks the address up again
            return fail(GBC_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        }
        g_addr[device] = static_cast<NoAllocScratch *>(p);
    }
    *out = g_addr[device];
    return GBC_OK;
}

__global__ void k_na_clear(NoAllocScratch *s, int64_t rows)
{
    const int64_t words = (rows + 31) / 32;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < rows; i += int64_t(gridDim.x) * blockDim.x) {
        s->spa[i] = ~0ull;
        if (i < words) s->mark[i] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        s->work = 0;
        s->err = 0;
    }
}

// One block takes kNaThreads vector entries at a time; their columns'
// entries are walked cooperatively (flattened with a block scan and a
// binary search over the per-entry offsets).
__global__ void __launch_bounds__(kNaThreads) k_na_expand(NoAllocScratch *s, int64_t rows, int64_t ncol,
                                                          int64_t nnz, const int64_t *cp, const int64_t *ir,
                                                          const int32_t *xind, const int64_t *xval, int64_t nx)
{
    __shared__ int64_t st[kNaThreads];
    __shared__ int32_t off[kNaThreads + 1];
    __shared__ int64_t val[kNaThreads];
    __shared__ int32_t wsum[kNaThreads / 32];
    __shared__ int64_t s_base;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (;;) {
        if (tid == 0) s_base = (int64_t)atomicAdd(&s->work, (unsigned long long)kNaThreads);
        __syncthreads();
        const int64_t base = s_base;
        __syncthreads();
        if (base >= nx) break;
        const int64_t f = base + tid;
        int len = 0;
        if (f < nx) {
            const int32_t c = xind[f];
            if (c < 0 || c >= ncol) {
                atomicOr(&s->err, 1);
            } else {
                const int64_t b = cp[c], e = cp[c + 1];
                if (b < 0 || e < b || e > nnz) {
                    atomicOr(&s->err, 2);
                } else {
                    st[tid] = b;
                    val[tid] = xval[f];
                    len = (int)(e - b);
                }
            }
        }
        // block exclusive scan of len
        int x = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[wid] = x;
        __syncthreads();
        int pre = 0, tot = 0;
        for (int w = 0; w < kNaThreads / 32; ++w) {
            if (w < wid) pre += wsum[w];
            tot += wsum[w];
        }
        off[tid] = pre + x - len;
        if (tid == kNaThreads - 1) off[kNaThreads] = tot;
        __syncthreads();
        for (int j = tid; j < tot; j += kNaThreads) {
            int lo = 0, hi = kNaThreads;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (off[mid] <= j)
                    lo = mid;
                else
                    hi = mid;
            }
            const int64_t r = ir[st[lo] + (j - off[lo])];
            if (r < 0 || r >= rows) {
                atomicOr(&s->err, 4);
                continue;
            }
            atomicMin(&s->spa[r], (unsigned long long)val[lo] ^ 0x8000000000000000ull);
            const uint32_t bit = 1u << (r & 31);
            if (!(s->mark[r >> 5] & bit)) atomicOr(&s->mark[r >> 5], bit);
        }
        __syncthreads();
    }
}

// Output offsets of the 32-row words: one block scans all words.
__global__ void __launch_bounds__(1024) k_na_positions(NoAllocScratch *s, int64_t words)
{
    __shared__ int64_t wsum[32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t per = (words + 1023) / 1024;
    const int64_t w0 = min(words, per * tid), w1 = min(words, w0 + per);
    int64_t c = 0;
    for (int64_t w = w0; w < w1; ++w) c += __popc(s->mark[w]);
    int64_t x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    int64_t pre = 0, tot = 0;
    for (int w = 0; w < 32; ++w) {
        if (w < wid) pre += wsum[w];
        tot += wsum[w];
    }
    int64_t run = pre + x - c;
    for (int64_t w = w0; w < w1; ++w) {
        s->pos[w] = run;
        run += __popc(s->mark[w]);
    }
    if (tid == 0) s->pos[words] = tot;
}

__global__ void k_na_emit(NoAllocScratch *s, int64_t words, int32_t *yind, int64_t *yval)
{
    const int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w >= words) return;
    uint32_t x = s->mark[w];
    int64_t p = s->pos[w];
    while (x) {
        const int b = __ffs(x) - 1;
        x &= x - 1;
        const int64_t r = w * 32 + b;
        yind[p] = (int32_t)r;
        yval[p] = (int64_t)(s->spa[r] ^ 0x8000000000000000ull);
        ++p;
    }
}

}  // namespace
}  // namespace gbc

using namespace gbc;

extern "C" {

int gbc_spmspv_select2ndmin_noalloc(int64_t nrow, int64_t ncol, int64_t nnz, const int64_t *cp, const int64_t *ir,
                                    const int32_t *indx, const int64_t *numx, int32_t veclen, int32_t *indy,
                                    int64_t *numy, int32_t *nnzy, void *stream)
{
    if (!nnzy) return fail(GBC_EINVAL, "null nnzy");
    if (nrow < 0 || ncol < 0 || nnz < 0 || veclen < 0) return fail(GBC_EINVAL, "negative size");
    if (nrow > kNoAllocMaxRows)
        return fail(GBC_EOVERFLOW, "gbc_spmspv_select2ndmin_noalloc handles at most 1048576 rows (its fixed "
                                   "working storage); use gbc_spmspv_select2ndmin_i64 for larger matrices");
    if ((ncol > 0 && !cp) || (nnz > 0 && !ir) || (veclen > 0 && (!indx || !numx)) || (nrow > 0 && (!indy || !numy)))
        return fail(GBC_EINVAL, "null array");
    int dev = 0;
    GBC_CUDA_TRY(cudaGetDevice(&dev));
    NoAllocScratch *sc = nullptr;
    GBC_TRY(scratch_address(dev, &sc));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t words = (nrow + 31) / 32;
    int num_sms = 0;
    GBC_CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
    k_na_clear<<<num_sms * 4, 256, 0, s>>>(sc, nrow);
    note_launch();
    if (veclen > 0) {
        const int64_t blocks = (veclen + kNaThreads - 1) / kNaThreads;
        k_na_expand<<<(unsigned)(blocks < num_sms * 4 ? blocks : num_sms * 4), kNaThreads, 0, s>>>(
            sc, nrow, ncol, nnz, cp, ir, indx, numx, veclen);
        note_launch();
    }
    k_na_positions<<<1, 1024, 0, s>>>(sc, words);
    note_launch();
    if (words > 0) {
        k_na_emit<<<(unsigned)((words + 255) / 256), 256, 0, s>>>(sc, words, indy, numy);
        note_launch();
    }
    GBC_CUDA_TRY(cudaGetLastError());
    int32_t err = 0;
    int64_t total = 0;
    GBC_CUDA_TRY(cudaMemcpyAsync(&err, &sc->err, sizeof(err), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaMemcpyAsync(&total, &sc->pos[words], sizeof(total), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    if (err) return fail(GBC_EINVAL, "vector index or matrix entry out of range");
    *nnzy = (int32_t)total;
    return GBC_OK;
}

}  // extern "C"
