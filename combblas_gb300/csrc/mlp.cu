// The sizing MLP (6 -> 32 -> 32 -> 1, ReLU), trained and evaluated by the
// kernels in this file.  Training is full-batch Adam on the mean squared
// error of normalised log2(1 + nnz) targets; per-parameter gradients are sums
// over samples reduced in a fixed order (one block per parameter, fixed tree),
// so training is deterministic.
#include <cmath>
#include <cstring>
#include <vector>

#include "mlp.cuh"

namespace gbc {

namespace {

// per-sample quantities kept for the gradient reduction (structure of arrays)
constexpr int kCX = 0;              // x[kNF] (normalised)
constexpr int kCH1 = kCX + kNF;     // h1[kH1]
constexpr int kCH2 = kCH1 + kH1;    // h2[kH2]
constexpr int kCD1 = kCH2 + kH2;    // dL/d(pre-activation 1)[kH1]
constexpr int kCD2 = kCD1 + kH1;    // dL/d(pre-activation 2)[kH2]
constexpr int kCDY = kCD2 + kH2;    // dL/dy
constexpr int kCE2 = kCDY + 1;      // squared error
constexpr int kNC = kCE2 + 1;

__device__ __forceinline__ void mlp_forward(const float *P, const float *x, float *h1, float *h2, float &y)
{
#pragma unroll 4
    for (int i = 0; i < kH1; ++i) {
        float z = P[kOffB1 + i];
#pragma unroll
        for (int f = 0; f < kNF; ++f) z += P[kOffW1 + i * kNF + f] * x[f];
        h1[i] = z > 0.f ? z : 0.f;
    }
    for (int i = 0; i < kH2; ++i) {
        float z = P[kOffB2 + i];
#pragma unroll 8
        for (int j = 0; j < kH1; ++j) z += P[kOffW2 + i * kH1 + j] * h1[j];
        h2[i] = z > 0.f ? z : 0.f;
    }
    float o = P[kOffB3];
#pragma unroll 8
    for (int j = 0; j < kH2; ++j) o += P[kOffW3 + j] * h2[j];
    y = o;
}

__device__ __forceinline__ void normalise(const float *norm, const float *raw, float *x)
{
#pragma unroll
    for (int f = 0; f < kNF; ++f) x[f] = (raw[f] - norm[f]) / norm[kNF + f];
}

__global__ void k_mlp_predict(const float *params, const float *norm, const float *feat, int64_t n, float *pred)
{
    __shared__ float P[kNP];
    __shared__ float N[kNNorm];
    for (int k = threadIdx.x; k < kNP; k += blockDim.x) P[k] = params[k];
    for (int k = threadIdx.x; k < kNNorm; k += blockDim.x) N[k] = norm[k];
    __syncthreads();
    for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < n; s += int64_t(gridDim.x) * blockDim.x) {
        float x[kNF], h1[kH1], h2[kH2], y;
        normalise(N, feat + s * kNF, x);
        mlp_forward(P, x, h1, h2, y);
        pred[s] = y * N[2 * kNF + 1] + N[2 * kNF];
    }
}

__global__ void k_mlp_fwd_bwd(const float *params, const float *norm, const float *feat, const float *target,
                              int64_t n, float *buf)
{
    __shared__ float P[kNP];
    __shared__ float N[kNNorm];
    for (int k = threadIdx.x; k < kNP; k += blockDim.x) P[k] = params[k];
    for (int k = threadIdx.x; k < kNNorm; k += blockDim.x) N[k] = norm[k];
    __syncthreads();
    for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < n; s += int64_t(gridDim.x) * blockDim.x) {
        float x[kNF], h1[kH1], h2[kH2], y;
        normalise(N, feat + s * kNF, x);
        mlp_forward(P, x, h1, h2, y);
        const float t = (target[s] - N[2 * kNF]) / N[2 * kNF + 1];
        const float e = y - t;
        const float dy = 2.f * e;
        float d2[kH2];
        for (int i = 0; i < kH2; ++i) d2[i] = h2[i] > 0.f ? dy * P[kOffW3 + i] : 0.f;
        for (int f = 0; f < kNF; ++f) buf[(int64_t)(kCX + f) * n + s] = x[f];
        for (int i = 0; i < kH1; ++i) buf[(int64_t)(kCH1 + i) * n + s] = h1[i];
        for (int i = 0; i < kH2; ++i) buf[(int64_t)(kCH2 + i) * n + s] = h2[i];
        for (int j = 0; j < kH1; ++j) {
            float g = 0.f;
            for (int i = 0; i < kH2; ++i) g += P[kOffW2 + i * kH1 + j] * d2[i];
            buf[(int64_t)(kCD1 + j) * n + s] = h1[j] > 0.f ? g : 0.f;
        }
        for (int i = 0; i < kH2; ++i) buf[(int64_t)(kCD2 + i) * n + s] = d2[i];
        buf[(int64_t)kCDY * n + s] = dy;
        buf[(int64_t)kCE2 * n + s] = e * e;
    }
}

// One block per parameter (plus one for the loss): mean over samples of the
// parameter's gradient term, summed in a fixed order.
__global__ void k_mlp_grad_reduce(const float *buf, int64_t n, float *grad)
{
    const int p = blockIdx.x;
    int ca, cb;  // gradient = mean over s of buf[ca][s] * (cb >= 0 ? buf[cb][s] : 1)
    if (p < kOffB1) {
        ca = kCD1 + (p - kOffW1) / kNF;
        cb = kCX + (p - kOffW1) % kNF;
    } else if (p < kOffW2) {
        ca = kCD1 + (p - kOffB1);
        cb = -1;
    } else if (p < kOffB2) {
        ca = kCD2 + (p - kOffW2) / kH1;
        cb = kCH1 + (p - kOffW2) % kH1;
    } else if (p < kOffW3) {
        ca = kCD2 + (p - kOffB2);
        cb = -1;
    } else if (p < kOffB3) {
        ca = kCDY;
        cb = kCH2 + (p - kOffW3);
    } else if (p == kOffB3) {
        ca = kCDY;
        cb = -1;
    } else {
        ca = kCE2;
        cb = -1;
    }
    double acc = 0.0;
    for (int64_t s = threadIdx.x; s < n; s += blockDim.x) {
        const double a = buf[(int64_t)ca * n + s];
        acc += cb >= 0 ? a * (double)buf[(int64_t)cb * n + s] : a;
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) grad[p] = (float)(red[0] / (double)n);
}

__global__ void k_mlp_adam(float *params, float *m, float *v, const float *grad, float lr, float b1, float b2,
                           float eps, float c1, float c2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kNP) return;
    const float g = grad[p];
    const float mm = b1 * m[p] + (1.f - b1) * g;
    const float vv = b2 * v[p] + (1.f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    params[p] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// Feature means and standard deviations (one block, fixed order).
__global__ void k_mlp_norm(const float *feat, const float *target, int64_t n, float *norm)
{
    __shared__ double red[256];
    for (int c = 0; c <= kNF; ++c) {
        double mean = 0, sq = 0;
        for (int pass = 0; pass < 2; ++pass) {
            double acc = 0;
            for (int64_t s = threadIdx.x; s < n; s += blockDim.x) {
                const double x = c < kNF ? feat[s * kNF + c] : target[s];
                acc += pass == 0 ? x : (x - mean) * (x - mean);
            }
            red[threadIdx.x] = acc;
            __syncthreads();
            for (int w = blockDim.x / 2; w > 0; w >>= 1) {
                if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
                __syncthreads();
            }
            if (pass == 0)
                mean = red[0] / (double)(n > 0 ? n : 1);
            else
                sq = red[0] / (double)(n > 0 ? n : 1);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            const float sd = sq > 1e-12 ? (float)sqrt(sq) : 1.0f;
            if (c < kNF) {
                norm[c] = (float)mean;
                norm[kNF + c] = sd;
            } else {
                norm[2 * kNF] = (float)mean;
                norm[2 * kNF + 1] = sd;
            }
        }
        __syncthreads();
    }
}

uint64_t splitmix(uint64_t &x)
{
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

std::vector<float> init_params(uint64_t seed)
{
    std::vector<float> P(kNP, 0.f);
    auto unif = [&](float lim) { return (float)((splitmix(seed) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0) * lim; };
    const float l1 = std::sqrt(6.f / (kNF + kH1)), l2 = std::sqrt(6.f / (kH1 + kH2)), l3 = std::sqrt(6.f / (kH2 + 1));
    for (int k = 0; k < kH1 * kNF; ++k) P[kOffW1 + k] = unif(l1);
    for (int k = 0; k < kH2 * kH1; ++k) P[kOffW2 + k] = unif(l2);
    for (int k = 0; k < kH2; ++k) P[kOffW3 + k] = unif(l3);
    for (int k = 0; k < kH1; ++k) P[kOffB1 + k] = 0.01f;
    for (int k = 0; k < kH2; ++k) P[kOffB2 + k] = 0.01f;
    return P;
}

template <typename T>
int to_device(Workspace &ws, const T *src, size_t n, int where, const T **out)
{
    if (where == GBC_DEVICE || n == 0) {
        *out = src;
        return GBC_OK;
    }
    T *d = nullptr;
    GBC_TRY(ws.alloc_n(&d, n));
    GBC_CUDA_TRY(cudaMemcpyAsync(d, src, n * sizeof(T), cudaMemcpyHostToDevice, ws.ctx->stream));
    *out = d;
    return GBC_OK;
}

// Full-batch gradient at the current parameters (grad[kNP] = parameter
// gradients, grad[kNP] = mean squared error), device outputs.
int mlp_gradient(Mlp *m, Workspace &ws, const float *feat, const float *target, int64_t n, float *buf, float *grad)
{
    cudaStream_t s = m->ctx->stream;
    const int grid = (int)std::min<int64_t>((int64_t)m->ctx->num_sms * 4, (n + 255) / 256 + 1);
    k_mlp_fwd_bwd<<<grid, 256, 0, s>>>(m->params, m->norm, feat, target, n, buf);
    note_launch();
    k_mlp_grad_reduce<<<kNP + 1, 256, 0, s>>>(buf, n, grad);
    note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    (void)ws;
    return GBC_OK;
}

}  // namespace

int mlp_predict_device(Mlp *m, const float *feat, int64_t n, float *pred, cudaStream_t s)
{
    if (n <= 0) return GBC_OK;
    const int grid = (int)std::min<int64_t>((int64_t)m->ctx->num_sms * 4, (n + 255) / 256);
    k_mlp_predict<<<grid, 256, 0, s>>>(m->params, m->norm, feat, n, pred);
    note_launch();
    GBC_CUDA_TRY(cudaGetLastError());
    return GBC_OK;
}

}  // namespace gbc

using namespace gbc;

extern "C" {

int gbc_mlp_destroy(gbc_mlp *m);

int gbc_mlp_create(gbc_context *ctx, uint64_t seed, gbc_mlp **out)
{
    if (!ctx || !out) return fail(GBC_EINVAL, "null argument");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    gbc_mlp *m = new gbc_mlp();
    m->ctx = ctx;
    int rc = device_alloc(ctx, (void **)&m->params, kNP * sizeof(float));
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&m->adam_m, kNP * sizeof(float));
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&m->adam_v, kNP * sizeof(float));
    if (rc == GBC_OK) rc = device_alloc(ctx, (void **)&m->norm, kNNorm * sizeof(float));
    if (rc != GBC_OK) {
        gbc_mlp_destroy(m);
        return rc;
    }
    std::vector<float> P = init_params(seed);
    std::vector<float> N(kNNorm, 0.f);
    for (int f = 0; f < kNF; ++f) N[kNF + f] = 1.f;
    N[2 * kNF + 1] = 1.f;
    cudaStream_t s = ctx->stream;
    cudaMemcpyAsync(m->params, P.data(), kNP * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(m->adam_m, 0, kNP * sizeof(float), s);
    cudaMemsetAsync(m->adam_v, 0, kNP * sizeof(float), s);
    cudaMemcpyAsync(m->norm, N.data(), kNNorm * sizeof(float), cudaMemcpyHostToDevice, s);
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    *out = m;
    return GBC_OK;
}

int gbc_mlp_destroy(gbc_mlp *m)
{
    if (!m) return GBC_OK;
    Context *c = m->ctx;
    device_free(c, m->params);
    device_free(c, m->adam_m);
    device_free(c, m->adam_v);
    device_free(c, m->norm);
    cudaStreamSynchronize(c->stream);
    delete m;
    return GBC_OK;
}

int gbc_mlp_num_params(void) { return kNP + kNNorm; }

// Parameters then normalisation block (kNP + kNNorm floats), host memory.
int gbc_mlp_get(gbc_mlp *m, float *host, float *margin)
{
    if (!m) return fail(GBC_EINVAL, "null model");
    cudaStream_t s = m->ctx->stream;
    if (host) {
        GBC_CUDA_TRY(cudaMemcpyAsync(host, m->params, kNP * sizeof(float), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(host + kNP, m->norm, kNNorm * sizeof(float), cudaMemcpyDeviceToHost, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
    }
    if (margin) *margin = m->margin;
    return GBC_OK;
}

int gbc_mlp_set(gbc_mlp *m, const float *host, float margin)
{
    if (!m) return fail(GBC_EINVAL, "null model");
    cudaStream_t s = m->ctx->stream;
    if (host) {
        GBC_CUDA_TRY(cudaMemcpyAsync(m->params, host, kNP * sizeof(float), cudaMemcpyHostToDevice, s));
        GBC_CUDA_TRY(cudaMemcpyAsync(m->norm, host + kNP, kNNorm * sizeof(float), cudaMemcpyHostToDevice, s));
        GBC_CUDA_TRY(cudaStreamSynchronize(s));
        m->trained = true;
    }
    m->margin = margin;
    return GBC_OK;
}

// Full-batch gradient at the current parameters (host output grad[kNP + 1]:
// parameter gradients then the mean squared error), with the model's current
// normalisation.  Used to check the backward kernels against the oracle.
int gbc_mlp_gradient(gbc_context *ctx, gbc_mlp *m, const float *feat, const float *target, int64_t n, float *grad,
                     int where)
{
    if (!ctx || !m || n <= 0) return fail(GBC_EINVAL, "bad argument");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    Workspace ws(ctx);
    const float *df = nullptr, *dt = nullptr;
    GBC_TRY(to_device(ws, feat, (size_t)n * kNF, where, &df));
    GBC_TRY(to_device(ws, target, (size_t)n, where, &dt));
    float *buf = nullptr, *g = nullptr;
    GBC_TRY(ws.alloc_n(&buf, (size_t)kNC * n));
    GBC_TRY(ws.alloc_n(&g, kNP + 1));
    GBC_TRY(mlp_gradient(m, ws, df, dt, n, buf, g));
    GBC_CUDA_TRY(cudaMemcpyAsync(grad, g, (kNP + 1) * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    GBC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return GBC_OK;
}

// Train on (features, log2(1 + nnz) targets): normalisation from the data,
// then `steps` full-batch Adam steps.  *loss_out = final mean squared error
// in normalised units; *resid_out (optional) = standard deviation of the
// prediction error in log2 units, from which the caller sets the margin.
int gbc_mlp_train(gbc_context *ctx, gbc_mlp *m, const float *feat, const float *target, int64_t n, int steps,
                  float lr, float *loss_out, int where)
{
    if (!ctx || !m || n <= 0 || steps < 0) return fail(GBC_EINVAL, "bad argument");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    const float *df = nullptr, *dt = nullptr;
    GBC_TRY(to_device(ws, feat, (size_t)n * kNF, where, &df));
    GBC_TRY(to_device(ws, target, (size_t)n, where, &dt));
    float *buf = nullptr, *g = nullptr;
    GBC_TRY(ws.alloc_n(&buf, (size_t)kNC * n));
    GBC_TRY(ws.alloc_n(&g, kNP + 1));
    k_mlp_norm<<<1, 256, 0, s>>>(df, dt, n, m->norm);
    note_launch();
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < steps; ++it) {
        GBC_TRY(mlp_gradient(m, ws, df, dt, n, buf, g));
        ++m->steps;
        const float c1 = 1.f - std::pow(b1, (float)m->steps), c2 = 1.f - std::pow(b2, (float)m->steps);
        k_mlp_adam<<<(kNP + 255) / 256, 256, 0, s>>>(m->params, m->adam_m, m->adam_v, g, lr, b1, b2, eps, c1, c2);
        note_launch();
    }
    GBC_TRY(mlp_gradient(m, ws, df, dt, n, buf, g));
    float loss = 0;
    GBC_CUDA_TRY(cudaMemcpyAsync(&loss, g + kNP, sizeof(float), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    if (loss_out) *loss_out = loss;
    m->trained = true;
    return GBC_OK;
}

int gbc_mlp_predict(gbc_context *ctx, gbc_mlp *m, const float *feat, int64_t n, float *pred, int where)
{
    if (!ctx || !m || n < 0) return fail(GBC_EINVAL, "bad argument");
    GBC_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    Workspace ws(ctx);
    const float *df = nullptr;
    GBC_TRY(to_device(ws, feat, (size_t)n * kNF, where, &df));
    float *dp = pred;
    if (where == GBC_HOST) GBC_TRY(ws.alloc_n(&dp, n + 1));
    GBC_TRY(mlp_predict_device(m, df, n, dp, s));
    if (where == GBC_HOST && n > 0)
        GBC_CUDA_TRY(cudaMemcpyAsync(pred, dp, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    GBC_CUDA_TRY(cudaStreamSynchronize(s));
    return GBC_OK;
}

}  // extern "C"
