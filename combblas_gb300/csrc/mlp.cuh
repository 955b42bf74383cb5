// Learned output-column sizing: a small MLP that predicts log2(1 + nnz) of
// each output column of C = A*B from per-column features, trained on the
// GPU on counts the exact symbolic pass produces.  It replaces the symbolic
// pass only for sizing: any column whose true count exceeds its predicted
// capacity is recomputed by the exact two-phase path, so the product itself
// is unchanged.
#pragma once

#include <stdint.h>

#include "gbc_internal.cuh"

namespace gbc {

constexpr int kNF = 6;   // features per column
constexpr int kH1 = 32;  // hidden widths
constexpr int kH2 = 32;
// parameter layout (floats): W1[kH1][kNF], b1[kH1], W2[kH2][kH1], b2[kH2], W3[kH2], b3
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kH1 * kNF;
constexpr int kOffW2 = kOffB1 + kH1;
constexpr int kOffB2 = kOffW2 + kH2 * kH1;
constexpr int kOffW3 = kOffB2 + kH2;
constexpr int kOffB3 = kOffW3 + kH2;
constexpr int kNP = kOffB3 + 1;
// normalisation block (floats): feature mean[kNF], feature std[kNF], target mean, target std
constexpr int kNNorm = 2 * kNF + 2;

struct Mlp {
    Context *ctx = nullptr;
    float *params = nullptr;  // device [kNP]
    float *adam_m = nullptr;  // device [kNP]
    float *adam_v = nullptr;  // device [kNP]
    float *norm = nullptr;    // device [kNNorm]
    int64_t steps = 0;        // Adam steps taken
    float margin = 1.0f;      // capacity = 2^(prediction + margin) (log2 units)
    bool trained = false;
};

// features[i*kNF + f] for the listed columns; computed in spgemm.cu.
// Predict log2(1 + nnz) for n feature rows (device arrays).
int mlp_predict_device(Mlp *m, const float *feat, int64_t n, float *pred, cudaStream_t s);

}  // namespace gbc

struct gbc_mlp : gbc::Mlp {};
