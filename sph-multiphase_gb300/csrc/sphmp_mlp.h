// sphmp_mlp.h — sizes, parameter layout and launchers of the corrector network
// (sphmp_mlp.cu). Host and device code include it.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sphmp.h"

namespace sphmp {
namespace mlp {

constexpr int kFeatures = 48;   // per-particle input features
constexpr int kInPad = 64;      // input width padded to a multiple of the MMA's K chunk
constexpr int kHidden = 128;    // width of the three hidden layers
constexpr int kOutputs = 4;     // velocity correction (3) + density correction
constexpr int kOutPad = 16;     // output width padded to the smallest MMA N

// FP32 master parameters, one flat array (PyTorch's Linear layout: W [out][in]).
constexpr int kOffParamW1 = 0;                                   // [128][48]
constexpr int kOffParamB1 = kOffParamW1 + kHidden * kFeatures;   // [128]
constexpr int kOffParamW2 = kOffParamB1 + kHidden;               // [128][128]
constexpr int kOffParamB2 = kOffParamW2 + kHidden * kHidden;     // [128]
constexpr int kOffParamW3 = kOffParamB2 + kHidden;               // [128][128]
constexpr int kOffParamB3 = kOffParamW3 + kHidden * kHidden;     // [128]
constexpr int kOffParamW4 = kOffParamB3 + kHidden;               // [4][128]
constexpr int kOffParamB4 = kOffParamW4 + kOutputs * kHidden;    // [4]
constexpr int kParams = kOffParamB4 + kOutputs;                  // 39,812

constexpr uint32_t kErrMmaTimeout = 1u << SPHMP_ERR_TIMEOUT;

// Device operands of the forward pass: padded bf16 weights (K-major rows),
// biases [b1 | b2 | b3 | b4 padded to 16], feature normalisation.
struct Packed {
    const __nv_bfloat16* w1;  // [128][64]
    const __nv_bfloat16* w2;  // [128][128]
    const __nv_bfloat16* w3;  // [128][128]
    const __nv_bfloat16* w4;  // [16][128]
    const float* bias;        // [3 * 128 + 16]
    const float* fshift;      // [48]: input = (feature - shift) * scale
    const float* fscale;      // [48]
};

struct PackedMut {
    __nv_bfloat16 *w1, *w2, *w3, *w4;
    __nv_bfloat16 *w2t, *w3t, *w4t;  // transposes for the backward pass: [128][128], [128][128], [128][16]
    float* bias;
};

// Training saves of the forward pass (all null for inference): the hidden
// layers' pre-activations z in FP16 and the bf16 layer inputs, all transposed
// ([width][ldh], feature-major).
struct Saves {
    __half *z1, *z2, *z3;
    __nv_bfloat16 *h0t, *h1t, *h2t, *h3t;  // h0t [64][ldh] (rows 48..63 zero), the others [128][ldh]
    int ldh;
};

cudaError_t launch_forward(const float* x, int n, const Packed& W, const Saves& S, float* y, uint32_t* err,
                           int num_sms, cudaStream_t s);
// D[split][M][N] = A[M][K] B[N][K]^T over the split's K range; N a multiple of 16, <= 128
cudaError_t launch_gemm_tn(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, float* D, int M, int N,
                           int K, int splits, uint32_t* err, cudaStream_t s);
// One Adam step (bias-corrected; lr <= 0: none) applied where the gradients are
// formed, each updated parameter also written into its bf16 operand positions
// (the padding of the packed layouts is written once by launch_pack).
struct AdamStep {
    float *p, *m, *v;
    float lr, b1, b2, eps, c1, c2;  // c1, c2: 1 - beta^step
    PackedMut w;
};
AdamStep adam_step(float* p, float* m, float* v, float lr, float b1, float b2, float eps, int step,
                   const PackedMut& w);

// The whole backward pass after launch_out_grad (fused, one persistent CTA per
// SM): gradients of every parameter into grads (flat layout), then the Adam
// step if adam.lr > 0. batch a multiple of 128; part: scratch of num_sms *
// kParams floats.
cudaError_t launch_backward(const __nv_bfloat16* dy, const Saves& S, const PackedMut& W, int batch, float* part,
                            float* grads, const AdamStep& adam, uint32_t* err, int num_sms, cudaStream_t s);
// dY (bf16 [batch][16], zero padded; transposed into dyt [4][ld] unless null) and
// the loss into *loss (unless null)
cudaError_t launch_out_grad(const float* y, const float* t, int batch, int ld, __nv_bfloat16* dy,
                            __nv_bfloat16* dyt, float* loss_part, float* loss, cudaStream_t s);
cudaError_t launch_pack(const float* p, const PackedMut& W, cudaStream_t s);

}  // namespace mlp
}  // namespace sphmp
