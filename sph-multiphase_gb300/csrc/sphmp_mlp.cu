// sphmp_mlp.cu — the learned large-step corrector's network on the tensor cores:
// a per-particle MLP 48 -> 128 -> 128 -> 128 -> 4 with SiLU, bf16 weights and
// activations, FP32 accumulation in TMEM (tcgen05.mma kind::f16), its backward
// pass and Adam.
//
// * k_mlp_forward: all four layers of 128-particle tiles in one persistent
//   kernel, four tiles in flight per CTA. The weights stay in shared memory;
//   each layer is one chain of MMAs
//   into TMEM, and its epilogue (bias, SiLU, bf16) writes the next layer's
//   operand tile back into shared memory. With the training saves it also
//   stores z of each hidden layer (FP16) and the bf16 layer inputs transposed
//   (feature-major), the operands of the backward pass.
// * k_mlp_backward: the whole backward pass in one persistent kernel, one CTA
//   per SM over 128-row tiles: dH GEMMs, the SiLU backward in their epilogues,
//   and the weight and bias gradients accumulated in TMEM over the CTA's tiles;
//   k_sum_partials adds the CTAs' partial gradients in a fixed order.
// * k_gemm_tn: D = A B^T for K-major bf16 A [M][K] and B [N][K] (N <= 128),
//   M in tiles of 128, K split over gridDim.y into FP32 partials (the library's
//   GEMM entry point).
// * elementwise kernels: the output gradient, the sum of the partial gradients
//   with the Adam step, and the packing of the FP32 master parameters into the
//   padded bf16 operand layouts.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "sphmp_mlp.h"
#include "sphmp_tc.cuh"

namespace sphmp {
namespace mlp {

using bf16 = __nv_bfloat16;

namespace {

// SiLU of the forward pass as z/2 (1 + tanh(z/2)) with the hardware tanh
// (tanh.approx.f32, relative error about 2^-11, below the bf16 rounding of the
// result): one special-function operation per element instead of two (exp and
// reciprocal), which bound the forward kernel's epilogues.
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float silu(float z) {
    const float hz = 0.5f * z;
    return fmaf(hz, tanh_approx(hz), hz);
}

__device__ __forceinline__ float silu_grad(float z) {
    const float s = __fdividef(1.f, 1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// ---------------------------------------------------------------------------
// Fused forward
// ---------------------------------------------------------------------------

constexpr int kGroups = 4;                     // tiles in flight per CTA
constexpr int kGroupThreads = 128;             // 4 warps: one TMEM lane quadrant each
constexpr int kFwdThreads = kGroups * kGroupThreads;
constexpr int kTile = 128;
// dynamic shared memory of the forward kernel
constexpr int kOffW1 = 0;                                  // [128 rows][64] kc 64
constexpr int kOffW2 = kOffW1 + kHidden * kInPad * 2;      // [128][128]
constexpr int kOffW3 = kOffW2 + kHidden * kHidden * 2;     // [128][128]
constexpr int kOffW4 = kOffW3 + kHidden * kHidden * 2;     // [16][128]
constexpr int kOffAct = kOffW4 + kOutPad * kHidden * 2;    // kGroups x [128][128] operand tiles
constexpr int kActBytes = kTile * kHidden * 2;
constexpr int kOffBias = kOffAct + kGroups * kActBytes;    // 3 * 128 + 16 floats
constexpr int kOffNorm = kOffBias + (3 * kHidden + kOutPad) * 4;  // shift[48], scale[48]
constexpr int kFwdSmem = kOffNorm + 2 * kFeatures * 4;
// TMEM: group g uses columns [128 g, 128 g + 128) for layers 1-3 and the first
// 16 of them again for layer 4 (after layer 3's epilogue has read them)
constexpr uint32_t kGroupTmemCols = 128;
constexpr uint32_t kFwdTmemCols = kGroups * kGroupTmemCols;
static_assert(kFwdTmemCols <= 512, "TMEM holds 512 columns");
static_assert(kFwdSmem > 116 * 1024, "one CTA per SM: the TMEM allocation takes every column");
static_assert(kFwdSmem <= 227 * 1024, "shared memory of one CTA");

__device__ __forceinline__ void stage_weights(uint8_t* dst, const bf16* src, int rows, int kc, int tid,
                                              int nthreads) {
    for (int q = tid; q < rows * (kc / 8); q += nthreads) {
        const int r = q / (kc / 8), k = (q % (kc / 8)) * 8;
        *reinterpret_cast<uint4*>(dst + tc::kmajor_offset(r, k, kc)) =
            *reinterpret_cast<const uint4*>(src + (size_t)r * kc + k);
    }
}

// one MMA chain: D[tmem_col ...] = act (K = kc) x W^T (N rows)
__device__ __forceinline__ void issue_layer(uint32_t tmem, uint32_t act, uint32_t w, int kc, int n, uint64_t* bar) {
    const uint32_t idesc = tc::idesc_bf16_f32(kTile, n);
    for (int ks = 0; ks < kc / 16; ks++)
        tc::mma_bf16(tmem, tc::kmajor_desc(act, kc, ks), tc::kmajor_desc(w, kc, ks), idesc, ks > 0 ? 1u : 0u);
    tc::mma_commit(bar);
}

// Every thread of the CTA waits; the CTA agrees on the outcome (a barrier).
__device__ __forceinline__ bool wait_all(uint64_t* bar, uint32_t& parity) {
    const bool ok = tc::mbar_wait(bar, parity, tc::kWaitLimitNs);
    parity ^= 1u;
    const bool all = __syncthreads_and(ok) != 0;
    tc::fence_after_sync();
    return all;
}

// shared-memory writes of this thread done: order them before the next MMA
__device__ __forceinline__ void handoff_to_mma() {
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
}

// The same for the 128 threads of one tile group (named barrier 1 + g).
__device__ __forceinline__ void group_sync(int g) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(kGroupThreads) : "memory");
}
__device__ __forceinline__ bool group_all(int g, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + g), "r"(kGroupThreads)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ bool group_wait(uint64_t* bar, uint32_t& parity, int g) {
    const bool ok = tc::mbar_wait(bar, parity, tc::kWaitLimitNs);
    parity ^= 1u;
    const bool all = group_all(g, ok);
    tc::fence_after_sync();
    return all;
}
__device__ __forceinline__ void group_handoff(int g) {
    tc::fence_async_smem();
    tc::fence_before_sync();
    group_sync(g);
}

// Epilogue of a hidden layer for this thread's row (all 128 columns): bias +
// SiLU, the bf16 activations into the operand tile (K = 128), the training saves.
__device__ __forceinline__ void hidden_epilogue(uint32_t tmem, int warp, int lane, const float* bias, uint8_t* act,
                                                int row0, int n, __half* z_save, bf16* ht_save, int ldh) {
    const int r = (warp & 3) * 32 + lane;
    const int grow = row0 + r;
    const bool live = grow < n;
#pragma unroll 1
    for (int c0 = 0; c0 < kHidden; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tc::tmem_lane_addr(tmem, warp, c0), v);
        float h[16];
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const float z = v[i] + bias[c0 + i];
            v[i] = z;
            h[i] = silu(z);
        }
        uint4 lo, hi;
        lo.x = pack2(h[0], h[1]); lo.y = pack2(h[2], h[3]); lo.z = pack2(h[4], h[5]); lo.w = pack2(h[6], h[7]);
        hi.x = pack2(h[8], h[9]); hi.y = pack2(h[10], h[11]); hi.z = pack2(h[12], h[13]); hi.w = pack2(h[14], h[15]);
        *reinterpret_cast<uint4*>(act + tc::kmajor_offset(r, c0, kHidden)) = lo;
        *reinterpret_cast<uint4*>(act + tc::kmajor_offset(r, c0 + 8, kHidden)) = hi;
        // the training saves, transposed ([feature][row]): rows 2k and 2k + 1 are adjacent,
        // so the even lane stores both with one 32-bit store (a warp writes 64 contiguous
        // bytes per feature): z in FP16 (relative error 2^-11) and the bf16 activations
        if (ht_save) {
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const float oh = __shfl_down_sync(0xffffffffu, h[i], 1);
                const float oz = __shfl_down_sync(0xffffffffu, v[i], 1);
                const size_t at = (size_t)(c0 + i) * ldh + grow;
                if ((lane & 1) == 0 && grow + 1 < n) {
                    *reinterpret_cast<uint32_t*>(ht_save + at) = pack2(h[i], oh);
                    const __half2 zz = __floats2half2_rn(v[i], oz);
                    *reinterpret_cast<__half2*>(z_save + at) = zz;
                } else if ((lane & 1) == 0 && live) {
                    ht_save[at] = __float2bfloat16_rn(h[i]);
                    z_save[at] = __float2half_rn(v[i]);
                }
            }
        }
    }
}

// kGroups independent tile pipelines per CTA (4 warps each), so that one
// group's epilogue runs while the others' MMAs and loads are in flight; the
// weights in shared memory are shared.
__global__ void __launch_bounds__(kFwdThreads, 1) k_mlp_forward(const float* __restrict__ x, int n,
                                                                 const Packed W, const Saves S,
                                                                 float* __restrict__ y, uint32_t* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bars[kGroups];
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = tid / kGroupThreads, gt = tid % kGroupThreads;
    uint8_t* act = smem + kOffAct + g * kActBytes;
    float* bias = reinterpret_cast<float*>(smem + kOffBias);
    float* fshift = reinterpret_cast<float*>(smem + kOffNorm);
    float* fscale = fshift + kFeatures;

    stage_weights(smem + kOffW1, W.w1, kHidden, kInPad, tid, kFwdThreads);
    stage_weights(smem + kOffW2, W.w2, kHidden, kHidden, tid, kFwdThreads);
    stage_weights(smem + kOffW3, W.w3, kHidden, kHidden, tid, kFwdThreads);
    stage_weights(smem + kOffW4, W.w4, kOutPad, kHidden, tid, kFwdThreads);
    for (int i = tid; i < 3 * kHidden + kOutPad; i += kFwdThreads) bias[i] = W.bias[i];
    for (int i = tid; i < kFeatures; i += kFwdThreads) {
        fshift[i] = W.fshift[i];
        fscale[i] = W.fscale[i];
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, kFwdTmemCols);
        tc::tmem_relinquish();
    }
    if (tid == 0)
        for (int k = 0; k < kGroups; k++) tc::mbar_init(&bars[k], 1);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base + (uint32_t)g * kGroupTmemCols;
    const uint32_t a_act = tc::smem_addr(act);
    uint64_t* bar = &bars[g];
    uint32_t parity = 0;
    bool ok = true;
    const int ntiles = (n + kTile - 1) / kTile;
    for (int t = kGroups * blockIdx.x + g; t < ntiles && ok; t += kGroups * gridDim.x) {
        const int row0 = t * kTile;
        // input tile: normalised features, bf16, K padded to 64 with zeros
        {
            const int r = gt;
            const int grow = row0 + r;
            const bool live = grow < n;
            const float4* src = reinterpret_cast<const float4*>(x + (size_t)(live ? grow : 0) * kFeatures);
#pragma unroll 2
            for (int c = 0; c < kFeatures / 8; c++) {  // 8 features at a time
                float f[8];
                const float4 a = live ? src[2 * c] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 b = live ? src[2 * c + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
                f[0] = a.x; f[1] = a.y; f[2] = a.z; f[3] = a.w; f[4] = b.x; f[5] = b.y; f[6] = b.z; f[7] = b.w;
#pragma unroll
                for (int i = 0; i < 8; i++) f[i] = live ? (f[i] - fshift[8 * c + i]) * fscale[8 * c + i] : 0.f;
                uint4 q;
                q.x = pack2(f[0], f[1]); q.y = pack2(f[2], f[3]); q.z = pack2(f[4], f[5]); q.w = pack2(f[6], f[7]);
                *reinterpret_cast<uint4*>(act + tc::kmajor_offset(r, 8 * c, kInPad)) = q;
                if (S.h0t) {  // transposed, a 32-bit store per row pair (as in the hidden layers)
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const float o = __shfl_down_sync(0xffffffffu, f[i], 1);
                        bf16* dst = S.h0t + (size_t)(8 * c + i) * S.ldh + grow;
                        if ((gt & 1) == 0 && grow + 1 < n) *reinterpret_cast<uint32_t*>(dst) = pack2(f[i], o);
                        else if ((gt & 1) == 0 && live) *dst = __float2bfloat16_rn(f[i]);
                    }
                }
            }
            const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
            *reinterpret_cast<uint4*>(act + tc::kmajor_offset(r, 48, kInPad)) = zero;
            *reinterpret_cast<uint4*>(act + tc::kmajor_offset(r, 56, kInPad)) = zero;
        }
        group_handoff(g);
        // layer 1
        if (gt == 0) {
            tc::fence_after_sync();
            issue_layer(tmem, a_act, tc::smem_addr(smem + kOffW1), kInPad, kHidden, bar);
        }
        if (!(ok = group_wait(bar, parity, g))) break;
        hidden_epilogue(tmem, warp, lane, bias, act, row0, n, S.z1, S.h1t, S.ldh);
        group_handoff(g);
        // layer 2
        if (gt == 0) {
            tc::fence_after_sync();
            issue_layer(tmem, a_act, tc::smem_addr(smem + kOffW2), kHidden, kHidden, bar);
        }
        if (!(ok = group_wait(bar, parity, g))) break;
        hidden_epilogue(tmem, warp, lane, bias + kHidden, act, row0, n, S.z2, S.h2t, S.ldh);
        group_handoff(g);
        // layer 3
        if (gt == 0) {
            tc::fence_after_sync();
            issue_layer(tmem, a_act, tc::smem_addr(smem + kOffW3), kHidden, kHidden, bar);
        }
        if (!(ok = group_wait(bar, parity, g))) break;
        hidden_epilogue(tmem, warp, lane, bias + 2 * kHidden, act, row0, n, S.z3, S.h3t, S.ldh);
        group_handoff(g);
        // layer 4 (N = 16: outputs 0..3 and zero padding)
        if (gt == 0) {
            tc::fence_after_sync();
            issue_layer(tmem, a_act, tc::smem_addr(smem + kOffW4), kHidden, kOutPad, bar);
        }
        if (!(ok = group_wait(bar, parity, g))) break;
        {
            float v[16];
            tc::tmem_ld16(tc::tmem_lane_addr(tmem, warp, 0), v);
            const int grow = row0 + gt;
            const float* b4 = bias + 3 * kHidden;
            if (grow < n)
                reinterpret_cast<float4*>(y)[grow] = make_float4(v[0] + b4[0], v[1] + b4[1], v[2] + b4[2], v[3] + b4[3]);
        }
        // the accumulator reads above come before the next tile's first MMA
        tc::fence_before_sync();
        group_sync(g);
        tc::fence_after_sync();
    }
    if (!ok) {
        if (gt == 0) atomicOr(err, kErrMmaTimeout);
        tc::mbar_wait(bar, parity ^ 1u, tc::kWaitLimitNs);  // the chain still in flight, bounded
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem_base, kFwdTmemCols);
}

// ---------------------------------------------------------------------------
// GEMM D = A B^T (K-major bf16 operands), split-K partials
// ---------------------------------------------------------------------------

constexpr int kGemmThreads = 128;
constexpr int kKc = 64;
// two stages of A tile + B tile (N <= 128): 64 KB, so at most 3 CTAs share an
// SM, 384 of its 512 TMEM columns at 128 each
constexpr int kStageBytes = kTile * kKc * 2 + 128 * kKc * 2;
constexpr int kGemmSmem = 2 * kStageBytes;

__global__ void __launch_bounds__(kGemmThreads) k_gemm_tn(const bf16* __restrict__ A, int lda,
                                                          const bf16* __restrict__ B, int ldb, float* __restrict__ D,
                                                          int M, int N, int K, int kper, uint32_t* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    // two stages of (A tile, B tile): chunk c + 1 loads while chunk c's MMAs run
    auto stage_a = [&](int c) { return smem + (c & 1) * kStageBytes; };
    auto stage_b = [&](int c) { return smem + (c & 1) * kStageBytes + kTile * kKc * 2; };
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTile;
    const int kb = blockIdx.y * kper, ke = min(K, kb + kper);
    const uint32_t ncols = N <= 32 ? 32u : N <= 64 ? 64u : 128u;
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, ncols);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(&bar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = tc::idesc_bf16_f32(kTile, N);
    auto load_chunk = [&](int k0, uint8_t* a_s, uint8_t* b_s) {
        for (int q = tid; q < kTile * (kKc / 8); q += kGemmThreads) {
            const int r = q >> 3, k = (q & 7) * 8;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (m0 + r < M && k0 + k < ke) v = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * lda + k0 + k);
            *reinterpret_cast<uint4*>(a_s + tc::kmajor_offset(r, k, kKc)) = v;
        }
        for (int q = tid; q < N * (kKc / 8); q += kGemmThreads) {
            const int r = q >> 3, k = (q & 7) * 8;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (k0 + k < ke) v = *reinterpret_cast<const uint4*>(B + (size_t)r * ldb + k0 + k);
            *reinterpret_cast<uint4*>(b_s + tc::kmajor_offset(r, k, kKc)) = v;
        }
    };
    uint32_t parity = 0;
    bool ok = true;
    const int nchunks = ke > kb ? (ke - kb + kKc - 1) / kKc : 0;
    if (nchunks > 0) load_chunk(kb, stage_a(0), stage_b(0));
    int chunks = 0;
    for (int c = 0; c < nchunks; c++) {
        handoff_to_mma();  // chunk c in shared memory for the tensor core
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t a = tc::smem_addr(stage_a(c)), b = tc::smem_addr(stage_b(c));
            for (int ks = 0; ks < kKc / 16; ks++)
                tc::mma_bf16(tmem, tc::kmajor_desc(a, kKc, ks), tc::kmajor_desc(b, kKc, ks), idesc,
                             (c > 0 || ks > 0) ? 1u : 0u);
            tc::mma_commit(&bar);
        }
        // the other stage was last read by chunk c - 1's MMAs, complete since the last wait
        if (c + 1 < nchunks) load_chunk(kb + (c + 1) * kKc, stage_a(c + 1), stage_b(c + 1));
        if (!(ok = wait_all(&bar, parity))) break;
        chunks++;
    }
    const int r = warp * 32 + lane;
    float* drow = D + ((size_t)blockIdx.y * M + (m0 + r)) * N;
    if (ok) {
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tc::tmem_lane_addr(tmem, warp, c0), v);
            if (m0 + r < M) {
                // four 16-byte stores per 16 columns (N is a multiple of 16, the partials 16-byte aligned)
                float4* d4 = reinterpret_cast<float4*>(drow + c0);
#pragma unroll
                for (int q = 0; q < 4; q++)
                    d4[q] = chunks ? make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3])
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    } else {
        if (tid == 0) atomicOr(err, kErrMmaTimeout);
        tc::mbar_wait(&bar, parity ^ 1u, tc::kWaitLimitNs);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// Fused backward: one persistent CTA per SM, 128-row tiles in turn
// ---------------------------------------------------------------------------
//
// For each tile (rows r of the batch), with dY = the output gradient:
//   dW4^T += H3^T dY          dH3 = dY W4
//   dZ3 = dH3 * SiLU'(Z3)     dW3 += dZ3^T H2   db3 += sum_r dZ3   dH2 = dZ3 W3   (Z saved in FP16)
//   dZ2 = dH2 * SiLU'(Z2)     dW2 += dZ2^T H1   db2 += sum_r dZ2   dH1 = dZ2 W2
//   dZ1 = dH1 * SiLU'(Z1)     dW1 += dZ1^T H0   db1 += sum_r dZ1
// The weight and bias gradients accumulate in TMEM over all tiles of the CTA
// (the bias sums as MMAs against a tile of ones), so nothing but the CTA's
// final partial sums goes to memory; dH of the current layer lives in the
// first 128 columns. Operands in shared memory, K-major without swizzling:
// the weights W4^T, W3^T, W2^T (resident), dY [rows][16] and dY^T [16][rows],
// dZ [rows][128] and dZ^T [128][rows] (written by the epilogues), and the saved
// layer inputs H^T [width][rows], double-buffered and copied with cp.async one
// step ahead of their MMA. The batch is a multiple of 128 rows (no tails). Warp
// w handles rows 32 (w % 4) .. + 31 (its TMEM lane quadrant) and columns
// 64 (w / 4) .. + 63 of every epilogue.
constexpr int kBwdThreads = 256;  // 8 warps: two per TMEM lane quadrant, one per column half
constexpr int kBOffW4t = 0;                                   // [128][16]   kc 16
constexpr int kBOffW3t = kBOffW4t + kHidden * kOutPad * 2;    // [128][128]  kc 128
constexpr int kBOffW2t = kBOffW3t + kHidden * kHidden * 2;    // [128][128]
constexpr int kBOffOnes = kBOffW2t + kHidden * kHidden * 2;   // [16][128]   kc 128, all 1
constexpr int kBOffDy = kBOffOnes + kOutPad * kTile * 2;      // [128][16]   kc 16
constexpr int kBOffDyt = kBOffDy + kTile * kOutPad * 2;       // [16][128]   kc 128
constexpr int kBOffDz = kBOffDyt + kOutPad * kTile * 2;       // [128][128]  kc 128
constexpr int kBOffDzt = kBOffDz + kTile * kHidden * 2;       // [128][128]  kc 128
constexpr int kBOffH = kBOffDzt + kHidden * kTile * 2;        // 2 x [128][128] kc 128
constexpr int kBwdSmem = kBOffH + 2 * kHidden * kTile * 2;
static_assert(kBwdSmem <= 227 * 1024, "shared memory of one CTA");
static_assert(kBwdSmem > 116 * 1024, "one CTA per SM: the TMEM allocation takes every column");
static_assert(kBwdSmem - kBOffDz >= kHidden * (kHidden + 4) * 4, "the partials' staging tile fits the operand buffers");
// TMEM columns
constexpr uint32_t kTcDh = 0, kTcW3 = 128, kTcW2 = 256, kTcW1 = 384, kTcW4 = 448, kTcB3 = 464, kTcB2 = 480,
                   kTcB1 = 496, kBwdTmemCols = 512;

__device__ __forceinline__ void cp_async16(uint8_t* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Copy the tile's columns [row0, row0 + 128) of ht [width][ld] into buf as a
// K-major operand (width rows, K = 128), 16 bytes per cp.async; one group.
__device__ __forceinline__ void issue_h_tile(uint8_t* buf, const bf16* ht, int width, int ld, int row0, int tid) {
    for (int q = tid; q < width * (kTile / 8); q += kBwdThreads) {
        const int f = q >> 4, j = q & 15;
        cp_async16(buf + tc::kmajor_offset(f, 8 * j, kTile), ht + (size_t)f * ld + row0 + 8 * j);
    }
    cp_async_commit();
}

// MMA chain D (+)= A B^T, K = 16 * ksteps, A and B K-major with K extent kc
__device__ __forceinline__ void mma_chain(uint32_t d, uint32_t a, uint32_t b, int kc, int ksteps, int n,
                                          bool accumulate) {
    const uint32_t idesc = tc::idesc_bf16_f32(kTile, n);
    for (int ks = 0; ks < ksteps; ks++)
        tc::mma_bf16(d, tc::kmajor_desc(a, kc, ks), tc::kmajor_desc(b, kc, ks), idesc,
                     (accumulate || ks > 0) ? 1u : 0u);
}

// This thread's row of z (FP16, saved transposed [feature][ldh]) for the 64
// features of its column half: one 2-byte load per feature, a warp reading 64
// contiguous bytes per feature.
__device__ __forceinline__ void load_z_half(const __half* __restrict__ zt, int ldh, int row0, int r, int half,
                                            __half (&zb)[64]) {
    const __half* src = zt + (size_t)(half * 64) * ldh + row0 + r;
#pragma unroll
    for (int f = 0; f < 64; f++) zb[f] = src[(size_t)f * ldh];
}

// Epilogue of a hidden layer: dZ = dH * SiLU'(Z) for this thread's row and column
// half, into the dZ operand (unless null) and the dZ^T operand. zb holds that
// half of the row of z (FP16, loaded by the caller before the MMAs it waited
// for). In dZ^T two lanes (rows 2k, 2k + 1) write one 32-bit word per feature.
__device__ __forceinline__ void bwd_epilogue(uint32_t tmem_dh, int warp, int lane, uint8_t* dz, uint8_t* dzt,
                                             const __half (&zb)[64]) {
    const int r = (warp & 3) * 32 + lane;
    const int half = warp >> 2;
#pragma unroll
    for (int ch = 0; ch < 4; ch++) {
        const int c0 = half * 64 + ch * 16;
        float v[16];
        tc::tmem_ld16(tc::tmem_lane_addr(tmem_dh, warp, c0), v);
        float h[16];
#pragma unroll
        for (int i = 0; i < 16; i++) h[i] = v[i] * silu_grad(__half2float(zb[ch * 16 + i]));
        if (dz) {
            uint4 lo, hi;
            lo.x = pack2(h[0], h[1]); lo.y = pack2(h[2], h[3]); lo.z = pack2(h[4], h[5]); lo.w = pack2(h[6], h[7]);
            hi.x = pack2(h[8], h[9]); hi.y = pack2(h[10], h[11]); hi.z = pack2(h[12], h[13]); hi.w = pack2(h[14], h[15]);
            *reinterpret_cast<uint4*>(dz + tc::kmajor_offset(r, c0, kHidden)) = lo;
            *reinterpret_cast<uint4*>(dz + tc::kmajor_offset(r, c0 + 8, kHidden)) = hi;
        }
        // dZ^T: element (feature, row) at kmajor_offset(feature, row): rows 2k and 2k + 1 are
        // adjacent bf16, so the even lane stores both (its odd neighbour's value by shuffle)
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const float other = __shfl_down_sync(0xffffffffu, h[i], 1);
            if ((lane & 1) == 0)
                *reinterpret_cast<uint32_t*>(dzt + tc::kmajor_offset(c0 + i, r, kTile)) = pack2(h[i], other);
        }
    }
}

// This CTA's partial gradients, in the flat parameter layout: row r of the
// accumulators is TMEM lane r; the two warps of a lane quadrant share the
// columns. The weight blocks go through a shared-memory tile (rows padded by 4
// floats) so that the global stores are contiguous; called by every thread
// once the operand buffers are free (tile: at least 128 x 132 floats).
__device__ __forceinline__ void bwd_store_partials(uint32_t tmem, int warp, int lane, int tid, bool have,
                                                   const float* db4, float* tile, float* __restrict__ out) {
    const int r = (warp & 3) * 32 + lane;
    const int half = warp >> 2;
    auto block = [&](uint32_t col, int ncols, float* dst) {  // dst [128][ncols] = D[.][col .. col + ncols)
        const int ts = ncols + 4;
        for (int c0 = 16 * half; c0 < ncols; c0 += 32) {
            float v[16];
            if (have) tc::tmem_ld16(tc::tmem_lane_addr(tmem + col, warp, c0), v);
#pragma unroll
            for (int q = 0; q < 4; q++)
                *reinterpret_cast<float4*>(tile + r * ts + c0 + 4 * q) =
                    have ? make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3])
                         : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
        const int q4 = ncols / 4;
        for (int q = tid; q < kHidden * q4; q += kBwdThreads) {
            const int rr = q / q4, cc = (q % q4) * 4;
            *reinterpret_cast<float4*>(dst + (size_t)rr * ncols + cc) = *reinterpret_cast<const float4*>(tile + rr * ts + cc);
        }
        __syncthreads();
    };
    block(kTcW3, kHidden, out + kOffParamW3);
    block(kTcW2, kHidden, out + kOffParamW2);
    block(kTcW1, kFeatures, out + kOffParamW1);
    // W4 (D[h][o] = dW4[o][h]) and the biases: one value per row and column, contiguous across lanes
    float v[16];
    if (half == 0) {
        if (have) tc::tmem_ld16(tc::tmem_lane_addr(tmem + kTcW4, warp, 0), v);
#pragma unroll
        for (int o = 0; o < kOutputs; o++) out[kOffParamW4 + o * kHidden + r] = have ? v[o] : 0.f;
        if (have) tc::tmem_ld16(tc::tmem_lane_addr(tmem + kTcB3, warp, 0), v);
        out[kOffParamB3 + r] = have ? v[0] : 0.f;
        if (r < kOutputs) out[kOffParamB4 + r] = db4[r];
    } else {
        if (have) tc::tmem_ld16(tc::tmem_lane_addr(tmem + kTcB2, warp, 0), v);
        out[kOffParamB2 + r] = have ? v[0] : 0.f;
        if (have) tc::tmem_ld16(tc::tmem_lane_addr(tmem + kTcB1, warp, 0), v);
        out[kOffParamB1 + r] = have ? v[0] : 0.f;
    }
}

__global__ void __launch_bounds__(kBwdThreads, 1) k_mlp_backward(const bf16* __restrict__ dy, const Saves S,
                                                                 const bf16* __restrict__ w2t,
                                                                 const bf16* __restrict__ w3t,
                                                                 const bf16* __restrict__ w4t, int batch,
                                                                 float* __restrict__ part, uint32_t* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ float db4s[4][kOutputs];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t* hb[2] = {smem + kBOffH, smem + kBOffH + kHidden * kTile * 2};
    const int ntiles = batch / kTile;
    int t = blockIdx.x;
    if (t < ntiles) {  // the first tile's H3^T and H2^T, in flight while the weights are staged
        issue_h_tile(hb[0], S.h3t, kHidden, S.ldh, t * kTile, tid);
        issue_h_tile(hb[1], S.h2t, kHidden, S.ldh, t * kTile, tid);
    }
    stage_weights(smem + kBOffW4t, w4t, kHidden, kOutPad, tid, kBwdThreads);
    stage_weights(smem + kBOffW3t, w3t, kHidden, kHidden, tid, kBwdThreads);
    stage_weights(smem + kBOffW2t, w2t, kHidden, kHidden, tid, kBwdThreads);
    {
        const bf16 one = __float2bfloat16_rn(1.f);
        for (int q = tid; q < kOutPad * kTile; q += kBwdThreads)
            *reinterpret_cast<bf16*>(smem + kBOffOnes + tc::kmajor_offset(q / kTile, q % kTile, kTile)) = one;
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, kBwdTmemCols);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(&bar, 1);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t a_w4t = tc::smem_addr(smem + kBOffW4t), a_w3t = tc::smem_addr(smem + kBOffW3t);
    const uint32_t a_w2t = tc::smem_addr(smem + kBOffW2t), a_ones = tc::smem_addr(smem + kBOffOnes);
    const uint32_t a_dy = tc::smem_addr(smem + kBOffDy), a_dyt = tc::smem_addr(smem + kBOffDyt);
    const uint32_t a_dz = tc::smem_addr(smem + kBOffDz), a_dzt = tc::smem_addr(smem + kBOffDzt);
    const uint32_t a_h[2] = {tc::smem_addr(hb[0]), tc::smem_addr(hb[1])};
    const int r = (warp & 3) * 32 + lane;
    float db4[kOutputs] = {0.f, 0.f, 0.f, 0.f};
    uint32_t parity = 0;
    bool ok = true;
    int done = 0;  // tiles of this CTA finished (the accumulators hold data once it is > 0)
    for (; t < ntiles && ok; t += gridDim.x) {
        const int row0 = t * kTile;
        const int tn = t + gridDim.x;  // the next tile of this CTA
        const bool acc = done > 0;
        // dY [rows][16] and dY^T [16][rows] from the output gradient (bf16 [batch][16], zero padded)
        if (warp < 4) {
            const uint4* src = reinterpret_cast<const uint4*>(dy + (size_t)(row0 + r) * kOutPad);
            const uint4 lo = src[0], hi = src[1];
            *reinterpret_cast<uint4*>(smem + kBOffDy + tc::kmajor_offset(r, 0, kOutPad)) = lo;
            *reinterpret_cast<uint4*>(smem + kBOffDy + tc::kmajor_offset(r, 8, kOutPad)) = hi;
            const bf16* e = reinterpret_cast<const bf16*>(&lo);
            const bf16* e2 = reinterpret_cast<const bf16*>(&hi);
#pragma unroll
            for (int o = 0; o < 8; o++) {
                *reinterpret_cast<bf16*>(smem + kBOffDyt + tc::kmajor_offset(o, r, kTile)) = e[o];
                *reinterpret_cast<bf16*>(smem + kBOffDyt + tc::kmajor_offset(o + 8, r, kTile)) = e2[o];
            }
#pragma unroll
            for (int o = 0; o < kOutputs; o++) db4[o] += __bfloat162float(e[o]);
        }
        __half zb[64];
        load_z_half(S.z3, S.ldh, row0, r, warp >> 2, zb);  // in flight while the MMAs run
        cp_async_wait<1>();  // H3^T
        handoff_to_mma();
        if (tid == 0) {
            tc::fence_after_sync();
            mma_chain(tmem + kTcW4, a_h[0], a_dyt, kTile, kTile / 16, kOutPad, acc);  // dW4^T += H3^T dY
            mma_chain(tmem + kTcDh, a_dy, a_w4t, kOutPad, 1, kHidden, false);          // dH3 = dY W4
            tc::mma_commit(&bar);
        }
        if (!(ok = wait_all(&bar, parity))) break;
        issue_h_tile(hb[0], S.h1t, kHidden, S.ldh, row0, tid);
        bwd_epilogue(tmem + kTcDh, warp, lane, smem + kBOffDz, smem + kBOffDzt, zb);
        load_z_half(S.z2, S.ldh, row0, r, warp >> 2, zb);
        cp_async_wait<1>();  // H2^T
        handoff_to_mma();
        if (tid == 0) {
            tc::fence_after_sync();
            mma_chain(tmem + kTcW3, a_dzt, a_h[1], kTile, kTile / 16, kHidden, acc);  // dW3 += dZ3^T H2
            mma_chain(tmem + kTcB3, a_dzt, a_ones, kTile, kTile / 16, kOutPad, acc);  // db3 (every column)
            mma_chain(tmem + kTcDh, a_dz, a_w3t, kHidden, kHidden / 16, kHidden, false);  // dH2 = dZ3 W3
            tc::mma_commit(&bar);
        }
        if (!(ok = wait_all(&bar, parity))) break;
        issue_h_tile(hb[1], S.h0t, kInPad, S.ldh, row0, tid);
        bwd_epilogue(tmem + kTcDh, warp, lane, smem + kBOffDz, smem + kBOffDzt, zb);
        load_z_half(S.z1, S.ldh, row0, r, warp >> 2, zb);
        cp_async_wait<1>();  // H1^T
        handoff_to_mma();
        if (tid == 0) {
            tc::fence_after_sync();
            mma_chain(tmem + kTcW2, a_dzt, a_h[0], kTile, kTile / 16, kHidden, acc);  // dW2 += dZ2^T H1
            mma_chain(tmem + kTcB2, a_dzt, a_ones, kTile, kTile / 16, kOutPad, acc);
            mma_chain(tmem + kTcDh, a_dz, a_w2t, kHidden, kHidden / 16, kHidden, false);  // dH1 = dZ2 W2
            tc::mma_commit(&bar);
        }
        if (!(ok = wait_all(&bar, parity))) break;
        if (tn < ntiles) issue_h_tile(hb[0], S.h3t, kHidden, S.ldh, tn * kTile, tid);
        bwd_epilogue(tmem + kTcDh, warp, lane, nullptr, smem + kBOffDzt, zb);
        if (tn < ntiles) cp_async_wait<1>();  // H0^T (the next tile's H3^T may still be in flight)
        else cp_async_wait<0>();
        handoff_to_mma();
        if (tid == 0) {
            tc::fence_after_sync();
            mma_chain(tmem + kTcW1, a_dzt, a_h[1], kTile, kTile / 16, kInPad, acc);  // dW1 += dZ1^T H0
            mma_chain(tmem + kTcB1, a_dzt, a_ones, kTile, kTile / 16, kOutPad, acc);
            tc::mma_commit(&bar);
        }
        if (!(ok = wait_all(&bar, parity))) break;
        if (tn < ntiles) issue_h_tile(hb[1], S.h2t, kHidden, S.ldh, tn * kTile, tid);
        done++;
    }
    cp_async_wait<0>();
    if (!ok) {
        if (tid == 0) atomicOr(err, kErrMmaTimeout);
        tc::mbar_wait(&bar, parity ^ 1u, tc::kWaitLimitNs);  // the chain still in flight, bounded
    }
    // db4: the sum over this CTA's rows (warps 0-3), in a fixed order
#pragma unroll
    for (int o = 0; o < kOutputs; o++) {
        float v = db4[o];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
        if (lane == 0 && warp < 4) db4s[warp][o] = v;
    }
    __syncthreads();
    float db4t[kOutputs];
#pragma unroll
    for (int o = 0; o < kOutputs; o++) db4t[o] = db4s[0][o] + db4s[1][o] + db4s[2][o] + db4s[3][o];
    bwd_store_partials(tmem, warp, lane, tid, ok && done > 0, db4t, reinterpret_cast<float*>(smem + kBOffDz),
                       part + (size_t)blockIdx.x * kParams);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem_base, kBwdTmemCols);
}

// grads[p] = the sum over the CTAs' partials: 64 parameters per block, four
// threads per parameter summing every fourth CTA's partial (a warp reads 32
// consecutive parameters of one partial), the four sums added in a fixed order;
// with an Adam step (adam.lr > 0) the parameter is updated in the same pass.
// Parameter p (flat layout) into its bf16 operand positions, as k_pack writes them.
__device__ __forceinline__ void pack_param(const PackedMut& W, int p, float val) {
    const bf16 b = __float2bfloat16_rn(val);
    if (p < kOffParamB1) {  // W1 [128][48] -> w1 [128][64]
        W.w1[(p / kFeatures) * kInPad + p % kFeatures] = b;
    } else if (p < kOffParamW2) {
        W.bias[p - kOffParamB1] = val;
    } else if (p < kOffParamB2) {  // W2 [128][128], and transposed
        const int i = p - kOffParamW2;
        W.w2[i] = b;
        W.w2t[(i % kHidden) * kHidden + i / kHidden] = b;
    } else if (p < kOffParamW3) {
        W.bias[kHidden + p - kOffParamB2] = val;
    } else if (p < kOffParamB3) {
        const int i = p - kOffParamW3;
        W.w3[i] = b;
        W.w3t[(i % kHidden) * kHidden + i / kHidden] = b;
    } else if (p < kOffParamW4) {
        W.bias[2 * kHidden + p - kOffParamB3] = val;
    } else if (p < kOffParamB4) {  // W4 [4][128] -> w4 [16][128], w4t [128][16]
        const int i = p - kOffParamW4;
        W.w4[i] = b;
        W.w4t[(i % kHidden) * kOutPad + i / kHidden] = b;
    } else {
        W.bias[3 * kHidden + p - kOffParamB4] = val;
    }
}

constexpr int kSumParams = 64;
__global__ void __launch_bounds__(4 * kSumParams) k_sum_partials(const float* __restrict__ part, int nparts,
                                                                 float* __restrict__ grads, const AdamStep adam) {
    __shared__ float sh[4][kSumParams];
    const int j = threadIdx.x / kSumParams, q = threadIdx.x % kSumParams;
    const int p = blockIdx.x * kSumParams + q;
    float s = 0.f;
    if (p < kParams)
        for (int k = j; k < nparts; k += 4) s += part[(size_t)k * kParams + p];
    sh[j][q] = s;
    __syncthreads();
    if (j != 0 || p >= kParams) return;
    const float g = (sh[0][q] + sh[1][q]) + (sh[2][q] + sh[3][q]);
    grads[p] = g;
    if (adam.lr > 0.f) {
        const float mi = adam.b1 * adam.m[p] + (1.f - adam.b1) * g;
        const float vi = adam.b2 * adam.v[p] + (1.f - adam.b2) * g * g;
        adam.m[p] = mi;
        adam.v[p] = vi;
        const float np = adam.p[p] - adam.lr * (mi / adam.c1) / (sqrtf(vi / adam.c2) + adam.eps);
        adam.p[p] = np;
        pack_param(adam.w, p, np);
    }
}

// ---------------------------------------------------------------------------
// Backward and optimiser helpers
// ---------------------------------------------------------------------------

// dY = 2 (y - t) / batch (the gradient of the mean over the batch of the
// squared output error), bf16, row-major [batch][16] and transposed [16][ld];
// per-block partial sums of the squared error.
__global__ void k_out_grad(const float4* __restrict__ y, const float4* __restrict__ t, int batch, int ld,
                           bf16* __restrict__ dy, bf16* __restrict__ dyt, float* __restrict__ loss_part) {
    __shared__ float red[256 / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float se = 0.f;
    if (i < batch) {
        const float4 a = y[i], b = t[i];
        const float d[4] = {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w};
        const float s = 2.f / (float)batch;
        uint4 lo, hi = make_uint4(0u, 0u, 0u, 0u);
        lo.x = pack2(s * d[0], s * d[1]);
        lo.y = pack2(s * d[2], s * d[3]);
        lo.z = 0u;
        lo.w = 0u;
        reinterpret_cast<uint4*>(dy + (size_t)i * kOutPad)[0] = lo;
        reinterpret_cast<uint4*>(dy + (size_t)i * kOutPad)[1] = hi;
#pragma unroll
        for (int o = 0; o < 4; o++) {
            if (dyt) dyt[(size_t)o * ld + i] = __float2bfloat16_rn(s * d[o]);
            se += d[o] * d[o];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) se += __shfl_xor_sync(0xffffffffu, se, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = se;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
        loss_part[blockIdx.x] = s;
    }
}

// loss = sum of the partials / batch (one block, fixed order)
__global__ void k_loss_sum(const float* __restrict__ part, int nparts, int batch, float* __restrict__ loss) {
    __shared__ float red[256];
    float s = 0.f;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = red[0] / (float)batch;
}


// FP32 master parameters -> padded bf16 operands (and their transposes) + biases
__global__ void k_pack(const float* __restrict__ p, PackedMut W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float* w1 = p + kOffParamW1;
    const float* w2 = p + kOffParamW2;
    const float* w3 = p + kOffParamW3;
    const float* w4 = p + kOffParamW4;
    if (i < kHidden * kInPad) {  // w1 [128][64]
        const int o = i / kInPad, k = i % kInPad;
        W.w1[i] = __float2bfloat16_rn(k < kFeatures ? w1[o * kFeatures + k] : 0.f);
    }
    if (i < kHidden * kHidden) {  // w2, w3 and their transposes
        const int o = i / kHidden, k = i % kHidden;
        W.w2[i] = __float2bfloat16_rn(w2[i]);
        W.w3[i] = __float2bfloat16_rn(w3[i]);
        W.w2t[k * kHidden + o] = __float2bfloat16_rn(w2[i]);
        W.w3t[k * kHidden + o] = __float2bfloat16_rn(w3[i]);
    }
    if (i < kOutPad * kHidden) {  // w4 [16][128], w4t [128][16]
        const int o = i / kHidden, k = i % kHidden;
        const float v = o < kOutputs ? w4[o * kHidden + k] : 0.f;
        W.w4[i] = __float2bfloat16_rn(v);
        W.w4t[k * kOutPad + o] = __float2bfloat16_rn(v);
    }
    if (i < 3 * kHidden + kOutPad) {
        float b;
        if (i < kHidden) b = p[kOffParamB1 + i];
        else if (i < 2 * kHidden) b = p[kOffParamB2 + i - kHidden];
        else if (i < 3 * kHidden) b = p[kOffParamB3 + i - 2 * kHidden];
        else b = (i - 3 * kHidden) < kOutputs ? p[kOffParamB4 + i - 3 * kHidden] : 0.f;
        W.bias[i] = b;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

cudaError_t launch_forward(const float* x, int n, const Packed& W, const Saves& S, float* y, uint32_t* err,
                           int num_sms, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    // per call (a host-side attribute of the current device): threads and devices stay independent
    cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem);
    if (e != cudaSuccess) return e;
    const int tiles = (n + kTile - 1) / kTile;
    const int pairs = (tiles + kGroups - 1) / kGroups;
    const int grid = pairs < num_sms ? pairs : num_sms;
    k_mlp_forward<<<grid, kFwdThreads, kFwdSmem, s>>>(x, n, W, S, y, err);
    return cudaGetLastError();
}

cudaError_t launch_gemm_tn(const bf16* A, int lda, const bf16* B, int ldb, float* D, int M, int N, int K,
                           int splits, uint32_t* err, cudaStream_t s) {
    if (M <= 0 || N <= 0 || N > 128 || (N % 16) != 0 || K < 0 || (K % 8) != 0 || splits < 1 || (lda % 8) != 0 ||
        (ldb % 8) != 0)
        return cudaErrorInvalidValue;
    int kper = (K + splits - 1) / splits;
    kper = (kper + kKc - 1) / kKc * kKc;
    if (kper == 0) kper = kKc;
    cudaError_t e = cudaFuncSetAttribute(k_gemm_tn, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    if (e != cudaSuccess) return e;
    dim3 grid((M + kTile - 1) / kTile, splits);
    k_gemm_tn<<<grid, kGemmThreads, kGemmSmem, s>>>(A, lda, B, ldb, D, M, N, K, kper, err);
    return cudaGetLastError();
}

cudaError_t launch_out_grad(const float* y, const float* t, int batch, int ld, bf16* dy, bf16* dyt, float* loss_part,
                            float* loss, cudaStream_t s) {
    const int blocks = (batch + 255) / 256;
    k_out_grad<<<blocks, 256, 0, s>>>(reinterpret_cast<const float4*>(y), reinterpret_cast<const float4*>(t), batch,
                                      ld, dy, dyt, loss_part);
    if (loss) k_loss_sum<<<1, 256, 0, s>>>(loss_part, blocks, batch, loss);
    return cudaGetLastError();
}

cudaError_t launch_backward(const bf16* dy, const Saves& S, const PackedMut& W, int batch, float* part,
                            float* grads, const AdamStep& adam, uint32_t* err, int num_sms, cudaStream_t s) {
    // the saved inputs are copied 16 bytes at a time: their row stride must keep that alignment
    if (batch <= 0 || batch % kTile != 0 || !S.z1 || !S.h0t || S.ldh % 8 != 0 || S.ldh < batch)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, kBwdSmem);
    if (e != cudaSuccess) return e;
    const int tiles = batch / kTile;
    const int grid = tiles < num_sms ? tiles : num_sms;
    k_mlp_backward<<<grid, kBwdThreads, kBwdSmem, s>>>(dy, S, W.w2t, W.w3t, W.w4t, batch, part, err);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_sum_partials<<<(kParams + kSumParams - 1) / kSumParams, 4 * kSumParams, 0, s>>>(part, grid, grads, adam);
    return cudaGetLastError();
}

AdamStep adam_step(float* p, float* m, float* v, float lr, float b1, float b2, float eps, int step,
                   const PackedMut& w) {
    return AdamStep{p, m, v, lr, b1, b2, eps, 1.f - powf(b1, (float)step), 1.f - powf(b2, (float)step), w};
}

cudaError_t launch_pack(const float* p, const PackedMut& W, cudaStream_t s) {
    k_pack<<<(kHidden * kHidden + 255) / 256, 256, 0, s>>>(p, W);
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace sphmp
