// sphmp_learned.cu — the learned large-step corrector: the correction kernel,
// the state comparison of the audit, and the network object (sphmp_corrector:
// parameters, Adam state, training buffers) with its C ABI
// (include/sphmp_learned.h). The network kernels are in sphmp_mlp.cu; the
// features are filled by the force pass of a corrected step (sphmp_features.cuh).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "sphmp.h"
#include "sphmp_device.cuh"
#include "sphmp_internal.h"

#include "sphmp_learned.h"
#include "sphmp_mlp.h"

using namespace sphmp;
using bf16 = __nv_bfloat16;

// ---------------------------------------------------------------------------
// Features and correction (one thread per particle of the internal order)
// ---------------------------------------------------------------------------

namespace sphmp {
namespace {

constexpr float kOutClamp = 4.f;

// Apply the network's outputs (times out_scale) to the step's result: outputs
// 0-2 are a displacement rate c (m/s), the position moves by c * dt_large (the
// large step's error is in its positions: a step of 8 dt overshoots 8 steps of
// dt by 28 a dt^2 while its velocity agrees to second order); output 3 scales
// the stored density of the result by 1 + output.
__global__ void __launch_bounds__(256) k_apply_correction(const __grid_constant__ DevParams P,
                                                          const __grid_constant__ DevBuffers B, float4* pos4,
                                                          const float4* __restrict__ y,
                                                          const float* __restrict__ out_scale,
                                                          const int32_t* __restrict__ ids, float dt_over_ss,
                                                          float4* __restrict__ corr) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= active_n(B)) return;
    if (ids[s] < 0) {
        corr[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    // outputs beyond kOutClamp standard deviations of the training targets are
    // extrapolation: clamped
    const float4 o = y[s];
    const float ox = fminf(fmaxf(o.x, -kOutClamp), kOutClamp), oy = fminf(fmaxf(o.y, -kOutClamp), kOutClamp);
    const float oz = fminf(fmaxf(o.z, -kOutClamp), kOutClamp), ow = fminf(fmaxf(o.w, -kOutClamp), kOutClamp);
    const float cx = ox * out_scale[0], cy = oy * out_scale[1], cz = oz * out_scale[2];
    const float cd = fmaxf(ow * out_scale[3], -0.5f);
    float4 p = pos4[s];
    p.x += cx * dt_over_ss; p.y += cy * dt_over_ss; p.z += cz * dt_over_ss;
    pos4[s] = p;
    float2 d = B.densp[s];
    d.x = d.x / (1.f + cd);
    B.densp[s] = d;
    corr[s] = make_float4(cx, cy, cz, cd);
}

// bornid -> internal index of the in-grid fluid particles of one state
__global__ void k_id_map(const __grid_constant__ DevBuffers B, const float4* __restrict__ pos4,
                         const float4* __restrict__ aprev4, int map_size, int32_t* __restrict__ map) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= active_n(B)) return;
    if (!(pos4[s].w > 0.f) || B.mgcell[s] == kUndef) return;
    const int32_t id = B.bornid[__float_as_uint(aprev4[s].w)];
    if (id >= 0 && id < map_size) map[id] = s;
}

// Differences of state b against state a over the particles in-grid fluid in
// both (matched by bornid): sums of (rho_b / rho_a - 1)^2, sum_k (alpha_b -
// alpha_a)^2, |v_b - v_a|^2, |v_a|^2, the count, |x_b - x_a|^2 (metres), and
// max |rho_b / rho_a - 1|.
constexpr int kCmpSums = 6;
__global__ void __launch_bounds__(256) k_compare(const __grid_constant__ DevParams Pb,
                                                 const __grid_constant__ DevBuffers Bb, const float4* __restrict__ pos_b,
                                                 const float4* __restrict__ vel_b, const float4* __restrict__ alpha_b,
                                                 const float4* __restrict__ aprev_b, const float2* __restrict__ dens_a,
                                                 const float4* __restrict__ pos_a, const float4* __restrict__ vel_a,
                                                 const float4* __restrict__ alpha_a, const int32_t* __restrict__ map,
                                                 int map_size, double* __restrict__ out) {
    __shared__ double sh[kCmpSums + 1][8];
    double acc[kCmpSums + 1] = {0, 0, 0, 0, 0, 0, 0};
    const int n = active_n(Bb);
    const double ss = Pb.ss;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const float4 pb = pos_b[s];
        if (!(pb.w > 0.f) || Bb.mgcell[s] == kUndef) continue;
        const int32_t id = Bb.bornid[__float_as_uint(aprev_b[s].w)];
        if (id < 0 || id >= map_size) continue;
        const int32_t j = map[id];
        if (j < 0) continue;
        const double rel = (double)dens_a[j].x / (double)Bb.densp[s].x - 1.0;  // stored inverses
        const float4 ab = alpha_b[s], aa = alpha_a[j];
        double da = (double)(ab.x - aa.x) * (ab.x - aa.x);
        if (Pb.nphase > 1) da += (double)(ab.y - aa.y) * (ab.y - aa.y);
        if (Pb.nphase > 2) da += (double)(ab.z - aa.z) * (ab.z - aa.z);
        const float4 vb = vel_b[s], va = vel_a[j], pa = pos_a[j];
        const double dx = ((double)pb.x - pa.x) * ss, dy = ((double)pb.y - pa.y) * ss, dz = ((double)pb.z - pa.z) * ss;
        acc[0] += rel * rel;
        acc[1] += da;
        acc[2] += (double)(vb.x - va.x) * (vb.x - va.x) + (double)(vb.y - va.y) * (vb.y - va.y) +
                  (double)(vb.z - va.z) * (vb.z - va.z);
        acc[3] += (double)va.x * va.x + (double)va.y * va.y + (double)va.z * va.z;
        acc[4] += 1.0;
        acc[5] += dx * dx + dy * dy + dz * dz;
        acc[6] = fmax(acc[6], fabs(rel));
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q <= kCmpSums; q++) {
        double v = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double u = __shfl_xor_sync(0xffffffffu, v, o);
            v = q == kCmpSums ? fmax(v, u) : v + u;
        }
        if (lane == 0) sh[q][w] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < kCmpSums; q++) {
            double t = 0.0;
            for (int k = 0; k < 8; k++) t += sh[q][k];
            atomicAdd(&out[q], t);
        }
        double m = 0.0;
        for (int k = 0; k < 8; k++) m = fmax(m, sh[kCmpSums][k]);
        atomicMax(reinterpret_cast<unsigned long long*>(&out[kCmpSums]), (unsigned long long)__double_as_longlong(m));
    }
}

}  // namespace

void launch_compare(const DevParams& Pa, const DevBuffers& Ba, const int* cur_a, const DevParams& Pb,
                    const DevBuffers& Bb, const int* cur_b, int32_t* map, int map_size, double* out, cudaStream_t s) {
    cudaMemsetAsync(map, 0xFF, sizeof(int32_t) * (size_t)map_size, s);
    cudaMemsetAsync(out, 0, sizeof(double) * (kCmpSums + 1), s);
    if (Pa.n > 0)
        k_id_map<<<(Pa.n + 255) / 256, 256, 0, s>>>(Ba, Ba.f4[POS][cur_a[POS]], Ba.f4[APREV][cur_a[APREV]], map_size,
                                                    map);
    if (Pb.n > 0)
        k_compare<<<2 * 152, 256, 0, s>>>(Pb, Bb, Bb.f4[POS][cur_b[POS]], Bb.f4[VEL][cur_b[VEL]],
                                          Bb.f4[ALPHA][cur_b[ALPHA]], Bb.f4[APREV][cur_b[APREV]], Ba.densp,
                                          Ba.f4[POS][cur_a[POS]], Ba.f4[VEL][cur_a[VEL]], Ba.f4[ALPHA][cur_a[ALPHA]],
                                          map, map_size, out);
}

void launch_apply_correction(const DevParams& P, const DevBuffers& B, const int* cur, const float* y,
                             const float* out_scale, const int32_t* ids, float dt_large, float* corr,
                             cudaStream_t s) {
    if (P.n <= 0) return;
    k_apply_correction<<<(P.n + 255) / 256, 256, 0, s>>>(P, B, B.f4[POS][cur[POS]], reinterpret_cast<const float4*>(y),
                                                         out_scale, ids, dt_large / P.ss,
                                                         reinterpret_cast<float4*>(corr));
}

}  // namespace sphmp

// ---------------------------------------------------------------------------
// The network object
// ---------------------------------------------------------------------------

struct sphmp_corrector {
    int max_batch = 0;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    int adam_step = 0;
    // parameters
    float* params = nullptr;  // [kParams] FP32 master
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    bf16 *w1 = nullptr, *w2 = nullptr, *w3 = nullptr, *w4 = nullptr, *w2t = nullptr, *w3t = nullptr, *w4t = nullptr;
    float* bias = nullptr;      // [3 * 128 + 16]
    float* norm = nullptr;      // fshift [48], fscale [48], out_scale [4]
    uint32_t* err = nullptr;
    // training buffers (max_batch rows): the hidden layers' z (FP16), outputs,
    // the layer inputs transposed, the output gradient
    __half *z1 = nullptr, *z2 = nullptr, *z3 = nullptr;
    float* y = nullptr;
    bf16 *h0t = nullptr, *h1t = nullptr, *h2t = nullptr, *h3t = nullptr;
    bf16* dy = nullptr;
    float* bpart = nullptr;     // the fused backward's per-CTA gradient partials [num_sms][kParams]
    float* loss_part = nullptr;
    float* loss = nullptr;
    std::vector<void*> allocs;
};

namespace {

thread_local char g_lerr[256];

sphmp_status lfail(sphmp_status st, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_lerr, sizeof(g_lerr), fmt, ap);
    va_end(ap);
    return record_error(st, g_lerr);
}

#define LCK(call)                                                                      \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) return lfail(SPHMP_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

template <class T>
sphmp_status lalloc(sphmp_corrector* c, T** p, size_t count) {
    void* q = nullptr;
    LCK(cudaMalloc(&q, sizeof(T) * (count ? count : 1)));
    LCK(cudaMemset(q, 0, sizeof(T) * (count ? count : 1)));
    c->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return SPHMP_OK;
}

mlp::Packed packed(const sphmp_corrector* c) {
    return mlp::Packed{c->w1, c->w2, c->w3, c->w4, c->bias, c->norm, c->norm + mlp::kFeatures};
}

mlp::PackedMut packed_mut(const sphmp_corrector* c) {
    return mlp::PackedMut{c->w1, c->w2, c->w3, c->w4, c->w2t, c->w3t, c->w4t, c->bias};
}

sphmp_status take_errors(sphmp_corrector* c) {
    uint32_t bits = 0;
    LCK(cudaMemcpyAsync(&bits, c->err, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
    LCK(cudaMemsetAsync(c->err, 0, sizeof(bits), c->stream));
    LCK(cudaStreamSynchronize(c->stream));
    if (bits & mlp::kErrMmaTimeout) return lfail(SPHMP_ERR_TIMEOUT, "a tensor-core wait ran out");
    return SPHMP_OK;
}

// forward with saves, output gradient, backward into c->grads
sphmp_status enqueue_backward(sphmp_corrector* c, const float* x, const float* t, int batch,
                              const mlp::AdamStep& adam, bool want_loss) {
    using namespace mlp;
    const cudaStream_t s = c->stream;
    const int ld = c->max_batch;
    const Saves S{c->z1, c->z2, c->z3, c->h0t, c->h1t, c->h2t, c->h3t, ld};
    LCK(launch_forward(x, batch, packed(c), S, c->y, c->err, c->num_sms, s));
    LCK(launch_out_grad(c->y, t, batch, ld, c->dy, nullptr, c->loss_part, want_loss ? c->loss : nullptr, s));
    LCK(launch_backward(c->dy, S, packed_mut(c), batch, c->bpart, c->grads, adam, c->err, c->num_sms, s));
    return SPHMP_OK;
}

sphmp_status check_batch(const sphmp_corrector* c, const float* x, const float* t, int batch) {
    if (!x || !t) return lfail(SPHMP_ERR_INVALID_ARG, "x and t must be device pointers");
    if (batch <= 0 || batch % 128 != 0 || batch > c->max_batch)
        return lfail(SPHMP_ERR_INVALID_ARG, "batch %d must be a positive multiple of 128 up to %d", batch, c->max_batch);
    return SPHMP_OK;
}

}  // namespace

// internal: used by the context's large step (sphmp_api.cu)
namespace sphmp {
cudaError_t corrector_forward_on(sphmp_corrector* c, const float* x, int n, float* y, uint32_t* err,
                                 cudaStream_t s) {
    return mlp::launch_forward(x, n, packed(c), mlp::Saves{}, y, err, c->num_sms, s);
}
const float* corrector_out_scale(const sphmp_corrector* c) { return c->norm + 2 * mlp::kFeatures; }
int corrector_device(const sphmp_corrector* c) { return c->device; }
}  // namespace sphmp

extern "C" {

sphmp_status sphmp_corrector_create(int32_t max_batch, void* stream, sphmp_corrector** out) {
    using namespace mlp;
    if (!out) return lfail(SPHMP_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (max_batch < 0 || max_batch % 128 != 0)
        return lfail(SPHMP_ERR_INVALID_ARG, "max_batch %d must be a non-negative multiple of 128", max_batch);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return lfail(SPHMP_ERR_NO_DEVICE, "no CUDA device available");
    }
    sphmp_corrector* c = new sphmp_corrector();
    c->max_batch = max_batch;
    c->stream = static_cast<cudaStream_t>(stream);
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    sphmp_status st = SPHMP_OK;
    auto A = [&](auto** p, size_t n) {
        if (st == SPHMP_OK) st = lalloc(c, p, n);
    };
    A(&c->params, kParams); A(&c->grads, kParams); A(&c->adam_m, kParams); A(&c->adam_v, kParams);
    A(&c->w1, kHidden * kInPad); A(&c->w2, kHidden * kHidden); A(&c->w3, kHidden * kHidden);
    A(&c->w4, kOutPad * kHidden); A(&c->w2t, kHidden * kHidden); A(&c->w3t, kHidden * kHidden);
    A(&c->w4t, kHidden * kOutPad); A(&c->bias, 3 * kHidden + kOutPad); A(&c->norm, 2 * kFeatures + kOutputs);
    A(&c->err, 1);
    const size_t B = (size_t)max_batch;
    if (B > 0) {
        A(&c->z1, kHidden * B); A(&c->z2, kHidden * B); A(&c->z3, kHidden * B);  // [128][max_batch]
        A(&c->y, B * 4);
        A(&c->h0t, (size_t)kInPad * B); A(&c->h1t, kHidden * B); A(&c->h2t, kHidden * B); A(&c->h3t, kHidden * B);
        A(&c->dy, B * kOutPad);
        A(&c->bpart, (size_t)c->num_sms * kParams);
        A(&c->loss_part, B / 256 + 1);
        A(&c->loss, 1);
    }
    if (st == SPHMP_OK && cudaDeviceSynchronize() != cudaSuccess)  // the zero fills (legacy default stream)
        st = lfail(SPHMP_ERR_CUDA, "zero fill of the corrector's buffers failed");
    if (st != SPHMP_OK) {
        sphmp_corrector_destroy(c);
        return st;
    }
    // identity normalisation
    std::vector<float> norm(2 * kFeatures + kOutputs, 1.f);
    for (int i = 0; i < kFeatures; i++) norm[i] = 0.f;
    if (cudaMemcpy(c->norm, norm.data(), sizeof(float) * norm.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        sphmp_corrector_destroy(c);
        return lfail(SPHMP_ERR_CUDA, "normalisation upload failed");
    }
    *out = c;
    return SPHMP_OK;
}

void sphmp_corrector_destroy(sphmp_corrector* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : c->allocs) cudaFree(p);
    delete c;
}

sphmp_status sphmp_corrector_set_params(sphmp_corrector* c, const float* params) {
    if (!c || !params) return lfail(SPHMP_ERR_INVALID_ARG, "bad arguments");
    for (int i = 0; i < mlp::kParams; i++)
        if (!isfinite(params[i])) return lfail(SPHMP_ERR_NOT_FINITE, "parameter %d is not finite", i);
    LCK(cudaMemcpyAsync(c->params, params, sizeof(float) * mlp::kParams, cudaMemcpyHostToDevice, c->stream));
    LCK(cudaMemsetAsync(c->adam_m, 0, sizeof(float) * mlp::kParams, c->stream));
    LCK(cudaMemsetAsync(c->adam_v, 0, sizeof(float) * mlp::kParams, c->stream));
    c->adam_step = 0;
    LCK(mlp::launch_pack(c->params, packed_mut(c), c->stream));
    LCK(cudaStreamSynchronize(c->stream));
    return SPHMP_OK;
}

sphmp_status sphmp_corrector_get_params(sphmp_corrector* c, float* params) {
    if (!c || !params) return lfail(SPHMP_ERR_INVALID_ARG, "bad arguments");
    LCK(cudaMemcpyAsync(params, c->params, sizeof(float) * mlp::kParams, cudaMemcpyDeviceToHost, c->stream));
    LCK(cudaStreamSynchronize(c->stream));
    return SPHMP_OK;
}

sphmp_status sphmp_corrector_set_normalisation(sphmp_corrector* c, const float* feat_shift, const float* feat_scale,
                                               const float* out_scale) {
    using namespace mlp;
    if (!c || !feat_shift || !feat_scale || !out_scale) return lfail(SPHMP_ERR_INVALID_ARG, "bad arguments");
    std::vector<float> norm(2 * kFeatures + kOutputs);
    for (int i = 0; i < kFeatures; i++) {
        norm[i] = feat_shift[i];
        norm[kFeatures + i] = feat_scale[i];
    }
    for (int i = 0; i < kOutputs; i++) norm[2 * kFeatures + i] = out_scale[i];
    for (float v : norm)
        if (!isfinite(v)) return lfail(SPHMP_ERR_NOT_FINITE, "normalisation not finite");
    LCK(cudaMemcpyAsync(c->norm, norm.data(), sizeof(float) * norm.size(), cudaMemcpyHostToDevice, c->stream));
    LCK(cudaStreamSynchronize(c->stream));
    return SPHMP_OK;
}

sphmp_status sphmp_corrector_forward(sphmp_corrector* c, const float* x, int32_t n, float* y) {
    if (!c || !x || !y || n < 0) return lfail(SPHMP_ERR_INVALID_ARG, "bad arguments");
    LCK(mlp::launch_forward(x, n, packed(c), mlp::Saves{}, y, c->err, c->num_sms, c->stream));
    return SPHMP_OK;
}

sphmp_status sphmp_corrector_gradients(sphmp_corrector* c, const float* x, const float* t, int32_t batch,
                                       float* grads, float* loss) {
    if (!c || !grads) return lfail(SPHMP_ERR_INVALID_ARG, "bad arguments");
    if (sphmp_status st = check_batch(c, x, t, batch)) return st;
    if (sphmp_status st = enqueue_backward(c, x, t, batch, mlp::AdamStep{}, loss != nullptr)) return st;
    LCK(cudaMemcpyAsync(grads, c->grads, sizeof(float) * mlp::kParams, cudaMemcpyDeviceToHost, c->stream));
    if (loss) LCK(cudaMemcpyAsync(loss, c->loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    return take_errors(c);
}

sphmp_status sphmp_corrector_train_step(sphmp_corrector* c, const float* x, const float* t, int32_t batch, float lr,
                                        float* loss) {
    if (!c) return lfail(SPHMP_ERR_INVALID_ARG, "corrector is NULL");
    if (sphmp_status st = check_batch(c, x, t, batch)) return st;
    if (!(lr > 0.f) || !isfinite(lr)) return lfail(SPHMP_ERR_INVALID_ARG, "lr must be > 0");
    c->adam_step++;
    const mlp::AdamStep adam =
        mlp::adam_step(c->params, c->adam_m, c->adam_v, lr, 0.9f, 0.999f, 1e-8f, c->adam_step, packed_mut(c));
    if (sphmp_status st = enqueue_backward(c, x, t, batch, adam, loss != nullptr)) {  // also repacks the operands
        c->adam_step--;
        return st;
    }
    if (loss) {
        LCK(cudaMemcpyAsync(loss, c->loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
        return take_errors(c);
    }
    return SPHMP_OK;
}

sphmp_status sphmp_corrector_sync(sphmp_corrector* c) {
    if (!c) return lfail(SPHMP_ERR_INVALID_ARG, "corrector is NULL");
    return take_errors(c);
}

sphmp_status sphmp_gemm_bf16_tn(const void* a, int32_t lda, const void* b, int32_t ldb, float* d, int32_t m,
                                int32_t n, int32_t k, int32_t splits, void* stream) {
    if (!a || !b || !d) return lfail(SPHMP_ERR_INVALID_ARG, "null operand");
    if (m <= 0 || n <= 0 || n > 128 || n % 16 != 0 || k < 0 || k % 8 != 0 || splits < 1 || lda % 8 != 0 ||
        ldb % 8 != 0 || lda < k || ldb < k)
        return lfail(SPHMP_ERR_INVALID_ARG, "unsupported GEMM shape m %d n %d k %d lda %d ldb %d splits %d", m, n, k,
                     lda, ldb, splits);
    uint32_t* err = nullptr;
    LCK(cudaMalloc(&err, sizeof(uint32_t)));
    LCK(cudaMemset(err, 0, sizeof(uint32_t)));
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = mlp::launch_gemm_tn(static_cast<const bf16*>(a), lda, static_cast<const bf16*>(b), ldb, d, m, n, k,
                                        splits, err, s);
    uint32_t bits = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, err, sizeof(bits), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(err);
    if (e != cudaSuccess) return lfail(SPHMP_ERR_CUDA, "gemm: %s", cudaGetErrorString(e));
    if (bits & mlp::kErrMmaTimeout) return lfail(SPHMP_ERR_TIMEOUT, "a tensor-core wait ran out");
    return SPHMP_OK;
}

}  // extern "C"
