// sphmp_features.cuh — the learned corrector's per-particle features, as an
// accumulator over the neighbours the force pass visits (the force pass of a
// corrected large step also fills the features, so that the neighbours are
// gathered once).
//
// Features of an in-grid fluid particle, from the state after the density pass
// of a step (pos, vel, 1/rho and p, fractions and rest density, g - a of the
// last advance) over its neighbours closer than h. With w = (1 - r^2/h^2)^3,
// g = (1 - r/h)^2, x_ij = x_i - x_j (metres), u = unit x_ij, vs = sqrt(|g| h):
//   0-2  v_i / vs                     3   rho_i / rho0_i - 1
//   4    p_i / (rho0_i vs^2)          5-7 alpha_i
//   8-10 (g - a)_i dt_large / vs      11  sum_fluid w
//   12-14 sum_fluid w x_ij / h        15-17 sum_fluid w (v_j - v_i) / vs
//   18   sum_fluid w (rho_j/rho0_j - rho_i/rho0_i)
//   19   sum_fluid w (p_j - p_i) / (rho0_i vs^2)
//   20-22 sum_fluid w (alpha_j - alpha_i)
//   23-28 sum_fluid w x x^T / h^2 (xx, yy, zz, xy, xz, yz)
//   29-31 sum_fluid g u               32  sum_fluid g (v_j - v_i).u / vs
//   33-35 sum_fluid g ((v_j - v_i) x u) / vs
//   36-38 sum_fluid g (p_i + p_j) u / (rho0_i vs^2)
//   39   fluid neighbours / 32        40  sum_boundary w
//   41-43 sum_boundary w x_ij / h     44  boundary neighbours / 32
//   45-47 sum_fluid g (alpha_j0 - alpha_i0) u
#pragma once

#include "sphmp_internal.h"

namespace sphmp {
namespace dev {

constexpr int kLearnedFeatures = 48;

struct LearnedFeatures {
    float f[kLearnedFeatures];
    float4 pi, vi, ai;
    float pres_i, reli, ivs, ips, ih, ih2, ir2;

    // own features; pi, vi, ai, di, gi: this particle's pos4, vel4, alpha4,
    // (1/rho, p), aprev4
    __device__ __forceinline__ void init(const DevParams& P, float4 pi_, float4 vi_, float4 ai_, float2 di, float4 gi,
                                         float vs, float dt_large) {
        pi = pi_;
        vi = vi_;
        ai = ai_;
        pres_i = di.y;
        const float rhoi = 1.f / di.x;
        reli = rhoi / ai.w;
        ivs = 1.f / vs;
        ips = 1.f / (ai.w * vs * vs);
        ih = 1.f / P.h;
        ih2 = ih * ih;
        ir2 = 1.f / P.r2;
#pragma unroll
        for (int k = 0; k < kLearnedFeatures; k++) f[k] = 0.f;
        f[0] = vi.x * ivs; f[1] = vi.y * ivs; f[2] = vi.z * ivs;
        f[3] = reli - 1.f;
        f[4] = di.y * ips;
        f[5] = ai.x; f[6] = P.nphase > 1 ? ai.y : 0.f; f[7] = P.nphase > 2 ? ai.z : 0.f;
        f[8] = gi.x * dt_large * ivs; f[9] = gi.y * dt_large * ivs; f[10] = gi.z * dt_large * ivs;
    }

    // neighbour j: pos4, (1/rho, p), vel4, alpha4
    __device__ __forceinline__ void pair(const DevParams& P, const float4 pj, const float2 dj, const float4 vj,
                                         const float4 aj) {
        const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
        const float dsq = dx * dx + dy * dy + dz * dz;
        if (!(dsq < P.r2 && dsq > 0.f)) return;
        const float rinv = rsqrtf(dsq);
        const float q2 = dsq * ir2, q = dsq * rinv * ih;
        const float w = (1.f - q2) * (1.f - q2) * (1.f - q2);
        const float g = (1.f - q) * (1.f - q);
        const float ux = dx * rinv, uy = dy * rinv, uz = dz * rinv;
        if (pj.w < 0.f) {  // boundary
            f[40] += w;
            f[41] += w * dx * ih; f[42] += w * dy * ih; f[43] += w * dz * ih;
            f[44] += 1.f / 32.f;
            return;
        }
        const float dvx = vj.x - vi.x, dvy = vj.y - vi.y, dvz = vj.z - vi.z;
        f[11] += w;
        f[12] += w * dx * ih; f[13] += w * dy * ih; f[14] += w * dz * ih;
        f[15] += w * dvx * ivs; f[16] += w * dvy * ivs; f[17] += w * dvz * ivs;
        f[18] += w * (__fdividef(1.f, dj.x * aj.w) - reli);
        f[19] += w * (dj.y - pres_i) * ips;
        f[20] += w * (aj.x - ai.x);
        f[21] += w * (P.nphase > 1 ? aj.y - ai.y : 0.f);
        f[22] += w * (P.nphase > 2 ? aj.z - ai.z : 0.f);
        const float wh2 = w * ih2;
        f[23] += wh2 * dx * dx; f[24] += wh2 * dy * dy; f[25] += wh2 * dz * dz;
        f[26] += wh2 * dx * dy; f[27] += wh2 * dx * dz; f[28] += wh2 * dy * dz;
        f[29] += g * ux; f[30] += g * uy; f[31] += g * uz;
        f[32] += g * (dvx * ux + dvy * uy + dvz * uz) * ivs;
        f[33] += g * (dvy * uz - dvz * uy) * ivs;
        f[34] += g * (dvz * ux - dvx * uz) * ivs;
        f[35] += g * (dvx * uy - dvy * ux) * ivs;
        const float pp = g * (pres_i + dj.y) * ips;
        f[36] += pp * ux; f[37] += pp * uy; f[38] += pp * uz;
        f[39] += 1.f / 32.f;
        const float da = g * (aj.x - ai.x);
        f[45] += da * ux; f[46] += da * uy; f[47] += da * uz;
    }

    __device__ __forceinline__ void store(float* row) const {
        float4* out = reinterpret_cast<float4*>(row);
#pragma unroll
        for (int i = 0; i < kLearnedFeatures / 4; i++)
            out[i] = make_float4(f[4 * i], f[4 * i + 1], f[4 * i + 2], f[4 * i + 3]);
    }
};

// A particle without features (boundary or out of the grid): zeros, id -1.
__device__ __forceinline__ void store_no_features(float* row, int32_t* id) {
    float4* out = reinterpret_cast<float4*>(row);
#pragma unroll
    for (int i = 0; i < kLearnedFeatures / 4; i++) out[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    *id = -1;
}

}  // namespace dev
}  // namespace sphmp
