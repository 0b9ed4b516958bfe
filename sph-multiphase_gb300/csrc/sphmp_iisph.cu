// sphmp_iisph.cu — the reference's IISPH step (implicit incompressible SPH) for
// sm_103a: ComputeDensityIISPH, ComputeDii / ComputeAii (PredictAdvection), the
// relaxed-Jacobi pressure iteration (Pressure_DP, Pressure_Iter) and
// IntegrateIISPH, SPH_Solver/fluids/fluid_system_kern.cu:637-1115, driven as
// fluid_system_host.cu:504-557 drives them.
//
// One thread per particle over the reference's 27 cells (gc + neighborid[c], in
// the reference's cell order; each cell is the index range [cstart, cend) of the
// sort), with the reference's cubic-spline kernel of support 2h and its
// gradient, and its cut-offs as written (the advection viscosity within 2h,
// every other gradient sum within h). As in the reference, `dens` (densp.x)
// holds the density itself after the IISPH density pass, not its inverse. The
// per-particle IISPH arrays (d_ii, a_ii, predicted density, the pressure
// iterates, sum_j d_ij p_j, the density residue) live in DevBuffers.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "sphmp_device.cuh"
#include "sphmp_internal.h"

namespace sphmp {

namespace {

using namespace dev;

// kern (fluid_system_kern.cu:637-645): the cubic spline of support 2h.
__device__ __forceinline__ float ii_kern(const DevParams& P, float dx, float dy, float dz) {
    const float q = sqrtf(dx * dx + dy * dy + dz * dz) / P.h;
    if (q > 2.f) return 0.f;
    if (q > 1.f) return __fmul_rn(__fmul_rn(0.25f, powf(2.f - q, 3.0f)), P.kspline);
    return __fmul_rn(1.f - __fmul_rn(__fmul_rn(1.5f, q), q) + __fmul_rn(0.75f, powf(q, 3.0f)), P.kspline);
}

// nablakern (:647-671): its gradient at x_ij = (dx, dy, dz).
__device__ __forceinline__ float3 ii_nabla(const DevParams& P, float dx, float dy, float dz) {
    const float rmod = sqrtf(dx * dx + dy * dy + dz * dz);
    const float q = rmod / P.h;
    float fac;
    if (q > 2.f) return make_float3(0.f, 0.f, 0.f);
    if (q > 1.f) fac = 0.75f * (2.f - q) * (2.f - q) * (-1.f) / P.h / rmod * P.kspline;
    else fac = (-3.f * q + 2.25f * q * q) / P.h / rmod * P.kspline;
    return make_float3(dx * fac, dy * fac, dz * fac);
}

// The reference's 27 cells around the cell particle s was sorted into.
template <class F>
__device__ __forceinline__ void ii_cells(const DevParams& P, const DevBuffers& B, uint32_t gc, F&& f) {
    for (int c = 0; c < 27; c++) {
        const uint32_t cell = gc + (uint32_t)P.neighborid[c];
        f(__ldg(&B.cstart[cell]), __ldg(&B.cend[cell]));
    }
}

__device__ __forceinline__ bool ii_fluid(const DevParams& P, const DevBuffers& B, int s, const float4* pos4) {
    return s < active_n(B) && B.mgcell[s] != kUndef && !(pos4[s].w < 0.f);
}

// ComputeDensityIISPH (:1067-1115): rho_i = sum over every candidate of kern(x_ij) m_j,
// m_j = mass_j (fluid) or restdens_i V_j (boundary).
__global__ void __launch_bounds__(kThreads) k_ii_density(const __grid_constant__ DevParams P,
                                                         const __grid_constant__ DevBuffers B,
                                                         const float4* __restrict__ pos4,
                                                         const float4* __restrict__ alpha4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (!ii_fluid(P, B, s, pos4)) return;
    const float4 pi = pos4[s];
    const float rho0 = alpha4[s].w;
    float sum = 0.f;
    ii_cells(P, B, B.mgcell[s], [&](uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0; j < j1; j++) {
            const float4 pj = __ldg(&pos4[j]);
            const float mj = pj.w > 0.f ? pj.w : rho0 * (-pj.w);
            const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
            sum += ii_kern(P, dx, dy, dz) * mj;
        }
    });
    B.densp[s].x = sum;
}

// ComputeDii (:673-799): the advection acceleration (the boundary's artificial
// viscosity within 2h, summed per cell, plus gravity) and veleval = vel + a dt;
// d_ii = -sum over fluid j within h of nabla W_ij m_j, / rho_i / rho_i * dt * dt.
__global__ void __launch_bounds__(kThreads) k_ii_dii(const __grid_constant__ DevParams P,
                                                     const __grid_constant__ DevBuffers B,
                                                     const float4* __restrict__ pos4,
                                                     const float4* __restrict__ vel4, float4* __restrict__ vev4,
                                                     const float4* __restrict__ alpha4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (!ii_fluid(P, B, s, pos4)) return;
    const float4 pi = pos4[s], vi = vel4[s];
    const float rho0 = alpha4[s].w;
    const float h = P.h, h2 = h * h;
    float ax = 0.f, ay = 0.f, az = 0.f;
    ii_cells(P, B, B.mgcell[s], [&](uint32_t j0, uint32_t j1) {
        float cx = 0.f, cy = 0.f, cz = 0.f;
        for (uint32_t j = j0; j < j1; j++) {
            const float4 pj = __ldg(&pos4[j]);
            if (!(pj.w < 0.f)) continue;  // only boundary neighbours contribute (fluid terms are commented out)
            const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            if (!(dist < 2.f * h && dist > 0.f)) continue;
            const float3 nw = ii_nabla(P, dx, dy, dz);
            const float4 vj = __ldg(&vel4[j]);
            float pij = dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z);
            if (pij < 0.f) {
                pij = (float)((double)pij / ((double)(dist * dist) + (double)h2 * 0.01));
                pij = pij * P.bvisc * P.h / 2.f / rho0;
                pij = rho0 * (-pj.w) * pij;
                cx += nw.x * pij; cy += nw.y * pij; cz += nw.z * pij;
            }
        }
        ax = ax + cx; ay = ay + cy; az = az + cz;
    });
    ax += P.grav[0]; ay += P.grav[1]; az += P.grav[2];
    vev4[s] = make_float4(vi.x + ax * P.dt, vi.y + ay * P.dt, vi.z + az * P.dt, 0.f);
    float3 d = make_float3(0.f, 0.f, 0.f);
    ii_cells(P, B, B.mgcell[s], [&](uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0; j < j1; j++) {
            const float4 pj = __ldg(&pos4[j]);
            const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            if (!(dist < h && dist > 0.f)) continue;
            if (pj.w < 0.f) continue;
            const float3 nw = ii_nabla(P, dx, dy, dz);
            d.x = d.x - nw.x * pj.w; d.y = d.y - nw.y * pj.w; d.z = d.z - nw.z * pj.w;
        }
    });
    const float rho = B.densp[s].x;
    B.iis_dii[s] = make_float4(d.x / rho / rho * P.dt * P.dt, d.y / rho / rho * P.dt * P.dt,
                               d.z / rho / rho * P.dt * P.dt, 0.f);
}

// ComputeAii (:801-908): rho_adv = rho_i + sum over fluid j within h of
// (veleval_i - veleval_j).nabla W_ij m_j dt (per cell), p_l = 0.5 p_i, and
// a_ii = sum over fluid j within h of (d_ii - d_ji).nabla W_ij m_j (per cell),
// d_ji = nabla W_ij m_i / rho_i / rho_i dt dt.
__global__ void __launch_bounds__(kThreads) k_ii_aii(const __grid_constant__ DevParams P,
                                                     const __grid_constant__ DevBuffers B,
                                                     const float4* __restrict__ pos4,
                                                     const float4* __restrict__ vev4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (!ii_fluid(P, B, s, pos4)) return;
    const float4 pi = pos4[s], vei = vev4[s], dii = B.iis_dii[s];
    const float2 dpi = B.densp[s];
    const float rho = dpi.x, mi = pi.w, h = P.h;
    float change = 0.f, aii = 0.f;
    ii_cells(P, B, B.mgcell[s], [&](uint32_t j0, uint32_t j1) {
        float sum = 0.f, sa = 0.f;
        for (uint32_t j = j0; j < j1; j++) {
            const float4 pj = __ldg(&pos4[j]);
            if (pj.w < 0.f) continue;
            const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            if (!(dist < h && dist > 0.f)) continue;
            const float3 nw = ii_nabla(P, dx, dy, dz);
            const float4 vej = __ldg(&vev4[j]);
            sum += ((vei.x - vej.x) * nw.x + (vei.y - vej.y) * nw.y + (vei.z - vej.z) * nw.z) * pj.w * P.dt;
            const float tx = dii.x - nw.x * mi / rho / rho * P.dt * P.dt;
            const float ty = dii.y - nw.y * mi / rho / rho * P.dt * P.dt;
            const float tz = dii.z - nw.z * mi / rho / rho * P.dt * P.dt;
            sa += (tx * nw.x + ty * nw.y + tz * nw.z) * pj.w;
        }
        change += sum;
        aii += sa;
    });
    B.iis_rho_adv[s] = rho + change;
    B.iis_pl[s] = 0.5f * dpi.y;
    B.iis_aii[s] = aii;
}

// Pressure_DP (:910-958): sum_j d_ij p_j = -dt dt sum over fluid j within h of
// nabla W_ij p_l,j m_j / rho_j / rho_j.
__global__ void __launch_bounds__(kThreads) k_ii_dp(const __grid_constant__ DevParams P,
                                                    const __grid_constant__ DevBuffers B,
                                                    const float4* __restrict__ pos4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (!ii_fluid(P, B, s, pos4)) return;
    const float4 pi = pos4[s];
    float3 d = make_float3(0.f, 0.f, 0.f);
    ii_cells(P, B, B.mgcell[s], [&](uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0; j < j1; j++) {
            const float4 pj = __ldg(&pos4[j]);
            if (pj.w < 0.f) continue;
            const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            if (!(dist < P.h && dist > 0.f)) continue;
            const float3 nw = ii_nabla(P, dx, dy, dz);
            const float rj = __ldg(&B.densp[j].x), plj = __ldg(&B.iis_pl[j]);
            d.x = d.x + nw.x * plj * pj.w / rj / rj * (-1.f);
            d.y = d.y + nw.y * plj * pj.w / rj / rj * (-1.f);
            d.z = d.z + nw.z * plj * pj.w / rj / rj * (-1.f);
        }
    });
    B.iis_dijpj[s] = make_float4(d.x * P.dt * P.dt, d.y * P.dt * P.dt, d.z * P.dt * P.dt, 0.f);
}

// Pressure_Iter (:960-1050) with omega 0.1: p_l1 = (1 - omega) p_l + omega / a_ii
// (rho0 - rho_adv - t), t = sum over fluid j within h of m_j (dijpj_i - d_jj p_l,j -
// (dijpj_j - d_ji p_l,i)).nabla W_ij (p_l1 = p_l where |a_ii| < 1e-5); the density
// residue rho_adv + t + a_ii p_l - rho0; accel = (d_ii p_l + dijpj) / dt / dt and
// pressure = p_l1. Boundary particles get residue 0; also the FP64 sums of the
// residue over all slots and of |residue| over in-grid fluid particles.
__global__ void __launch_bounds__(kThreads) k_ii_iter(const __grid_constant__ DevParams P,
                                                      const __grid_constant__ DevBuffers B,
                                                      const float4* __restrict__ pos4,
                                                      const float4* __restrict__ alpha4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    double r_all = 0.0, r_abs = 0.0, cnt = 0.0;
    if (s < active_n(B)) {
        const float4 pi = pos4[s];
        if (pi.w < 0.f) {
            B.iis_res[s] = 0.f;
        } else if (B.mgcell[s] != kUndef) {
            const float4 dii = B.iis_dii[s], dpi = B.iis_dijpj[s];
            const float rho = B.densp[s].x, pli = B.iis_pl[s], mi = pi.w;
            float ut = 0.f;
            ii_cells(P, B, B.mgcell[s], [&](uint32_t j0, uint32_t j1) {
                for (uint32_t j = j0; j < j1; j++) {
                    const float4 pj = __ldg(&pos4[j]);
                    if (pj.w < 0.f) continue;
                    const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
                    const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
                    if (!(dist < P.h && dist > 0.f)) continue;
                    const float3 nw = ii_nabla(P, dx, dy, dz);
                    const float4 djj = __ldg(&B.iis_dii[j]), dpj = __ldg(&B.iis_dijpj[j]);
                    const float plj = __ldg(&B.iis_pl[j]);
                    const float kx = dpj.x - nw.x * mi / rho / rho * P.dt * P.dt * pli;
                    const float ky = dpj.y - nw.y * mi / rho / rho * P.dt * P.dt * pli;
                    const float kz = dpj.z - nw.z * mi / rho / rho * P.dt * P.dt * pli;
                    const float tx = dpi.x - djj.x * plj - kx, ty = dpi.y - djj.y * plj - ky;
                    const float tz = dpi.z - djj.z * plj - kz;
                    ut += pj.w * (tx * nw.x + ty * nw.y + tz * nw.z);
                }
            });
            const float omega = 0.1f, aii = B.iis_aii[s], rho0 = alpha4[s].w, radv = B.iis_rho_adv[s];
            const float pl1 = fabsf(aii) < 0.00001f ? pli : (1.f - omega) * pli + omega / aii * (rho0 - radv - ut);
            B.iis_pl1[s] = pl1;
            const float res = -rho0 + (radv + ut + aii * pli);
            B.iis_res[s] = res;
            B.accel4[s] = make_float4((dii.x * pli + dpi.x) / P.dt / P.dt, (dii.y * pli + dpi.y) / P.dt / P.dt,
                                      (dii.z * pli + dpi.z) / P.dt / P.dt, 0.f);
            B.densp[s].y = pl1;
            r_all = res;
            r_abs = fabs((double)res);
            cnt = 1.0;
        }
    }
    // block sums into red[8..10]: residue over all slots, |residue| and the count of in-grid fluid
    __shared__ double sh[3][kThreads / 32];
    double v[3] = {r_all, r_abs, cnt};
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 3; q++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
        if (lane == 0) sh[q][warp] = v[q];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; w++) t += sh[threadIdx.x][w];
        atomicAdd(&B.red[8 + threadIdx.x], t);
    }
}

// The device copy press_l = press_l1 that ends each iteration (:535).
__global__ void __launch_bounds__(kThreads) k_ii_swap(const __grid_constant__ DevBuffers B) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s < active_n(B)) B.iis_pl[s] = B.iis_pl1[s];
}

// IntegrateIISPH (:1052-1065): vel = veleval + accel dt; pos += vel dt / simscale.
__global__ void __launch_bounds__(kThreads) k_ii_integrate(const __grid_constant__ DevParams P,
                                                           const __grid_constant__ DevBuffers B,
                                                           float4* __restrict__ pos4, float4* __restrict__ vel4,
                                                           const float4* __restrict__ vev4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (!ii_fluid(P, B, s, pos4)) return;
    const float4 ve = vev4[s], a = B.accel4[s];
    float4 v = vel4[s], p = pos4[s];
    v.x = ve.x + a.x * P.dt;
    v.y = ve.y + a.y * P.dt;
    v.z = ve.z + a.z * P.dt;
    p.x += v.x * P.dt / P.ss;
    p.y += v.y * P.dt / P.ss;
    p.z += v.z * P.dt / P.ss;
    vel4[s] = v;
    pos4[s] = p;
}

inline int blocks_for(int n) { return (n + kThreads - 1) / kThreads; }

}  // namespace

void launch_iisph_density(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    k_ii_density<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]], B.f4[ALPHA][cur[ALPHA]]);
}

void launch_iisph_predict(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    k_ii_dii<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]], B.f4[VEL][cur[VEL]],
                                                  B.f4[VEV][cur[VEV]], B.f4[ALPHA][cur[ALPHA]]);
    k_ii_aii<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]], B.f4[VEV][cur[VEV]]);
}

void launch_iisph_iteration(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    cudaMemsetAsync(B.red + 8, 0, sizeof(double) * 3, s);
    if (P.n <= 0) return;
    k_ii_dp<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]]);
    k_ii_iter<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]], B.f4[ALPHA][cur[ALPHA]]);
    k_ii_swap<<<blocks_for(P.n), kThreads, 0, s>>>(B);
}

void launch_iisph_integrate(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    k_ii_integrate<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]], B.f4[VEL][cur[VEL]],
                                                        B.f4[VEV][cur[VEV]]);
}

}  // namespace sphmp
