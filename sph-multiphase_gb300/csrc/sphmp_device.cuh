// sphmp_device.cuh — device helpers and the per-pair physics of the multiphase
// SPH step used by the kernels in sphmp_kernels.cu.
//
// The physics follows the reference kernels of ZP-Z/sph-multiphase:
//   density / EOS      SPH_Solver/fluids/fluid_system_kern.cu:214-247, 279-318
//   force              SPH_Solver/fluids/fluid_system_kern.cu:325-424
//   drift velocity     SPH_Solver/fluids/multiphase.cu:19-166
//   alpha advance      SPH_Solver/fluids/multiphase.cu:169-272
//   correction         SPH_Solver/fluids/multiphase.cu:275-349
//   project-U force    SPH_Solver/fluids/multiphase.cu:488-616
//   advance            SPH_Solver/fluids/fluid_system_kern.cu:426-534
// in FP32, with Kahan-compensated density and volume-fraction sums.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "sphmp_internal.h"

namespace sphmp {
namespace dev {

constexpr int kThreads = 256;

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

// Kahan-compensated float accumulator.
struct Kahan {
    float s, c;
    __device__ __forceinline__ Kahan() : s(0.f), c(0.f) {}
    __device__ __forceinline__ void add(float y) {
        float yy = __fsub_rn(y, c);
        float t = __fadd_rn(s, yy);
        c = __fsub_rn(__fsub_rn(t, s), yy);
        s = t;
    }
};

// Grid coordinate in cell units, the reference's (pos - gridmin) * gridIdfac.
__device__ __forceinline__ float grid_t(float p, float gmin, float fac) { return __fmul_rn(__fsub_rn(p, gmin), fac); }
// int(t) is only defined inside the int range; outside it (and for NaN) the
// particle is out of the grid.
__device__ __forceinline__ bool t_ok(float t) { return t > -2147483520.f && t < 2147483520.f; }

__device__ __forceinline__ uint32_t cell_key(const DevParams& P, float x, float y, float z) {
    const float tx = grid_t(x, P.gmin[0], P.fac[0]);
    const float ty = grid_t(y, P.gmin[1], P.fac[1]);
    const float tz = grid_t(z, P.gmin[2], P.fac[2]);
    if (!(t_ok(tx) && t_ok(ty) && t_ok(tz))) return kUndef;
    const int gx = __float2int_rz(tx), gy = __float2int_rz(ty), gz = __float2int_rz(tz);
    if (gx >= 1 && gx < P.rx - 1 && gy >= 1 && gy < P.ry - 1 && gz >= 1 && gz < P.rz - 1)
        return (uint32_t)((gy * P.rz + gz) * P.rx + gx);
    return kUndef;
}

// Octant (h-subcell inside its 2h cell) of an in-grid position: bit 0 = x half,
// bit 1 = z half, bit 2 = y half, from int(2 t) with t the reference's grid coordinate.
__device__ __forceinline__ uint32_t octant_of(const DevParams& P, const float4 p) {
    const int hx = __float2int_rz(2.f * grid_t(p.x, P.gmin[0], P.fac[0]));
    const int hy = __float2int_rz(2.f * grid_t(p.y, P.gmin[1], P.fac[1]));
    const int hz = __float2int_rz(2.f * grid_t(p.z, P.gmin[2], P.fac[2]));
    return (uint32_t)(((hy & 1) * 2 + (hz & 1)) * 2 + (hx & 1));
}

__device__ __forceinline__ void set_err(const DevBuffers& B, uint32_t bit) { atomicOr(B.err, bit); }

// Grid coordinates (x, y, z) of an in-grid cell id, (gy * rz + gz) * rx + gx.
__device__ __forceinline__ void cell_coords(const DevParams& P, uint32_t cell, int (&g)[3]) {
    g[0] = (int)(cell % (uint32_t)P.rx);
    const uint32_t yz = cell / (uint32_t)P.rx;
    g[2] = (int)(yz % (uint32_t)P.rz);
    g[1] = (int)(yz / (uint32_t)P.rz);
}

// Visit the candidate slots of an in-grid particle at (x, y, z) registered in
// cell `cell` by the last sort: the reference's 3x3x3 cells around that cell
// (contributeDensity and the other neighbour loops scan gc + neighborid[c]).
// While the positions are the ones the sort binned (P.narrow), the block is
// narrowed along each axis to the cells within [t - R, t + R] of the position
// (R = h in cell units plus a margin), which hold every particle within h of
// it; after the particles have moved (a pass called without a new sort) the
// whole block is scanned, as the reference does. The stored cell lies in the
// grid's interior, so every cell visited exists. In the linear cell order the
// cells along x are adjacent in the sorted arrays, so each (y, z) row of cells
// is one contiguous slot range; in the Morton order each cell is its own range.
template <class F>
__device__ __forceinline__ void for_candidate_rows(const DevParams& P, const DevBuffers& B, uint32_t cell, float x,
                                                   float y, float z, F&& f) {
    const uint32_t* __restrict__ cstart = B.cstart;
    const float t[3] = {grid_t(x, P.gmin[0], P.fac[0]), grid_t(y, P.gmin[1], P.fac[1]),
                        grid_t(z, P.gmin[2], P.fac[2])};
    int g[3];
    cell_coords(P, cell, g);
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        lo[a] = g[a] - 1;
        hi[a] = g[a] + 1;
        if (P.narrow) {
            lo[a] = max(lo[a], __float2int_rd(t[a] - P.srad[a]));
            hi[a] = min(hi[a], __float2int_rd(t[a] + P.srad[a]));
        }
    }
    for (int yy = lo[1]; yy <= hi[1]; yy++) {
        for (int zz = lo[2]; zz <= hi[2]; zz++) {
            const int base = (yy * P.rz + zz) * P.rx;
            if (P.morton) {
                for (int xx = lo[0]; xx <= hi[0]; xx++) f(__ldg(&cstart[base + xx]), __ldg(&B.cend[base + xx]));
            } else {
                f(__ldg(&cstart[base + lo[0]]), __ldg(&cstart[base + hi[0] + 1]));
            }
        }
    }
}

// The candidates one by one (see for_candidate_rows: each row is the slot range [j0, j1)).
template <class F>
__device__ __forceinline__ void for_candidates(const DevParams& P, const DevBuffers& B, uint32_t cell, float x,
                                               float y, float z, F&& f) {
    for_candidate_rows(P, B, cell, x, y, z, [&](uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0; j < j1; j++) f(j);
    });
}

// Neighbour index lists: entry k of particle s at ((k / 4) * cap + s) * 4 + k % 4,
// i.e. groups of four consecutive entries per particle with the groups
// column-major: a warp reads one group row (entries 4g .. 4g + 3 of its 32
// particles) as one coalesced 512-byte load, and a walk holds the next three
// indices in registers before it needs them.
__device__ __forceinline__ size_t nbr_at(size_t cap, uint32_t s, uint32_t k) {
    return ((size_t)(k >> 2) * cap + (size_t)s) * 4u + (k & 3u);
}

// Group rows of the lists are streamed from DRAM (the lists outgrow L2); the
// walk asks L2 for the row kListPrefetch groups ahead, so the load of a group
// rarely waits on DRAM.
constexpr uint32_t kListPrefetch = 2;

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// The candidates marked in mask words wd0, wd0 + step, ... of particle s's
// bucket mask list (bucket `bid`, whose range table in btab maps sequence
// position e to index e + delta of the range holding e).
template <class F>
__device__ __forceinline__ void for_mask_words(const DevParams& P, const DevBuffers& B, int s, uint32_t bid,
                                               uint32_t wd0, uint32_t step, F&& f) {
    const uint32_t* __restrict__ tab = B.btab + (size_t)bid * kTabStride;
    const uint32_t nw = (__ldg(&tab[18]) + 31u) >> 5;
    const size_t cap = (size_t)P.cap;
    int r = 0;
    uint32_t end = __ldg(&tab[1]), delta = __ldg(&tab[20]);
    for (uint32_t wd = wd0; wd < nw; wd += step) {
        uint32_t m = __ldg(&B.nmask[(size_t)wd * cap + s]);
        while (m != 0u) {
            const uint32_t e = (wd << 5) + (uint32_t)(__ffs(m) - 1);
            m &= m - 1u;
            while (e >= end) {  // ends at tab[18] = the sequence length > e
                r++;
                end = __ldg(&tab[r + 1]);
                delta = __ldg(&tab[20 + r]);
            }
            f(e + delta);
        }
    }
}

// Visit the neighbours of particle s from the index list of the density pass
// when it is valid and did not overflow, from the bucket mask list when the
// index list overflowed, otherwise by the cell search.
template <class F>
__device__ __forceinline__ void for_slot_list(const DevParams& P, const DevBuffers& B, int s, float x, float y,
                                              float z, F&& f) {
    if (P.list_mode != 0) {
        const uint32_t raw = B.nbr_cnt[s];
        if (raw & kMaskList) {
            for_mask_words(P, B, s, raw & ~kMaskList, 0u, 1u, f);
            return;
        }
        const uint32_t cnt = raw & ~kHeavyFlag;  // kRescan stays above kMaxNbr
        if (cnt <= (uint32_t)kMaxNbr) {
            const uint4* __restrict__ grp = reinterpret_cast<const uint4*>(B.nbr) + s;
            const size_t cap = (size_t)P.cap;
            const uint32_t ng = (cnt + 3u) >> 2;
            for (uint32_t g = 0; g < kListPrefetch && g < ng; g++) prefetch_l2(grp + (size_t)g * cap);
            for (uint32_t g = 0; g < ng; g++) {
                if (g + kListPrefetch < ng) prefetch_l2(grp + (size_t)(g + kListPrefetch) * cap);
                const uint4 q = __ldg(grp + (size_t)g * cap);
                const uint32_t k = g << 2;
                f(q.x);
                if (k + 1u < cnt) f(q.y);
                if (k + 2u < cnt) f(q.z);
                if (k + 3u < cnt) f(q.w);
            }
            return;
        }
    }
    for_candidates(P, B, B.mgcell[s], x, y, z, f);
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Heavy particles: in the force and alpha passes every warp first takes heavy
// particles from hq (one particle per warp, its neighbours shared out over the
// lanes) while any are left, then its own 32 particles without the heavy ones.
// In a squeezed cluster all 32 particles of a warp can have hundreds of
// neighbours; walked by their own threads they would hold that warp for
// hundreds of dependent list steps while the rest of the GPU idles.
__device__ __forceinline__ bool is_heavy(const DevParams& P, uint32_t raw) {
    return P.list_mode != 0 && (raw & (kHeavyFlag | kMaskList)) != 0u;
}

// The next queue entry for the calling warp (every lane calls), or n when the
// queue of n entries is used up; the atomic is skipped once the counter has
// passed n, so that the warps arriving after the queue is empty do not all
// serialise on it.
__device__ __forceinline__ uint32_t next_item(uint32_t* ctr, uint32_t n, unsigned lane) {
    uint32_t v = n;
    if (lane == 0 && *(volatile uint32_t*)ctr < n) v = min(atomicAdd(ctr, 1u), n);
    return __shfl_sync(0xffffffffu, v, 0);
}

// The neighbours of particle s shared out over the 32 lanes of the warp (every
// lane calls with the same s): list entries k = lane, lane + 32, ..., or each
// row of the cell search likewise. The caller reduces the lanes' partial sums.
template <class F>
__device__ __forceinline__ void warp_for_slot_list(const DevParams& P, const DevBuffers& B, int s, float x, float y,
                                                   float z, F&& f) {
    const unsigned lane = lane_id();
    if (P.list_mode != 0) {
        const uint32_t raw = B.nbr_cnt[s];
        if (raw & kMaskList) {  // one mask word (32 candidates) per lane at a time
            for_mask_words(P, B, s, raw & ~kMaskList, lane, 32u, f);
            return;
        }
        const uint32_t cnt = raw & ~kHeavyFlag;
        if (cnt <= (uint32_t)kMaxNbr) {
            const size_t cap = (size_t)P.cap;
            for (uint32_t k = lane; k < cnt; k += 32) f(__ldg(B.nbr + nbr_at(cap, (uint32_t)s, k)));
            return;
        }
    }
    for_candidate_rows(P, B, B.mgcell[s], x, y, z, [&](uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0 + lane; j < j1; j += 32) f(j);
    });
}

// ---------------------------------------------------------------------------
// Density + EOS (MfComputePressureCUDA)
// ---------------------------------------------------------------------------

// Tait (2.5 * rho0 * ((rho/rho0)^7 - 1)) or the linear extension, clamped at
// 0; rho == 0 reads as 1. The reference's 2.5 is a double literal, so its two
// products are taken in double (fluid_system_kern.cu:310) and rounded to float
// once, as here.
__device__ __forceinline__ float2 density_result(const DevParams& P, float wsum, float rho0) {
    float rho = wsum * P.kpoly6;
    if (rho == 0.f) rho = 1.f;
    float p;
    if (P.eos == SPHMP_EOS_LINEAR) p = P.eos_k * (rho - rho0);
    else p = (float)(2.5 * (double)rho0 * (double)(powf(rho / rho0, 7.0f) - 1.0f));
    if (p < 0.f) p = 0.f;
    return make_float2(1.f / rho, p);
}

// ---------------------------------------------------------------------------
// Force + drift velocity (MfComputeForceCUDA, MfComputeDriftVelCUDA)
// ---------------------------------------------------------------------------

// Neighbour record of particle s for the alpha pass, 80 contiguous bytes:
//   {x, y, z, md}, {veleval xyz, alpha_0}, {alpha_1, alpha_2, u_0x, u_0y},
//   {u_0z, u_1xyz}, {u_2xyz, 0}
// with md = mass * (1/rho) for fluid particles and -1 for boundary particles
// (which exchange no volume fraction), u_k the drift velocities. (A 96-byte
// record read with three 32-byte loads measured slower: 0.314 against
// 0.295 ms per alpha pass, from the larger records missing L2.)
__device__ __forceinline__ void write_nrec(const DevBuffers& B, int s, const float4 p, float md, const float4 ve,
                                           const float (&a)[3], const float (&u)[9]) {
    float4* r = B.nrec + (size_t)s * kNrecFloat4;
    r[0] = make_float4(p.x, p.y, p.z, md);
    r[1] = make_float4(ve.x, ve.y, ve.z, a[0]);
    r[2] = make_float4(a[1], a[2], u[0], u[1]);
    r[3] = make_float4(u[2], u[3], u[4], u[5]);
    r[4] = make_float4(u[6], u[7], u[8], 0.f);
}

// The five float4 of neighbour j's record (the fifth only with three phases).
// (Reading the 80-byte records with three aligned 32-byte loads from the
// 32-byte boundary at or below each record measured slower: 0.306 against
// 0.291 ms per alpha pass at full size.)
template <int NP>
__device__ __forceinline__ void read_nrec(const DevBuffers& B, uint32_t j, float4 (&q)[5]) {
    const float4* __restrict__ r = B.nrec + (size_t)j * kNrecFloat4;
    q[0] = __ldg(r);
    q[1] = __ldg(r + 1);
    q[2] = __ldg(r + 2);
    q[3] = __ldg(r + 3);
    q[4] = NP > 2 ? __ldg(r + 4) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// Accumulates the force (contributeForce_new) and / or the drift-velocity terms
// (contributeDriftVel) of one in-grid fluid particle over its neighbours.
// `pair` takes the neighbour's pos4, (1/rho, p), vel4 and alpha4.
template <bool FORCE, bool DRIFT, int NP>
struct ForceDrift {
    static constexpr int K = NP > 0 ? NP : 1;
    float4 pi, vi;
    float idens, ipress, ivisc, rho0;
    float ia[3];
    float mc[K];
    float relax_coef, invdens;
    float fx, fy, fz;
    float3 dv[K], ag[K];  // dv: the pressure-gradient sums of phase k until finish() forms the drift term

    __device__ __forceinline__ void init(const DevParams& P, float4 pi_, float4 vi_, float2 dpi, float4 ai) {
        pi = pi_;
        vi = vi_;
        idens = dpi.x;
        ipress = dpi.y;
        ivisc = vi_.w;
        rho0 = ai.w;
        ia[0] = ai.x; ia[1] = ai.y; ia[2] = ai.z;
        fx = fy = fz = 0.f;
        relax_coef = invdens = 0.f;
        if (DRIFT) {
            relax_coef = P.relax / ivisc;
            invdens = 1.f / rho0;
#pragma unroll
            for (int k = 0; k < NP; k++) {
                mc[k] = ia[k] * P.dens_k[k] * invdens;
                dv[k] = make_float3(0.f, 0.f, 0.f);
                ag[k] = make_float3(0.f, 0.f, 0.f);
            }
        }
    }

    __device__ __forceinline__ void pair(const DevParams& P, const float4 pj, const float2 dpj, const float4 vj,
                                         const float4 aj) {
        const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
        const float dsq = dx * dx + dy * dy + dz * dz;
        if (!(dsq < P.r2 && dsq > 0.f)) return;
        const float rinv = rsqrtf(dsq);  // 1/r; r = dsq/r
        const float c = P.h - dsq * rinv;
        const float g1 = P.kspikydiff * c * c * rinv;
        if (pj.w > 0.f) {  // fluid neighbour
            const float g = g1 * pj.w * dpj.x;
            if (FORCE) {
                const float pm = -0.5f * g * dpj.y * idens;
                fx += dx * pm; fy += dy * pm; fz += dz * pm;
                const float vm = g * (ivisc + vj.w) * idens;
                fx += (vi.x - vj.x) * vm; fy += (vi.y - vj.y) * vm; fz += (vi.z - vj.z) * vm;
            }
            if (DRIFT) {
                const float ja[3] = {aj.x, aj.y, aj.z};
                // the pressure-gradient terms summed per phase; the mass-weighted
                // phase average is subtracted once per particle (finish): the sum
                // over pairs of (pg_k - sum_k' mc_k' pg_k') is linear in pg
#pragma unroll
                for (int k = 0; k < NP; k++) {
                    const float pm = g * (-ia[k] * ipress + ja[k] * dpj.y);
                    dv[k].x += pm * dx; dv[k].y += pm * dy; dv[k].z += pm * dz;
                    const float ga = (ja[k] - ia[k]) * g;
                    ag[k].x += ga * dx; ag[k].y += ga * dy; ag[k].z += ga * dz;
                }
            }
        } else if (FORCE) {  // boundary neighbour, volume V_j = -w
            const float V = -pj.w;
            const float pm = -g1 * rho0 * V * ipress * idens * idens;
            fx += dx * pm; fy += dy * pm; fz += dz * pm;
            float pij = (vi.x - vj.x) * dx + (vi.y - vj.y) * dy + (vi.z - vj.z) * dz;
            if (pij < 0.f) {
                pij = pij / (dsq + P.r2 * 0.01f);
                pij = pij * P.bvisc * P.h / 2.f / rho0;
                pij = g1 * rho0 * V * pij;
                fx += dx * pij; fy += dy * pij; fz += dz * pij;
            }
        }
    }

    // Sum the lanes' partial sums (warp-cooperative particles); every lane gets the totals.
    __device__ __forceinline__ void warp_reduce() {
        if (FORCE) {
            fx = warp_sum_f(fx);
            fy = warp_sum_f(fy);
            fz = warp_sum_f(fz);
        }
        if (DRIFT) {
#pragma unroll
            for (int k = 0; k < NP; k++) {
                dv[k].x = warp_sum_f(dv[k].x); dv[k].y = warp_sum_f(dv[k].y); dv[k].z = warp_sum_f(dv[k].z);
                ag[k].x = warp_sum_f(ag[k].x); ag[k].y = warp_sum_f(ag[k].y); ag[k].z = warp_sum_f(ag[k].z);
            }
        }
    }

    // mfComputeDriftVel's closing terms (multiphase.cu:131-163) and the stores.
    // `vev` (the particle's veleval) is only read when FORCE and DRIFT run
    // together: that pass also writes the particle's neighbour record for the
    // alpha pass (write_nrec).
    __device__ __forceinline__ void finish(const DevParams& P, const DevBuffers& B, int s, const float4 ap,
                                           const float4 vev = make_float4(0.f, 0.f, 0.f, 0.f)) {
        if (FORCE) B.accel4[s] = make_float4(fx, fy, fz, 0.f);
        if (DRIFT) {
            const float cc = P.cont * P.cont2;
            const float cs = P.cont * P.cont1 * P.sigma;
            float3 out[K], st[K];
            float dsum = 0.f;
            float3 ssum = make_float3(0.f, 0.f, 0.f);
            {  // dv_k = -relax (sum pg_k - sum_k' mc_k' sum pg_k')
                float3 psum = make_float3(0.f, 0.f, 0.f);
#pragma unroll
                for (int k = 0; k < NP; k++) {
                    psum.x += dv[k].x * mc[k]; psum.y += dv[k].y * mc[k]; psum.z += dv[k].z * mc[k];
                }
#pragma unroll
                for (int k = 0; k < NP; k++) {
                    dv[k].x = -(relax_coef * (dv[k].x - psum.x));
                    dv[k].y = -(relax_coef * (dv[k].y - psum.y));
                    dv[k].z = -(relax_coef * (dv[k].z - psum.z));
                }
            }
#pragma unroll
            for (int k = 0; k < NP; k++) {
                out[k] = make_float3(cc * dv[k].x, cc * dv[k].y, cc * dv[k].z);
                const float temp = ia[k];
                dsum += temp * P.dens_k[k] * P.dens_k[k] * invdens;
                // `temp > 0.0001` in double is exactly `temp > 1e-4f` in float
                st[k] = temp > 1e-4f ? make_float3(ag[k].x / temp, ag[k].y / temp, ag[k].z / temp)
                                     : make_float3(0.f, 0.f, 0.f);
                ssum.x += st[k].x * temp * P.dens_k[k] * invdens;
                ssum.y += st[k].y * temp * P.dens_k[k] * invdens;
                ssum.z += st[k].z * temp * P.dens_k[k] * invdens;
            }
#pragma unroll
            for (int k = 0; k < NP; k++) {
                const float tdiff = (P.dens_k[k] - dsum) * relax_coef;
                out[k].x += ap.x * tdiff; out[k].y += ap.y * tdiff; out[k].z += ap.z * tdiff;
                out[k].x -= cs * (st[k].x - ssum.x);
                out[k].y -= cs * (st[k].y - ssum.y);
                out[k].z -= cs * (st[k].z - ssum.z);
                B.drift4[(size_t)k * P.cap + s] = make_float4(out[k].x, out[k].y, out[k].z, 0.f);
            }
            if (FORCE) {
                float u[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int k = 0; k < NP; k++) {
                    u[3 * k] = out[k].x;
                    u[3 * k + 1] = out[k].y;
                    u[3 * k + 2] = out[k].z;
                }
                write_nrec(B, s, pi, pi.w * idens, vev, ia, u);
            }
        }
    }
};


// ---------------------------------------------------------------------------
// Project-U force (ComputeForce_projectu)
// ---------------------------------------------------------------------------

// contributeForce_projectu (multiphase.cu:488-575) for one in-grid fluid
// particle: fluid neighbours give pressure with p_i + p_j, viscosity on
// veleval and the drift-velocity tensor of every phase; boundary neighbours
// give pressure (rest-density ratio, times omega) and, when approaching, the
// artificial viscosity (times visc_factor); every neighbour gives the XSPH
// term -(ve_i - ve_j) (h^2 - r^2)^3 m_j (2 / (1/D_j + 1/D_i)) kpoly6 / 2, with
// D the stored inverse density (the boundary volume for boundary particles).
// `pair` takes the neighbour's pos4, (1/rho, p), veleval, viscosity, rest
// density, raw mass, start-of-step fractions and drift velocities.
template <int NP>
struct ProjectU {
    float4 pi, vei;
    float idens, ipress, ivisc, rho0;
    float ia[3];
    float3 um[NP];
    float fx, fy, fz;
    float xx, xy, xz;

    __device__ __forceinline__ void init(float4 pi_, float4 vei_, float2 dpi, float visc, float rho0_,
                                         float4 apre, const float3* um_) {
        pi = pi_;
        vei = vei_;
        idens = dpi.x;
        ipress = dpi.y;
        ivisc = visc;
        rho0 = rho0_;
        ia[0] = apre.x; ia[1] = apre.y; ia[2] = apre.z;
#pragma unroll
        for (int k = 0; k < NP; k++) um[k] = um_[k];
        fx = fy = fz = 0.f;
        xx = xy = xz = 0.f;
    }

    __device__ __forceinline__ void pair(const DevParams& P, const float4 pj, const float2 dpj, const float4 vej,
                                         float viscj, float rho0j, float mj, const float4 aj, const float4* uj) {
        const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
        const float dsq = dx * dx + dy * dy + dz * dz;
        if (!(dsq < P.r2 && dsq > 0.f)) return;
        const float rinv = rsqrtf(dsq);
        const float c = P.h - dsq * rinv;
        const float g1 = P.kspikydiff * c * c * rinv;
        const float vx = vei.x - vej.x, vy = vei.y - vej.y, vz = vei.z - vej.z;
        float dj;  // the neighbour's stored inverse density (boundary: volume)
        if (pj.w > 0.f) {
            dj = dpj.x;
            const float g = g1 * mj * dj;
            const float pm = -0.5f * g * (ipress + dpj.y) * idens;
            fx += dx * pm; fy += dy * pm; fz += dz * pm;
            const float vm = g * (ivisc + viscj) * idens;
            fx += vx * vm; fy += vy * vm; fz += vz * vm;
            const float ja[3] = {aj.x, aj.y, aj.z};
#pragma unroll
            for (int k = 0; k < NP; k++) {
                const float tj = g * (uj[k].x * dx + uj[k].y * dy + uj[k].z * dz) * ja[k];
                const float ti = g * (um[k].x * dx + um[k].y * dy + um[k].z * dz) * ia[k];
                const float f = P.dens_k[k] * idens;
                fx += (tj * uj[k].x + ti * um[k].x) * f;
                fy += (tj * uj[k].y + ti * um[k].y) * f;
                fz += (tj * uj[k].z + ti * um[k].z) * f;
            }
        } else {
            dj = -pj.w;
            const float gb = g1 * rho0 * mj / rho0j;
            const float pm = -gb * ipress * idens * idens * P.omega;
            fx += dx * pm; fy += dy * pm; fz += dz * pm;
            float pij = vx * dx + vy * dy + vz * dz;
            if (pij < 0.f) {
                // the reference adds r2 in unscaled units (simData.r2 / d2) to the scaled distance
                pij = pij / (dsq + P.r2 / (P.ss * P.ss) * 0.01f);
                pij = pij * 2.f * P.h * (ivisc + viscj) * idens / 2.f;
                pij = -gb * pij * P.visc_factor;
                fx += dx * pij; fy += dy * pij; fz += dz * pij;
            }
        }
        const float cx = P.r2 - dsq;
        const float ave = 2.f / (1.f / dj + 1.f / idens);
        const float xt = cx * cx * cx * mj * ave * P.kpoly6 * 0.5f;
        xx -= vx * xt; xy -= vy * xt; xz -= vz * xt;
    }
};

// ---------------------------------------------------------------------------
// Volume-fraction advance (MfComputeAlphaAdvanceCUDA)
// ---------------------------------------------------------------------------

// Alpha change of one in-grid fluid particle (contributeAlphaChange), Kahan-
// compensated per phase. `pair` takes the neighbour's pos4, md = mass * (1/rho),
// veleval, alpha4 and drift velocities.
//
// Per pair and phase k the reference adds
//   -(0.5 cm (a_jk + a_ik) dot1) - cm (a_jk u_jk + a_ik u_ik) . d
// with cm the kernel-gradient factor times md and dot1 = (v_j - v_i) . d. The
// terms in a_ik are the particle's own fraction times the sums S_dot = sum cm
// dot1 and S_d = sum cm d, which are taken once for all phases (plain FP32
// sums); the neighbour terms -cm a_jk (0.5 dot1 + u_jk . d) are summed per phase
// (Kahan), and result() adds -a_ik (0.5 S_dot + u_ik . S_d) to each phase's
// compensated sum. Boundary neighbours (pos4.w <= 0) exchange no fraction.
template <int NP>
struct AlphaChange {
    float4 pi, vei;
    float ia[3];
    Kahan acc[NP];
    const float4* udrift;  // the particle's own drift velocity of phase k at udrift[k * ustride]
    size_t ustride;
    float sdot = 0.f, sdx = 0.f, sdy = 0.f, sdz = 0.f;

    // u is the particle's drift velocity of phase 0 (phase k at u[k * stride]),
    // read after the neighbour walk, in result().
    __device__ __forceinline__ void init(const float4 pi_, const float4 vei_, const float4 ai, const float4* u,
                                         size_t stride) {
        pi = pi_;
        vei = vei_;
        ia[0] = ai.x; ia[1] = ai.y; ia[2] = ai.z;
        udrift = u;
        ustride = stride;
    }

    __device__ __forceinline__ void pair(const DevParams& P, const float4 pj, const float md, const float4 vej,
                                         const float4 aj, const float4* uj) {
        if (!(pj.w > 0.f)) return;
        const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
        const float dsq = dx * dx + dy * dy + dz * dz;
        if (!(dsq < P.r2 && dsq > 0.f)) return;
        const float rinv = rsqrtf(dsq);
        const float c = P.h - dsq * rinv;
        const float cm = P.kspikydiff * c * c * rinv * md;
        const float dot1 = (vej.x - vei.x) * dx + (vej.y - vei.y) * dy + (vej.z - vei.z) * dz;
        const float ja[3] = {aj.x, aj.y, aj.z};
        sdot += cm * dot1;
        sdx += cm * dx;
        sdy += cm * dy;
        sdz += cm * dz;
        const float hd = 0.5f * dot1;
#pragma unroll
        for (int k = 0; k < NP; k++) {
            const float ud = uj[k].x * dx + uj[k].y * dy + uj[k].z * dz;
            acc[k].add(-(cm * (ja[k] * (hd + ud))));
        }
    }

    // Sum the lanes' compensated partial sums (warp-cooperative particles).
    __device__ __forceinline__ void warp_reduce() {
#pragma unroll
        for (int k = 0; k < NP; k++) {
            acc[k].s = warp_sum_f(acc[k].s - acc[k].c);
            acc[k].c = 0.f;
        }
        sdot = warp_sum_f(sdot);
        sdx = warp_sum_f(sdx);
        sdy = warp_sum_f(sdy);
        sdz = warp_sum_f(sdz);
    }

    // dalpha * dt clamped at -0.99, added to the start-of-step fraction.
    __device__ __forceinline__ void result(const DevParams& P, float (&out)[3]) {
#pragma unroll
        for (int k = 0; k < NP; k++) {
            const float4 um = udrift[(size_t)k * ustride];
            const float own = 0.5f * sdot + (um.x * sdx + um.y * sdy + um.z * sdz);
            acc[k].add(-(ia[k] * own));
            float ch = acc[k].s * P.dt;
            // `ch < -0.99` in double is exactly `ch <= -0.99f` in float
            if (ch <= -0.99f) ch = -0.99f;
            out[k] = ch + ia[k];
        }
    }
};

// mfComputeCorrection (multiphase.cu:275-349) for one particle. `a` holds the
// advanced fractions on entry and the corrected ones on exit; `apre` are the
// start-of-step fractions (argmax fallback).
template <int NP>
__device__ __forceinline__ void correct(const DevParams& P, float (&a)[3], const float (&apre)[3], float dens,
                                        float rho0, float& pmod, float& newrho0, float& newvisc) {
    float before[3];
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < NP; k++) {
        before[k] = a[k];
        if (a[k] < 0.f) a[k] = 0.f;
        sum += a[k];
    }
    const bool flag = sum > 0.f;
    if (!flag) sum = 1.f;
    int maxcat = 0;
#pragma unroll
    for (int k = 1; k < NP; k++)
        if (apre[k] > apre[maxcat]) maxcat = k;
    const float inv = 1.f / sum;
    const float x = 1.f / (dens * rho0);
    const float coef = -(6.f * powf(x, 7.0f) + 1.f) * P.pintstiff;
    float pm = 0.f;
#pragma unroll
    for (int k = 0; k < NP; k++) {
        a[k] = flag ? a[k] * inv : (k == maxcat ? 1.f : 0.f);
        pm += coef * P.dens_k[k] * (a[k] - before[k]);
    }
    float nd = 0.f, nv = 0.f;
#pragma unroll
    for (int k = 0; k < NP; k++) {
        nd += a[k] * P.dens_k[k];
        nv += a[k] * P.visc_k[k];
    }
    pmod = pm;
    newrho0 = nd;
    newvisc = nv;
}

// AdvanceParticles (fluid_system_kern.cu:426-534) for one in-grid non-boundary
// particle, with un-contracted float operations in the reference's order.
__device__ __forceinline__ void advance_one(const DevParams& P, float4& p, float4& v, float4& ve, float4& ap,
                                            const float4 acc) {
    const float a[3] = {__fadd_rn(acc.x, P.grav[0]), __fadd_rn(acc.y, P.grav[1]), __fadd_rn(acc.z, P.grav[2])};
    float* pp[3] = {&p.x, &p.y, &p.z};
    float* vv[3] = {&v.x, &v.y, &v.z};
    float* ee[3] = {&ve.x, &ve.y, &ve.z};
    float* aa[3] = {&ap.x, &ap.y, &ap.z};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float v0 = *vv[k];
        const float vn = __fadd_rn(__fmul_rn(a[k], P.dt), v0);
        *pp[k] = __fadd_rn(*pp[k], __fdiv_rn(__fmul_rn(vn, P.dt), P.ss));
        *ee[k] = __fmul_rn(__fadd_rn(v0, vn), 0.5f);
        *vv[k] = vn;
        *aa[k] = __fsub_rn(P.grav[k], a[k]);
    }
}

// Fused alpha + correction + advance of one slot (reads in*, returns the new
// values of the five float4 fields). `alpha_sum` runs the neighbour loop.
template <int NP, bool MP, class AlphaSum>
__device__ __forceinline__ void pass_c_slot(const DevParams& P, const DevBuffers& B, int s, bool undef, float4& p,
                                            float4& v, float4& ve, float4& al, float4& ap, AlphaSum&& alpha_sum) {
    if (p.w < 0.f) return;  // boundary: never advanced
    if (undef) {
        p.x = -1000.f; p.y = -1000.f; p.z = -1000.f;
        v.x = 0.f; v.y = 0.f; v.z = 0.f;
        return;
    }
    if (MP) {
        const float ia[3] = {al.x, al.y, al.z};
        float a[3] = {al.x, al.y, al.z};
        alpha_sum(a);
        float pmod, nr, nv;
        correct<NP>(P, a, ia, B.densp[s].x, al.w, pmod, nr, nv);
        al = make_float4(a[0], a[1], a[2], nr);
        v.w = nv;
        B.pmod[s] = pmod;
    }
    advance_one(P, p, v, ve, ap, B.accel4[s]);
}

}  // namespace dev
}  // namespace sphmp
