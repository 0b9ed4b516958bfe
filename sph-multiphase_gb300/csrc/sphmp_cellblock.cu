// sphmp_cellblock.cu — neighbour passes organised by cell blocks.
//
// One CTA takes one 2h cell with members at a time. The candidates of every
// member lie in the 4x4x4 block of h-subcells around the cell (the cell's own
// 2x2x2 subcells plus one subcell on each side). The CTA copies that block into
// shared memory once, bucket by bucket from the octant order (each bucket is a
// contiguous range), in a fixed order: subcells x fastest, then z, then y. A
// member's 27 subcells are then nine contiguous runs of the stage.
//
//  * density pass: every member scans its nine runs (about 216 candidates),
//    accumulates the density and writes its neighbour list as 16-bit stage
//    indices;
//  * force + drift pass and alpha + correction + advance pass: the CTA stages
//    the same block (identical positions, so identical stage indices) with the
//    neighbour fields the pass needs, and every member walks its list in
//    shared memory.
//
// A block with more candidates than a pass can stage is handled with global
// gathers: a list entry e is decoded to its octant-order position through the
// block's bucket table. A block too large for the density stage falls back to
// slot lists (nbr_cnt flag kListGlobal); a list longer than kMaxNbr is redone
// by the cell search.
//
// Pairs are restricted to the 3x3x3 h-subcells around a particle. Two particles
// in subcells two apart along an axis are more than one subcell apart, and the
// subcell edge equals h up to the float rounding of the grid size (below
// 1e-7 h), so such a pair lies within 1e-7 h of the cutoff, where the kernels
// (h^2 - r^2)^3 and (h - r)^2 are below 1e-13 of their values at r = h/2.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sphmp_device.cuh"
#include "sphmp_internal.h"

namespace sphmp {

namespace {

using namespace dev;

// Bucket table of a cell block: start[q] is the first stage index of subcell q
// (q = (y * 4 + z) * 4 + x, block-local), start[64] the number staged; kbeg[q]
// the first octant-order position of its bucket.
struct BlockIdx {
    uint32_t start[65];
    uint32_t kbeg[64];
    uint32_t wtot;
};

__device__ __forceinline__ void block_setup(const DevParams& P, const DevBuffers& B, uint32_t c, BlockIdx& bi) {
    const int tid = threadIdx.x;
    const int gx = (int)(c % (uint32_t)P.rx);
    const int gr = (int)(c / (uint32_t)P.rx);
    const int gz = gr % P.rz, gy = gr / P.rz;
    uint32_t cnt = 0;
    if (tid < 64) {
        const int a = tid & 3, zc = (tid >> 2) & 3, yb = tid >> 4;
        const int hx = 2 * gx - 1 + a, hz = 2 * gz - 1 + zc, hy = 2 * gy - 1 + yb;
        const uint32_t cc = (uint32_t)(((hy >> 1) * P.rz + (hz >> 1)) * P.rx + (hx >> 1));
        const uint32_t cs = __ldg(&B.cstart[cc]), ce = __ldg(&B.cstart[cc + 1]);
        uint32_t kb = cs;
        if (cs != ce) {
            const int oc = ((hy & 1) * 2 + (hz & 1)) * 2 + (hx & 1);
            kb = __ldg(&B.oct_start[(size_t)cc * 8 + oc]);
            const uint32_t ke = oc == 7 ? ce : __ldg(&B.oct_start[(size_t)cc * 8 + oc + 1]);
            cnt = ke - kb;
        }
        bi.kbeg[tid] = kb;
    }
    uint32_t x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if ((int)lane_id() >= o) x += y;
    }
    if (tid == 31) bi.wtot = x;
    __syncthreads();
    if (tid < 64) {
        const uint32_t incl = x + (tid >= 32 ? bi.wtot : 0u);
        bi.start[tid] = incl - cnt;
        if (tid == 63) bi.start[64] = incl;
    }
    __syncthreads();
}

// Octant-order position of stage index e (bisection over the bucket table).
__device__ __forceinline__ uint32_t stage_pos(const BlockIdx& bi, uint32_t e) {
    int lo = 0, hi = 64;
#pragma unroll
    for (int it = 0; it < 6; it++) {
        const int mid = (lo + hi) >> 1;
        if (bi.start[mid] <= e) lo = mid;
        else hi = mid;
    }
    return bi.kbeg[lo] + (e - bi.start[lo]);
}

// The nine stage runs of a member with octant oc: run r covers subcells
// (x-1..x+1) of row (y', z').
struct Runs {
    int a, zc, yb;
    __device__ __forceinline__ explicit Runs(uint32_t oc)
        : a(1 + (int)(oc & 1u)), zc(1 + (int)((oc >> 1) & 1u)), yb(1 + (int)(oc >> 2)) {}
    __device__ __forceinline__ void bounds(const BlockIdx& bi, int r, uint32_t& e0, uint32_t& e1) const {
        const int yy = yb - 1 + r / 3, zz = zc - 1 + r % 3;
        const int row = (yy * 4 + zz) * 4;
        e0 = bi.start[row + a - 1];
        e1 = bi.start[row + a + 2];
    }
};

// Density of one member with candidates from the octant order in global memory
// and a slot list (the octant-order kernel's method), for blocks too large to stage.
__device__ void density_global(const DevParams& P, const DevBuffers& B, uint32_t s, const float4 pi, float rho0,
                               uint32_t flag) {
    const float t[3] = {grid_t(pi.x, P.gmin[0], P.fac[0]), grid_t(pi.y, P.gmin[1], P.fac[1]),
                        grid_t(pi.z, P.gmin[2], P.fac[2])};
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int g2 = 2 * __float2int_rz(t[a]);
        const float u = 2.f * t[a];
        const float R = 2.f * P.srad[a];
        lo[a] = max(g2 - 2, __float2int_rd(u - R));
        hi[a] = min(g2 + 3, __float2int_rd(u + R));
    }
    Kahan sum;
    uint32_t cnt = 0;
    uint32_t* __restrict__ col = B.nbr + s;
    const size_t cap = (size_t)P.cap;
    for (int hy = lo[1]; hy <= hi[1]; hy++) {
        const int cy = hy >> 1, oy = hy & 1;
        for (int hz = lo[2]; hz <= hi[2]; hz++) {
            const int cz = hz >> 1, oz = hz & 1;
            const int rowc = (cy * P.rz + cz) * P.rx;
            for (int cx = lo[0] >> 1; cx <= (hi[0] >> 1); cx++) {
                const uint32_t c = (uint32_t)(rowc + cx);
                const uint32_t ce = __ldg(&B.cstart[c + 1]);
                if (__ldg(&B.cstart[c]) == ce) continue;
                const int oxlo = max(lo[0] - 2 * cx, 0), oxhi = min(hi[0] - 2 * cx, 1);
                const int bq = (oy * 2 + oz) * 2;
                const uint32_t k0 = __ldg(&B.oct_start[(size_t)c * 8 + bq + oxlo]);
                const uint32_t k1 = (bq + oxhi == 7) ? ce : __ldg(&B.oct_start[(size_t)c * 8 + bq + oxhi + 1]);
                float part = 0.f;
                for (uint32_t k = k0; k < k1; k++) {
                    const float4 pj = __ldg(&B.pos4o[k]);
                    const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
                    const float dsq = dx * dx + dy * dy + dz * dz;
                    const float cc = P.r2 - dsq;
                    const float m = pj.w > 0.f ? pj.w : rho0 * (-pj.w);
                    part = fmaf(dsq < P.r2 ? cc * cc * cc : 0.f, m, part);
                    const bool lst = dsq > 0.f && dsq < P.r2list;
                    if (lst && cnt < (uint32_t)kMaxNbr) col[cnt * cap] = __ldg(&B.oidx[k]);
                    cnt += lst ? 1u : 0u;
                }
                sum.add(part);
            }
        }
    }
    B.nbr_cnt[s] = cnt | flag;
    B.densp[s] = density_result(P, sum.s, rho0);
}

// ---------------------------------------------------------------------------
// Density + EOS
// ---------------------------------------------------------------------------

template <bool SS1>
__global__ void __launch_bounds__(kBlk) k_density_blk(const __grid_constant__ DevParams P,
                                                      const __grid_constant__ DevBuffers B,
                                                      const float4* __restrict__ alpha4) {
    __shared__ BlockIdx bi;
    __shared__ float4 sp[kStageDens];
    const uint32_t nact = *B.act_n;
    const float r2 = P.r2, r2list = P.r2list, ss = P.ss;
    const size_t cap = (size_t)P.cap;
    for (uint32_t ci = blockIdx.x; ci < nact; ci += gridDim.x) {
        const uint32_t c = B.act[ci];
        block_setup(P, B, c, bi);
        const uint32_t T = bi.start[64];
        const bool staged = T <= (uint32_t)kStageDens;
        if (staged)
            for (uint32_t e = threadIdx.x; e < T; e += kBlk) sp[e] = __ldg(&B.pos4o[stage_pos(bi, e)]);
        __syncthreads();
        const uint32_t cs = B.cstart[c], ce = B.cstart[c + 1];
        for (uint32_t o = cs + threadIdx.x; o < ce; o += kBlk) {
            const uint32_t s = B.oidx[o];
            const float4 pi = B.pos4o[o];
            if (pi.w < 0.f) {  // boundary: carries its volume, no pressure, needs no list
                B.densp[s] = make_float2(-pi.w, 0.f);
                B.nbr_cnt[s] = 0;
                continue;
            }
            const float rho0 = alpha4[s].w;
            if (!staged) {
                density_global(P, B, s, pi, rho0, kListGlobal);
                continue;
            }
            const Runs runs(octant_of(P, pi));
            Kahan sum;
            uint32_t cnt = 0;
            uint16_t* __restrict__ col = B.nbr16 + s;
            for (int r = 0; r < 9; r++) {
                uint32_t e0, e1;
                runs.bounds(bi, r, e0, e1);
                float part = 0.f;
                for (uint32_t e = e0; e < e1; e++) {
                    const float4 pj = sp[e];
                    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                    if (!SS1) { dx *= ss; dy *= ss; dz *= ss; }
                    const float dsq = dx * dx + dy * dy + dz * dz;
                    const float cc = r2 - dsq;
                    const float m = pj.w > 0.f ? pj.w : rho0 * (-pj.w);
                    part = fmaf(dsq < r2 ? cc * cc * cc : 0.f, m, part);
                    const bool lst = dsq > 0.f && dsq < r2list;
                    if (lst && cnt < (uint32_t)kMaxNbr) col[cnt * cap] = (uint16_t)e;
                    cnt += lst ? 1u : 0u;
                }
                sum.add(part);
            }
            B.nbr_cnt[s] = cnt;
            B.densp[s] = density_result(P, sum.s, rho0);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Force + drift velocity
// ---------------------------------------------------------------------------

template <bool FORCE, bool DRIFT, int NP>
__global__ void __launch_bounds__(kBlk) k_force_blk(const __grid_constant__ DevParams P,
                                                    const __grid_constant__ DevBuffers B,
                                                    const float4* __restrict__ pos4,
                                                    const float4* __restrict__ vel4,
                                                    const float4* __restrict__ alpha4,
                                                    const float4* __restrict__ aprev4) {
    extern __shared__ float4 dyn[];
    float4* sp = dyn;
    float4* sv = sp + kStageForce;
    float4* sa = sv + kStageForce;
    float2* sdp = reinterpret_cast<float2*>(sa + kStageForce);
    __shared__ BlockIdx bi;
    const uint32_t nact = *B.act_n;
    const size_t cap = (size_t)P.cap;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint32_t ci = blockIdx.x; ci < nact; ci += gridDim.x) {
        const uint32_t c = B.act[ci];
        block_setup(P, B, c, bi);
        const uint32_t T = bi.start[64];
        const bool staged = T <= (uint32_t)kStageForce;
        if (staged) {
            for (uint32_t e = threadIdx.x; e < T; e += kBlk) {
                const uint32_t k = stage_pos(bi, e);
                const uint32_t j = __ldg(&B.oidx[k]);
                sp[e] = __ldg(&B.pos4o[k]);
                sdp[e] = __ldg(&B.densp[j]);
                if (FORCE) sv[e] = __ldg(&vel4[j]);
                if (DRIFT) sa[e] = __ldg(&alpha4[j]);
            }
        }
        __syncthreads();
        const uint32_t cs = B.cstart[c], ce = B.cstart[c + 1];
        for (uint32_t o = cs + threadIdx.x; o < ce; o += kBlk) {
            const uint32_t s = B.oidx[o];
            const float4 pi = B.pos4o[o];
            if (pi.w < 0.f) {
                if (FORCE) B.accel4[s] = zero4;
                continue;
            }
            ForceDrift<FORCE, DRIFT, NP> acc;
            acc.init(P, pi, vel4[s], B.densp[s], alpha4[s]);
            const uint32_t raw = B.nbr_cnt[s];
            auto global_pair = [&](uint32_t j) {
                acc.pair(P, __ldg(&pos4[j]), __ldg(&B.densp[j]), FORCE ? __ldg(&vel4[j]) : zero4,
                         DRIFT ? __ldg(&alpha4[j]) : zero4);
            };
            if ((raw & kListGlobal) || raw > (uint32_t)kMaxNbr) {
                for_slot_list(P, B, s, pi.x, pi.y, pi.z, global_pair);
            } else if (staged) {
                const uint16_t* __restrict__ col = B.nbr16 + s;
#pragma unroll 2
                for (uint32_t k = 0; k < raw; k++) {
                    const uint32_t e = col[k * cap];
                    acc.pair(P, sp[e], sdp[e], FORCE ? sv[e] : zero4, DRIFT ? sa[e] : zero4);
                }
            } else {
                const uint16_t* __restrict__ col = B.nbr16 + s;
                for (uint32_t k = 0; k < raw; k++) global_pair(__ldg(&B.oidx[stage_pos(bi, col[k * cap])]));
            }
            acc.finish(P, B, s, DRIFT ? aprev4[s] : zero4);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Alpha advance + correction + advance
// ---------------------------------------------------------------------------

// MODE 0: advance only; 1: alpha advance + correction + advance (all five float4
// fields to S.out); 2: alpha advance only (fractions to S.out[ALPHA]).
template <int NP, int MODE>
__global__ void __launch_bounds__(kBlk) k_pass_c_blk(const __grid_constant__ DevParams P,
                                                     const __grid_constant__ DevBuffers B,
                                                     const __grid_constant__ F4Set S) {
    extern __shared__ float4 dyn[];
    float4* sp = dyn;
    float4* sve = sp + kStagePassC;
    float4* sa = sve + kStagePassC;
    float4* su = sa + kStagePassC;                                   // NP * kStagePassC, phase-major
    float* smd = reinterpret_cast<float*>(su + NP * kStagePassC);   // mass * (1/rho), 0 for boundary
    __shared__ BlockIdx bi;
    const uint32_t nact = *B.act_n;
    const size_t cap = (size_t)P.cap;
    constexpr bool MP = MODE != 0;
    for (uint32_t ci = blockIdx.x; ci < nact; ci += gridDim.x) {
        const uint32_t c = B.act[ci];
        bool staged = false;
        if (MP) {
            block_setup(P, B, c, bi);
            const uint32_t T = bi.start[64];
            staged = T <= (uint32_t)kStagePassC;
            if (staged) {
                for (uint32_t e = threadIdx.x; e < T; e += kBlk) {
                    const uint32_t k = stage_pos(bi, e);
                    const uint32_t j = __ldg(&B.oidx[k]);
                    const float4 p = __ldg(&B.pos4o[k]);
                    sp[e] = p;
                    smd[e] = p.w > 0.f ? p.w * __ldg(&B.densp[j]).x : 0.f;
                    sve[e] = __ldg(&S.in[VEV][j]);
                    sa[e] = __ldg(&S.in[ALPHA][j]);
#pragma unroll
                    for (int q = 0; q < NP; q++) su[q * kStagePassC + e] = __ldg(&B.drift4[(size_t)q * cap + j]);
                }
            }
            __syncthreads();
        }
        const uint32_t cs = B.cstart[c], ce = B.cstart[c + 1];
        for (uint32_t o = cs + threadIdx.x; o < ce; o += kBlk) {
            const uint32_t s = B.oidx[o];
            float4 p = S.in[POS][s], v = S.in[VEL][s], ve = S.in[VEV][s], al = S.in[ALPHA][s], ap = S.in[APREV][s];
            const float4 pi = p, vei = ve, ai = al;
            auto alpha_sum = [&](float (&a)[3]) {
                float3 um[NP];
#pragma unroll
                for (int q = 0; q < NP; q++) {
                    const float4 u = B.drift4[(size_t)q * cap + s];
                    um[q] = make_float3(u.x, u.y, u.z);
                }
                AlphaChange<NP> acc;
                acc.init(pi, vei, ai, um);
                auto global_pair = [&](uint32_t j) {
                    const float4 pj = __ldg(&S.in[POS][j]);
                    const float2 dpj = __ldg(&B.densp[j]);
                    float4 uj[NP];
#pragma unroll
                    for (int q = 0; q < NP; q++) uj[q] = __ldg(&B.drift4[(size_t)q * cap + j]);
                    acc.pair(P, pj, pj.w * dpj.x, __ldg(&S.in[VEV][j]), __ldg(&S.in[ALPHA][j]), uj);
                };
                const uint32_t raw = B.nbr_cnt[s];
                if ((raw & kListGlobal) || raw > (uint32_t)kMaxNbr) {
                    for_slot_list(P, B, s, pi.x, pi.y, pi.z, global_pair);
                } else if (staged) {
                    const uint16_t* __restrict__ col = B.nbr16 + s;
#pragma unroll 2
                    for (uint32_t k = 0; k < raw; k++) {
                        const uint32_t e = col[k * cap];
                        float4 uj[NP];
#pragma unroll
                        for (int q = 0; q < NP; q++) uj[q] = su[q * kStagePassC + e];
                        acc.pair(P, sp[e], smd[e], sve[e], sa[e], uj);
                    }
                } else {
                    const uint16_t* __restrict__ col = B.nbr16 + s;
                    for (uint32_t k = 0; k < raw; k++) global_pair(__ldg(&B.oidx[stage_pos(bi, col[k * cap])]));
                }
                acc.result(P, a);
            };
            if (MODE == 2) {
                if (!(p.w < 0.f)) {
                    float a[3] = {al.x, al.y, al.z};
                    alpha_sum(a);
                    al = make_float4(a[0], a[1], a[2], al.w);
                }
                S.out[ALPHA][s] = al;
            } else {
                pass_c_slot<NP, MP>(P, B, s, false, p, v, ve, al, ap, alpha_sum);
                S.out[POS][s] = p;
                S.out[VEL][s] = v;
                S.out[VEV][s] = ve;
                S.out[ALPHA][s] = al;
                S.out[APREV][s] = ap;
            }
        }
        if (MP) __syncthreads();
    }
}

// The out-of-grid slots [n_in, n): parked by the advance (or copied for MODE 2).
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_pass_c_undef(const __grid_constant__ DevParams P,
                                                           const __grid_constant__ DevBuffers B,
                                                           const __grid_constant__ F4Set S) {
    const uint32_t s = B.cstart[P.G] + blockIdx.x * kThreads + threadIdx.x;
    if (s >= (uint32_t)P.n) return;
    float4 p = S.in[POS][s], v = S.in[VEL][s], ve = S.in[VEV][s], al = S.in[ALPHA][s], ap = S.in[APREV][s];
    if (MODE == 2) {
        S.out[ALPHA][s] = al;
        return;
    }
    pass_c_slot<1, false>(P, B, (int)s, true, p, v, ve, al, ap, [](float (&)[3]) {});
    S.out[POS][s] = p;
    S.out[VEL][s] = v;
    S.out[VEV][s] = ve;
    S.out[ALPHA][s] = al;
    S.out[APREV][s] = ap;
}

// Resident CTAs of kernel K on all SMs (one instance per kernel, computed once;
// raises the dynamic shared-memory limit first when the kernel needs more than 48 KB).
template <auto K>
int grid_for(size_t dyn_smem) {
    static int cached = 0;
    if (!cached) {
        if (dyn_smem > 48 * 1024)
            cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_smem);
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, K, kBlk, dyn_smem);
        cached = (per > 0 ? per : 1) * (sms > 0 ? sms : 1);
    }
    return cached;
}

F4Set set_of(const DevBuffers& B, const int* cur) {
    F4Set S;
    for (int f = 0; f < kNumFloat4Fields; f++) {
        S.in[f] = B.f4[f][cur[f]];
        S.out[f] = B.f4[f][cur[f] ^ 1];
    }
    return S;
}

template <bool F, bool D, int NP>
void force_blk(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    const size_t smem = (size_t)kStageForce * (3 * sizeof(float4) + sizeof(float2));
    k_force_blk<F, D, NP><<<grid_for<k_force_blk<F, D, NP>>(smem), kBlk, smem, s>>>(P, B, B.f4[POS][cur[POS]], B.f4[VEL][cur[VEL]], B.f4[ALPHA][cur[ALPHA]],
                                             B.f4[APREV][cur[APREV]]);
}

template <int NP, int MODE>
void pass_c_blk(const DevParams& P, const DevBuffers& B, const F4Set& S, cudaStream_t s) {
    const size_t smem = MODE == 0 ? 0 : (size_t)kStagePassC * ((3 + NP) * sizeof(float4) + sizeof(float));
    k_pass_c_blk<NP, MODE><<<grid_for<k_pass_c_blk<NP, MODE>>(smem), kBlk, smem, s>>>(P, B, S);
    k_pass_c_undef<MODE><<<(P.n + kThreads - 1) / kThreads, kThreads, 0, s>>>(P, B, S);
}

}  // namespace

void launch_density_blk(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    if (P.ss == 1.f)
        k_density_blk<true><<<grid_for<k_density_blk<true>>(0), kBlk, 0, s>>>(P, B, B.f4[ALPHA][cur[ALPHA]]);
    else
        k_density_blk<false><<<grid_for<k_density_blk<false>>(0), kBlk, 0, s>>>(P, B, B.f4[ALPHA][cur[ALPHA]]);
}

void launch_force_drift_blk(const DevParams& P, const DevBuffers& B, const int* cur, bool force, bool drift,
                            cudaStream_t s) {
    if (P.n <= 0 || (!force && !drift)) return;
    if (force && !drift) return force_blk<true, false, 0>(P, B, cur, s);
    const int np = P.nphase;
    if (force) {
        if (np == 1) force_blk<true, true, 1>(P, B, cur, s);
        else if (np == 2) force_blk<true, true, 2>(P, B, cur, s);
        else force_blk<true, true, 3>(P, B, cur, s);
    } else {
        if (np == 1) force_blk<false, true, 1>(P, B, cur, s);
        else if (np == 2) force_blk<false, true, 2>(P, B, cur, s);
        else force_blk<false, true, 3>(P, B, cur, s);
    }
}

void launch_pass_c_blk(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    const F4Set S = set_of(B, cur);
    if (!P.multiphase) return pass_c_blk<1, 0>(P, B, S, s);
    if (P.nphase == 1) pass_c_blk<1, 1>(P, B, S, s);
    else if (P.nphase == 2) pass_c_blk<2, 1>(P, B, S, s);
    else pass_c_blk<3, 1>(P, B, S, s);
}

void launch_alpha_advance_blk(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    // only the alpha buffers flip; the other fields are read from cur and written nowhere
    F4Set S = set_of(B, cur);
    if (P.nphase == 1) pass_c_blk<1, 2>(P, B, S, s);
    else if (P.nphase == 2) pass_c_blk<2, 2>(P, B, S, s);
    else pass_c_blk<3, 2>(P, B, S, s);
}

}  // namespace sphmp
