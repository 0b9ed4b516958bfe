// sphmp_kernels.cu — CUDA kernels of the multiphase SPH step for sm_103a.
//
// Reference parity notes (ZP-Z/sph-multiphase):
//  * the hash reproduces InitialSort (SPH_Solver/fluids/fluid_system_kern.cu:36-64)
//    with the same float operations, so cell ids are bit-identical;
//  * the sort reproduces thrust::sort_by_key's stable order (fluid_system_host.cu:164-166)
//    by ranking every cell's members by their pre-sort slot, and also builds the
//    internal order of the particle state (cells as sorted, members grouped by
//    h-subcell inside each cell);
//  * neighbour sums follow the reference formulas (fluid_system_kern.cu:183-424,
//    multiphase.cu:19-349) in FP32 over the pairs closer than h, found by the
//    bucket density kernel (one warp per h-subcell, the 27 h-subcells around it)
//    and kept as index lists for the force, drift and volume-fraction passes;
//  * the advance reproduces AdvanceParticles (fluid_system_kern.cu:426-534) with
//    un-contracted float operations, so it is bit-identical given the same accel.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "sphmp_device.cuh"
#include "sphmp_features.cuh"
#include "sphmp_emit.h"
#include "sphmp_internal.h"

namespace sphmp {

namespace {

using namespace dev;

// ---------------------------------------------------------------------------
// Hash + histogram (GetParticleIndexCUDA)
// ---------------------------------------------------------------------------

// One block = one chunk of kHashBlock slots. In-grid slots take a rank inside
// their cell from a warp-aggregated atomic (the order is fixed later by the
// cell sort); out-of-grid slots get their exact rank inside the chunk, and the
// chunk totals are scanned later, which places them in slot order.
__global__ void __launch_bounds__(kHashBlock) k_hash(const __grid_constant__ DevParams P,
                                                     const __grid_constant__ DevBuffers B,
                                                     const float4* __restrict__ pos4) {
    __shared__ uint32_t wcount[kHashBlock / 32];
    const int i = blockIdx.x * kHashBlock + threadIdx.x;
    const bool valid = i < active_n(B);
    uint32_t key = kUndef;
    if (valid) {
        const float4 p = pos4[B.opos[i]];
        key = cell_key(P, p.x, p.y, p.z);
        B.key[i] = key;
        B.mgcell[i] = key;
        if (key != kUndef) B.octk[i] = (uint8_t)octant_of(P, p);  // for the per-cell octant order
    }
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const bool und = valid && key == kUndef;
    const unsigned ub = __ballot_sync(0xffffffffu, und);
    if (lane == 0) wcount[warp] = __popc(ub);
    __syncthreads();
    if (warp == 0) {
        constexpr int nw = kHashBlock / 32;
        uint32_t v = lane < nw ? wcount[lane] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if ((int)lane >= o) x += y;
        }
        if ((int)lane < nw) wcount[lane] = x - v;
        if ((int)lane == nw - 1) B.uchunk[blockIdx.x] = x;
    }
    __syncthreads();
    if (und) B.arank[i] = wcount[warp] + __popc(ub & lanemask_lt());
    const bool in = valid && key != kUndef;
    const unsigned im = __ballot_sync(0xffffffffu, in);
    if (in) {
        const unsigned peers = __match_any_sync(im, key);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(&B.ccount[key], (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        B.arank[i] = base + __popc(peers & lanemask_lt());
    }
}

// ---------------------------------------------------------------------------
// Prefix sums (GetGridListCUDA, part 1)
// ---------------------------------------------------------------------------

// Exclusive scan of one value per thread across a 1024-thread block.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t ws[32];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if ((int)lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if ((int)lane >= o) w += y;
        }
        ws[lane] = w;
    }
    __syncthreads();
    const uint32_t off = warp ? ws[warp - 1] : 0u;
    *total = ws[31];
    __syncthreads();
    return off + x - v;
}

__device__ __forceinline__ void load4(const uint32_t* in, int len, int idx, uint32_t v[4]) {
    if (idx + 3 < len && ((reinterpret_cast<uintptr_t>(in + idx) & 15u) == 0)) {
        const uint4 q = *reinterpret_cast<const uint4*>(in + idx);
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = (idx + k < len) ? in[idx + k] : 0u;
    }
}

// Counts of the cells at scan positions idx .. idx + 3: cell = position in the
// linear order, corder[position] in the Morton order.
__device__ __forceinline__ void load4_cells(const DevParams& P, const DevBuffers& B, int idx, uint32_t v[4]) {
    if (!P.morton) {
        load4(B.ccount, P.G, idx, v);
        return;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = idx + k < P.G ? B.ccount[B.corder[idx + k]] : 0u;
}

// Phase A: block sums of the cell histogram.
__global__ void __launch_bounds__(kScanBlock) k_scan_reduce(const __grid_constant__ DevParams P,
                                                            const __grid_constant__ DevBuffers B) {
    const int idx = (blockIdx.x * kScanBlock + threadIdx.x) * kScanItems;
    uint32_t v[4];
    load4_cells(P, B, idx, v);
    uint32_t total;
    block_excl_scan(v[0] + v[1] + v[2] + v[3], &total);
    if (threadIdx.x == 0) B.bsum[blockIdx.x] = total;
}

// Phase B: one block scans the block sums and the out-of-grid chunk counts.
__global__ void __launch_bounds__(kScanBlock) k_scan_top(const __grid_constant__ DevParams P,
                                                         const __grid_constant__ DevBuffers B, int nblocks,
                                                         int nchunks) {
    uint32_t carry = 0;
    for (int base = 0; base < nblocks; base += kScanBlock) {
        const int k = base + threadIdx.x;
        const uint32_t v = k < nblocks ? B.bsum[k] : 0u;
        uint32_t total;
        const uint32_t e = block_excl_scan(v, &total);
        if (k < nblocks) B.bsum[k] = carry + e;
        carry += total;
    }
    const uint32_t nin = carry;
    carry = 0;
    for (int base = 0; base < nchunks; base += kScanBlock) {
        const int k = base + threadIdx.x;
        const uint32_t v = k < nchunks ? B.uchunk[k] : 0u;
        uint32_t total;
        const uint32_t e = block_excl_scan(v, &total);
        if (k < nchunks) B.uchunk[k] = carry + e;
        carry += total;
    }
    if (threadIdx.x == 0) {
        B.cstart[P.G] = nin;
        B.cstart[P.G + 1] = (uint32_t)active_n(B);
        B.big[0] = 0u;
        *B.act_n = 0u;
        *B.wq_n = 0u;
        *B.hq_n = 0u;
    }
}

// Phase C: cell starts, the reference's mgridoff / mgridcnt, and the list of
// cells too large for the warp sort.
__global__ void __launch_bounds__(kScanBlock) k_scan_apply(const __grid_constant__ DevParams P,
                                                           const __grid_constant__ DevBuffers B) {
    const int idx = (blockIdx.x * kScanBlock + threadIdx.x) * kScanItems;
    uint32_t v[4];
    load4_cells(P, B, idx, v);
    uint32_t total;
    uint32_t run = B.bsum[blockIdx.x] + block_excl_scan(v[0] + v[1] + v[2] + v[3], &total);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (idx + k < P.G) {
            const int c = P.morton ? (int)B.corder[idx + k] : idx + k;
            B.cstart[c] = run;
            B.cend[c] = run + v[k];
            B.mgridoff[c] = v[k] ? (int32_t)run : 0;
            B.mgridcnt[c] = (int32_t)v[k];
            if (v[k]) B.act[atomicAdd(B.act_n, 1u)] = (uint32_t)c;
            if (v[k] > (uint32_t)kWarpSortMax) {
                if (v[k] > (uint32_t)kCtaSortMax) {
                    set_err(B, kErrCellOverflow);  // left unsorted; keep its octant ranges in bounds
                    for (int b = 0; b < 8; b++) B.oct_start[(size_t)c * 8 + b] = run;
                } else {
                    const uint32_t slot = atomicAdd(&B.big[0], 1u);
                    B.big[1 + slot] = (uint32_t)c;
                }
            }
        }
        run += v[k];
    }
}

// ---------------------------------------------------------------------------
// Scatter + per-cell stable order (GetGridListCUDA, part 2)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kThreads) k_scatter(const __grid_constant__ DevParams P,
                                                      const __grid_constant__ DevBuffers B) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= active_n(B)) return;
    const uint32_t key = B.key[i];
    const uint32_t r = B.arank[i];
    if (key != kUndef) {
        B.sidx[B.cstart[key] + r] = (uint32_t)i;
    } else {
        const uint32_t d = B.cstart[P.G] + B.uchunk[i / kHashBlock] + r;
        B.midsort[d] = (uint32_t)i;
        B.mgcell[d] = kUndef;
        B.mgndx[d] = kUndef;
        B.osrc[d] = B.opos[i];  // out-of-grid particles keep slot order at the end
        B.oidx[d] = d;
    }
}

// Bitonic sort of 32*E keys held E per lane (element index = lane*E + r),
// ascending, entirely in registers.
template <int E>
__device__ __forceinline__ void warp_bitonic(uint32_t (&v)[E]) {
    const unsigned lane = lane_id();
    constexpr int M = 32 * E;
#pragma unroll
    for (int k = 2; k <= M; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= E) {
                const int lj = j / E;
#pragma unroll
                for (int r = 0; r < E; r++) {
                    const uint32_t o = __shfl_xor_sync(0xffffffffu, v[r], lj);
                    const unsigned idx = lane * E + r;
                    const bool asc = (idx & k) == 0;
                    const bool lower = (idx & j) == 0;
                    const uint32_t mn = min(v[r], o), mx = max(v[r], o);
                    v[r] = (lower == asc) ? mn : mx;
                }
            } else {
#pragma unroll
                for (int r = 0; r < E; r++) {
                    const int p = r ^ j;
                    if (p > r) {
                        const unsigned idx = lane * E + r;
                        const bool asc = (idx & k) == 0;
                        const uint32_t a = v[r], b = v[p];
                        const bool sw = asc ? (a > b) : (a < b);
                        v[r] = sw ? b : a;
                        v[p] = sw ? a : b;
                    }
                }
            }
        }
    }
}

// Write the internal order of cell c from the key (octant << shift | member index)
// held at sorted position q (cellstart + q is its internal index): the member's
// previous internal index (osrc), its slot (oidx) and the bucket starts.
__device__ __forceinline__ void emit_octant(const DevBuffers& B, uint32_t c, uint32_t start, uint32_t cnt, uint32_t q,
                                            uint32_t key, uint32_t prev_oct, int shift, uint32_t pre_slot,
                                            uint32_t* bst = nullptr) {
    const uint32_t oct = key >> shift;
    const uint32_t idx = key & ((1u << shift) - 1u);
    if (q < cnt) {
        B.osrc[start + q] = B.opos[pre_slot];
        B.oidx[start + q] = start + idx;
    }
    // bucket starts: every bucket in (prev_oct, oct] begins at q (8 marks past the end)
    const uint32_t hi = q < cnt ? oct : 8u;
    for (uint32_t b = prev_oct + 1; b <= hi && b < 8; b++) {
        B.oct_start[(size_t)c * 8 + b] = start + q;
        if (bst) bst[b] = start + q;
    }
    if (q == cnt - 1)
        for (uint32_t b = oct + 1; b < 8; b++) {
            B.oct_start[(size_t)c * 8 + b] = start + cnt;
            if (bst) bst[b] = start + cnt;
        }
}

// Queue the member windows after the first of bucket (c, b) = members [m0, m1)
// for the density pass (one warp per window of P.bwin members).
__device__ __forceinline__ void push_windows(const DevParams& P, const DevBuffers& B, uint32_t c, uint32_t b,
                                             uint32_t m0, uint32_t m1) {
    const uint32_t W = (uint32_t)P.bwin;
    if (m1 <= m0 + W) return;
    const uint32_t nw = (m1 - m0 - 1) / W;  // <= (m1 - m0) / kBucketWindowMin: wq never overflows
    const uint32_t base = atomicAdd(B.wq_n, nw);
    for (uint32_t i = 0; i < nw; i++) B.wq[base + i] = make_uint2(c * 8u + b, m0 + (i + 1) * W);
}

template <int E>
__device__ __forceinline__ void warp_sort_cell(const DevParams& P, const DevBuffers& B, const float4* __restrict__ pos_in,
                                               uint32_t* wsm, uint32_t* bst, uint32_t c, uint32_t start, uint32_t cnt) {
    uint32_t v[E];
    const unsigned lane = lane_id();
#pragma unroll
    for (int r = 0; r < E; r++) {
        const uint32_t idx = lane * E + r;
        v[r] = idx < cnt ? B.sidx[start + idx] : 0xFFFFFFFFu;
    }
    warp_bitonic<E>(v);
    // stable order: pre-sort slots ascending
    uint32_t key[E];
#pragma unroll
    for (int r = 0; r < E; r++) {
        const uint32_t idx = lane * E + r;
        wsm[idx] = v[r];
        key[r] = 0xFFFFFFFFu;
        if (idx < cnt) {
            B.midsort[start + idx] = v[r];
            B.mgcell[start + idx] = c;
            B.mgndx[start + idx] = idx;
            key[r] = ((uint32_t)B.octk[v[r]] << 8) | idx;
        }
    }
    // octant order: sort (octant, member index)
    warp_bitonic<E>(key);
    __syncwarp();
    const uint32_t last_prev = __shfl_up_sync(0xffffffffu, key[E - 1], 1);
#pragma unroll
    for (int r = 0; r < E; r++) {
        const uint32_t q = lane * E + r;
        const uint32_t pk = r > 0 ? key[r - 1] : (lane > 0 ? last_prev : 0xFFFFFFFFu);
        const uint32_t prev_oct = (q == 0) ? 0xFFFFFFFFu : (pk == 0xFFFFFFFFu ? 8u : pk >> 8);
        if (q <= cnt) {
            const uint32_t k = key[r];
            const uint32_t pre = q < cnt ? wsm[k & 255u] : 0u;
            emit_octant(B, c, start, cnt, q, q < cnt ? k : (8u << 8), prev_oct, 8, pre, bst);
        }
    }
    __syncwarp();  // the bucket starts in bst are visible to the whole warp
    if (lane < 8 && cnt > (uint32_t)P.bwin) {
        const uint32_t b0 = bst[lane];
        const uint32_t b1 = lane == 7 ? start + cnt : bst[lane + 1];
        push_windows(P, B, c, lane, b0, b1);
    }
    __syncwarp();
}

// One warp per cell (cells of up to kWarpSortMax members).
// Six blocks per SM (at most 40 registers): the warps' dependent load chains
// overlap; the large-cell paths spill a little (cell order 0.071 -> 0.066 ms per
// step on the 2^20-particle scene; 77 registers without the bound).
__global__ void __launch_bounds__(kThreads, 6) k_cell_sort(const __grid_constant__ DevParams P,
                                                        const __grid_constant__ DevBuffers B,
                                                        const float4* __restrict__ pos_in) {
    __shared__ uint32_t sm[kThreads / 32][kWarpSortMax];
    __shared__ uint32_t bs[kThreads / 32][8];  // the bucket starts of the warp's current cell
    uint32_t* wsm = sm[threadIdx.x >> 5];
    uint32_t* bst = bs[threadIdx.x >> 5];
    const int nwarps = (gridDim.x * kThreads) >> 5;
    const uint32_t nact = *B.act_n;  // the occupied cells, listed by the scan
    for (uint32_t a = (blockIdx.x * kThreads + threadIdx.x) >> 5; a < nact; a += (uint32_t)nwarps) {
        const uint32_t c = B.act[a];
        const uint32_t start = B.cstart[c];
        const uint32_t cnt = B.cend[c] - start;
        if (cnt == 0 || cnt > (uint32_t)kWarpSortMax) continue;
        if (cnt <= 32) warp_sort_cell<1>(P, B, pos_in, wsm, bst, c, start, cnt);
        else if (cnt <= 64) warp_sort_cell<2>(P, B, pos_in, wsm, bst, c, start, cnt);
        else if (cnt <= 128) warp_sort_cell<4>(P, B, pos_in, wsm, bst, c, start, cnt);
        else warp_sort_cell<8>(P, B, pos_in, wsm, bst, c, start, cnt);
    }
}

__device__ __forceinline__ void cta_bitonic(uint32_t* sm, uint32_t M) {
    for (uint32_t k = 2; k <= M; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t t = threadIdx.x; t < M; t += blockDim.x) {
                const uint32_t p = t ^ j;
                if (p > t) {
                    const bool asc = (t & k) == 0;
                    const uint32_t a = sm[t], q = sm[p];
                    if (asc ? (a > q) : (a < q)) { sm[t] = q; sm[p] = a; }
                }
            }
            __syncthreads();
        }
    }
}

// One CTA per large cell (kWarpSortMax < members <= kCtaSortMax): bitonic sorts in shared memory.
__global__ void __launch_bounds__(1024) k_big_cell_sort(const __grid_constant__ DevParams P,
                                                        const __grid_constant__ DevBuffers B,
                                                        const float4* __restrict__ pos_in) {
    __shared__ uint32_t sm[kCtaSortMax];
    const uint32_t nbig = B.big[0];
    for (uint32_t b = blockIdx.x; b < nbig; b += gridDim.x) {
        const uint32_t c = B.big[1 + b];
        const uint32_t start = B.cstart[c];
        const uint32_t cnt = B.cend[c] - start;
        uint32_t M = 1;
        while (M < cnt) M <<= 1;
        for (uint32_t k = threadIdx.x; k < M; k += blockDim.x) sm[k] = k < cnt ? B.sidx[start + k] : 0xFFFFFFFFu;
        __syncthreads();
        cta_bitonic(sm, M);
        for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
            B.midsort[start + k] = sm[k];
            B.mgcell[start + k] = c;
            B.mgndx[start + k] = k;
        }
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < M; k += blockDim.x)
            sm[k] = k < cnt ? (((uint32_t)B.octk[B.midsort[start + k]] << 13) | k) : 0xFFFFFFFFu;
        __syncthreads();
        cta_bitonic(sm, M);
        for (uint32_t q = threadIdx.x; q <= cnt && q < M + 1; q += blockDim.x) {
            const uint32_t k = q < cnt ? sm[q] : (8u << 13);
            const uint32_t pk = q == 0 ? 0xFFFFFFFFu : sm[q - 1];
            const uint32_t prev_oct = q == 0 ? 0xFFFFFFFFu : (pk >> 13);
            const uint32_t pre = q < cnt ? B.midsort[start + (k & 0x1FFFu)] : 0u;
            emit_octant(B, c, start, cnt, q, k, prev_oct, 13, pre);
        }
        __syncthreads();
        if (threadIdx.x < 8) {
            const uint32_t b0 = B.oct_start[(size_t)c * 8 + threadIdx.x];
            const uint32_t b1 = threadIdx.x == 7 ? start + cnt : B.oct_start[(size_t)c * 8 + threadIdx.x + 1];
            push_windows(P, B, c, threadIdx.x, b0, b1);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Reorder (RearrageDataCUDA)
// ---------------------------------------------------------------------------


// Every particle, out-of-grid ones included, moves to its new internal index
// (the reference gathers every slot: its `int cell != GRID_UNDEF` test at
// fluid_system_kern.cu:104-108 compares against a 64-bit literal on LP64 hosts
// and is always true there; out-of-grid particles are parked at (-1000)^3 by the
// advance), and the slot -> index map follows (no kernel reads opos between the
// cell order, which reads the old map, and this one).
__global__ void __launch_bounds__(kThreads) k_rearrange(const __grid_constant__ DevParams P,
                                                        const __grid_constant__ DevBuffers B,
                                                        const __grid_constant__ F4Set S) {
    const int o = blockIdx.x * kThreads + threadIdx.x;
    const int n = active_n(B);
    if (o >= n) return;
    uint32_t src = B.osrc[o];
    if (src >= (uint32_t)n) src = o;  // only after a cell-overflow error (flagged by the scan)
#pragma unroll
    for (int f = 0; f < kNumFloat4Fields; f++) S.out[f][o] = S.in[f][src];
    const uint32_t slot = B.oidx[o];
    if (slot < (uint32_t)n) B.opos[slot] = (uint32_t)o;
}

// New internal order = the sorted slot order (midsort given, no octant order).
__global__ void __launch_bounds__(kThreads) k_slot_order(const __grid_constant__ DevParams P,
                                                         const __grid_constant__ DevBuffers B) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B)) return;
    const uint32_t m = B.midsort[s];
    B.osrc[s] = m < (uint32_t)active_n(B) ? B.opos[m] : (uint32_t)s;
    B.oidx[s] = (uint32_t)s;
}

// ---------------------------------------------------------------------------
// Boundary volume (ComputeBoundaryDensity)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kThreads) k_boundary_volume(const __grid_constant__ DevParams P,
                                                              const __grid_constant__ DevBuffers B,
                                                              const float4* __restrict__ pos4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B) || B.mgcell[s] == kUndef) return;
    const float4 pi = pos4[s];
    if (!(pi.w < 0.f)) return;
    Kahan sum;
    for_candidates(P, B, B.mgcell[s], pi.x, pi.y, pi.z, [&](uint32_t j) {
        const float4 pj = __ldg(&pos4[j]);
        if (!(pj.w < 0.f)) return;
        const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
        const float dsq = dx * dx + dy * dy + dz * dz;
        if (dsq < P.r2) {
            const float c = P.r2 - dsq;
            sum.add(c * c * c);
        }
    });
    float v = sum.s * P.kpoly6;
    if (v == 0.f) v = 1.f;
    B.vtmp[s] = 1.f / v;
}

__global__ void __launch_bounds__(kThreads) k_boundary_volume_store(const __grid_constant__ DevParams P,
                                                                    const __grid_constant__ DevBuffers B,
                                                                    float4* __restrict__ pos4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B) || B.mgcell[s] == kUndef) return;
    float4 p = pos4[s];
    if (!(p.w < 0.f)) return;
    p.w = -B.vtmp[s];
    pos4[s] = p;
    B.densp[s] = make_float2(-p.w, 0.f);
}

// ---------------------------------------------------------------------------
// Density + EOS pressure (MfComputePressureCUDA)
// ---------------------------------------------------------------------------

// Density + EOS, one warp per octant bucket (the members of one h-subcell).
// Every member of a bucket has its neighbours within the 27 h-subcells around
// it: a pair closer than h is at most one subcell apart per axis, up to the
// rounding of the grid coordinate (a pair that rounding puts two subcells apart
// is within 1e-4 h of the cutoff, where the kernels and their gradients vanish
// to below 1e-7 of a typical term). The 27 subcells form 18 contiguous index
// ranges (per (y, z) row: the x-neighbour bucket in the adjacent cell and the
// two buckets of the same cell); their concatenation is the bucket's candidate
// sequence, recorded in btab. A warp takes one window of up to P.bwin (<= 32)
// members of a bucket (one member per lane, broadcast by shuffles) and the
// bucket's candidates in blocks of 32 * kBucketChunks held in registers, one
// per lane and chunk; for each block it walks the window's members, every lane
// testing its candidates against the member. The neighbour list of a member is
// the ballot of those tests, one mask word per 32 candidates, without the
// member itself. The density terms are non-negative; each lane sums at most
// kBucketChunks of them per block, the lanes are summed pairwise and the blocks
// with Kahan compensation (in the member's lane), so the relative rounding
// error of a member's sum stays below (kBucketChunks + 6) * 2^-24. Warps take
// work items from a shared counter (their costs differ by orders of magnitude):
// the first window of every bucket, then the further windows of large buckets,
// which the cell sort queued in wq, so that no bucket serialises on one warp.
// The candidate sequence of bucket (c, q): the 27 h-subcells around it as 18
// contiguous index ranges, two per (y, z) subcell row (the x-neighbour bucket in
// the adjacent cell, and both x buckets of the bucket's own cell column). Lane i
// < 18 computes range i; the warp scans the lengths. Range starts and sequence
// offsets go to the warp's shared table (offset[18] = length T); lane i < 18
// returns its range start and offset in st / off.
__device__ __forceinline__ uint32_t bucket_ranges(const DevParams& P, const DevBuffers& B, uint32_t c, uint32_t q,
                                                  unsigned lane, uint32_t* rstart, uint32_t* roff, uint32_t& st,
                                                  uint32_t& off) {
    const int cx = (int)(c % (uint32_t)P.rx);
    const int cyz = (int)(c / (uint32_t)P.rx);
    const int cz = cyz % P.rz, cy = cyz / P.rz;
    const int ox = (int)(q & 1u), oz = (int)((q >> 1) & 1u), oy = (int)(q >> 2);
    uint32_t len = 0;
    st = 0;
    if (lane < 18) {
        const int r = (int)(lane >> 1), part = (int)(lane & 1u);
        const int sy = 2 * cy + oy + r / 3 - 1, sz = 2 * cz + oz + r % 3 - 1;
        const int oyz = ((sy & 1) * 2 + (sz & 1)) * 2;
        int ccx, xlo, xhi;
        if ((ox == 0) == (part == 0)) {  // the single x-neighbour bucket in the adjacent cell
            ccx = ox == 0 ? cx - 1 : cx + 1;
            xlo = xhi = ox == 0 ? 1 : 0;
        } else {                         // both x buckets of the bucket's own cell column
            ccx = cx;
            xlo = 0;
            xhi = 1;
        }
        const uint32_t cc = (uint32_t)(((sy >> 1) * P.rz + (sz >> 1)) * P.rx + ccx);
        const uint32_t cs = __ldg(&B.cstart[cc]), ce = __ldg(&B.cend[cc]);
        if (cs < ce) {
            st = __ldg(&B.oct_start[(size_t)cc * 8 + oyz + xlo]);
            const uint32_t en = (oyz + xhi == 7) ? ce : __ldg(&B.oct_start[(size_t)cc * 8 + oyz + xhi + 1]);
            len = en - st;
        }
    }
    uint32_t inc = len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, inc, d);
        if ((int)lane >= d) inc += v;
    }
    const uint32_t T = __shfl_sync(0xffffffffu, inc, 31);
    off = inc - len;
    if (lane < 18) {
        rstart[lane] = st;
        roff[lane] = off;
    }
    if (lane == 18) roff[18] = T;
    __syncwarp();
    return T;
}

// Index of candidate e of the sequence; r is the caller's range cursor (e must
// not decrease between calls with the same cursor).
__device__ __forceinline__ uint32_t seq_index(const uint32_t* rstart, const uint32_t* roff, int& r, uint32_t e) {
    while (roff[r + 1] <= e) r++;
    return rstart[r] + (e - roff[r]);
}

constexpr int kBucketChunks = 8;

__device__ __forceinline__ uint32_t next_bucket(uint32_t* ctr, unsigned lane) {
    uint32_t v = 0;
    if (lane == 0) v = atomicAdd(ctr, 1u);
    return __shfl_sync(0xffffffffu, v, 0);
}

template <bool SS1>
__global__ void __launch_bounds__(kThreads, 4) k_density_bucket(const __grid_constant__ DevParams P,
                                                                const __grid_constant__ DevBuffers B,
                                                                const float4* __restrict__ pos4,
                                                                const float4* __restrict__ alpha4) {
    constexpr int kWarps = kThreads / 32;
    __shared__ uint32_t tab[kWarps][2][20];                 // range starts and sequence offsets
    const unsigned lane = lane_id();
    const int w = threadIdx.x >> 5;
    uint32_t* rstart = tab[w][0];
    uint32_t* roff = tab[w][1];
    const uint32_t nb = *B.act_n * 8u;
    const uint32_t nitems = nb + *B.wq_n;  // the first window of every bucket, then the queued windows
    const size_t cap = (size_t)P.cap;
    const float r2 = P.r2, r2list = P.r2list, ss = P.ss;
    const float kFar = __int_as_float(0x7f800000);  // +inf: never within range
    for (uint32_t it = next_bucket(B.dctr, lane); it < nitems; it = next_bucket(B.dctr, lane)) {
        uint32_t c, q, w0;
        if (it < nb) {
            c = __ldg(&B.act[it >> 3]);
            q = it & 7u;
            w0 = __ldg(&B.oct_start[(size_t)c * 8 + q]);
        } else {
            const uint2 e = B.wq[it - nb];
            c = e.x >> 3;
            q = e.x & 7u;
            w0 = e.y;
        }
        const uint32_t bid = c * 8u + q;
        const uint32_t m0 = __ldg(&B.oct_start[(size_t)bid]);
        const uint32_t m1 = q == 7 ? __ldg(&B.cend[c]) : __ldg(&B.oct_start[(size_t)bid + 1]);
        if (w0 >= m1) continue;
        const uint32_t w1 = min(m1, w0 + (uint32_t)P.bwin);
        // the window's members, one per lane; boundary members carry their volume and need no list
        const uint32_t tl = w0 + lane;
        float4 pm = make_float4(kFar, kFar, kFar, -1.f);
        float rm = 0.f;
        if (tl < w1) {
            pm = __ldg(&pos4[tl]);
            if (pm.w < 0.f) {
                B.densp[tl] = make_float2(-pm.w, 0.f);
                B.nbr_cnt[tl] = 0;
            } else {
                rm = __ldg(&alpha4[tl]).w;
            }
        }
        const uint32_t fluid = __ballot_sync(0xffffffffu, tl < w1 && pm.w >= 0.f);
        if (!fluid) continue;
        uint32_t st, off;
        const uint32_t T = bucket_ranges(P, B, c, q, lane, rstart, roff, st, off);
        const bool masked = T <= 32u * kMaskWords;
        if (masked && w0 == m0) {  // the bucket's range table, once per bucket
            uint32_t* __restrict__ bt = B.btab + (size_t)bid * kTabStride;
            if (lane < 18) {
                bt[lane] = off;
                bt[20 + lane] = st - off;
            }
            if (lane == 18) bt[18] = T;
        }
        const uint32_t lst = masked ? (kMaskList | bid) : kRescan;
        // sequence position of member t = t + self_base: the bucket lies in the range of its own
        // cell column on its own subcell row (range 8 + part, part = 1 for the low x half)
        const int rs = 8 + ((q & 1u) == 0u ? 1 : 0);
        const uint32_t self_base = __shfl_sync(0xffffffffu, off, rs) - __shfl_sync(0xffffffffu, st, rs);
        Kahan msum;  // lane i: member w0 + i, summed over the candidate blocks
        int r = 0;
        const float2 R2 = make_float2(r2, r2), NEG1 = make_float2(-1.f, -1.f);
        for (uint32_t base = 0; base < T; base += 32u * kBucketChunks) {
            // chunks 2p and 2p + 1 side by side in float2 pairs (packed FP32 arithmetic):
            // negated coordinates and w (fluid mass > 0, minus the boundary volume < 0; 0 for padding)
            float2 NX[kBucketChunks / 2], NY[kBucketChunks / 2], NZ[kBucketChunks / 2], CW[kBucketChunks / 2];
            bool bnd = false;
#pragma unroll
            for (int pr = 0; pr < kBucketChunks / 2; pr++) {
                float4 c2[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const uint32_t e = base + lane + 32u * (2 * pr + h);
                    c2[h] = make_float4(kFar, kFar, kFar, 0.f);
                    if (e < T) c2[h] = __ldg(&pos4[seq_index(rstart, roff, r, e)]);
                    bnd |= c2[h].w < 0.f;
                }
                NX[pr] = make_float2(-c2[0].x, -c2[1].x);
                NY[pr] = make_float2(-c2[0].y, -c2[1].y);
                NZ[pr] = make_float2(-c2[0].z, -c2[1].z);
                CW[pr] = make_float2(c2[0].w, c2[1].w);
            }
            const int nch = (int)min((T - base + 31u) >> 5, (uint32_t)kBucketChunks);
            const uint32_t word0 = base >> 5;
            // The member loop, with boundary candidates in the block or without (the usual case:
            // no volume weights and no rest density to broadcast, so fewer live registers).
            // The weight of a candidate is its mass, or rho0 V for a boundary particle; without
            // boundary candidates rho0 * 0 + m is m exactly, so both forms give the same sums.
            auto members = [&](auto with_boundary) {
                constexpr bool BND = decltype(with_boundary)::value;
                float2 CM[kBucketChunks / 2], CV[kBucketChunks / 2];
#pragma unroll
                for (int pr = 0; pr < kBucketChunks / 2; pr++) {
                    CM[pr] = CW[pr];
                    CV[pr] = make_float2(0.f, 0.f);
                    if (BND) {
                        CM[pr] = make_float2(fmaxf(CW[pr].x, 0.f), fmaxf(CW[pr].y, 0.f));
                        CV[pr] = make_float2(fmaxf(-CW[pr].x, 0.f), fmaxf(-CW[pr].y, 0.f));
                    }
                }
                for (uint32_t fm = fluid; fm != 0u; fm &= fm - 1u) {
                    const int i = __ffs(fm) - 1;
                    const float px = __shfl_sync(0xffffffffu, pm.x, i);
                    const float py = __shfl_sync(0xffffffffu, pm.y, i);
                    const float pz = __shfl_sync(0xffffffffu, pm.z, i);
                    const float rho0 = BND ? __shfl_sync(0xffffffffu, rm, i) : 0.f;
                    const float2 PX = make_float2(px, px), PY = make_float2(py, py), PZ = make_float2(pz, pz);
                    const float2 RHO = make_float2(rho0, rho0);
                    const uint32_t t = w0 + (uint32_t)i;
                    float2 acc = make_float2(0.f, 0.f);
                    uint32_t mine = 0;  // lane k keeps the mask word of chunk k
#pragma unroll
                    for (int pr = 0; pr < kBucketChunks / 2; pr++) {
                        if (2 * pr < nch) {
                            float2 dx = __fadd2_rn(PX, NX[pr]), dy = __fadd2_rn(PY, NY[pr]), dz = __fadd2_rn(PZ, NZ[pr]);
                            if (!SS1) {
                                const float2 SS = make_float2(ss, ss);
                                dx = __fmul2_rn(dx, SS);
                                dy = __fmul2_rn(dy, SS);
                                dz = __fmul2_rn(dz, SS);
                            }
                            float2 dsq = __fmul2_rn(dx, dx);
                            dsq = __ffma2_rn(dy, dy, dsq);
                            dsq = __ffma2_rn(dz, dz, dsq);
                            float2 cc = __ffma2_rn(dsq, NEG1, R2);  // r2 - dsq, rounded once
                            cc.x = fmaxf(cc.x, 0.f);                // 0 outside h (and for the padding lanes)
                            cc.y = fmaxf(cc.y, 0.f);
                            const float2 c3 = __fmul2_rn(__fmul2_rn(cc, cc), cc);
                            acc = __ffma2_rn(c3, BND ? __ffma2_rn(RHO, CV[pr], CM[pr]) : CM[pr], acc);
                            // coincident particles stay in the list (every consumer skips r == 0);
                            // the member itself is cleared below
                            const uint32_t b0 = __ballot_sync(0xffffffffu, dsq.x < r2list);
                            const uint32_t b1 = __ballot_sync(0xffffffffu, dsq.y < r2list);
                            mine = lane == (unsigned)(2 * pr) ? b0 : mine;
                            mine = lane == (unsigned)(2 * pr + 1) ? b1 : mine;
                        }
                    }
                    const uint32_t es = t + self_base - base;  // the member's own bit, if in this block
                    if (es < 32u * kBucketChunks && lane == (es >> 5)) mine &= ~(1u << (es & 31u));
                    if (masked && (int)lane < nch) B.nmask[(size_t)(word0 + lane) * cap + t] = mine;
                    const float part = warp_sum_f(acc.x + acc.y);
                    if (lane == (unsigned)i) msum.add(part);
                }
            };
            if (__any_sync(0xffffffffu, bnd))
                members(std::true_type{});
            else
                members(std::false_type{});
        }
        if (tl < w1 && pm.w >= 0.f) {
            B.nbr_cnt[tl] = lst;
            B.densp[tl] = density_result(P, msum.s, rm);
        }
    }
}

// Index lists from the bucket mask lists: bit e of a member's mask stands for
// candidate e of its bucket's sequence, whose index is e plus the offset of the
// sequence range holding e (btab). One thread per in-grid particle; the lanes
// of a warp emit their n-th entries together and store each group of four as
// one 16-byte word, so that every group row of the lists is written by one
// coalesced store. A particle with more
// than kMaxNbr neighbours keeps its mask list (nbr_cnt = kMaskList | bucket),
// which the passes decode directly. Particles with more than P.heavy
// neighbours (their lists flagged kHeavyFlag), with mask lists or left to the
// cell search are queued in hq for the force and alpha passes.
__global__ void __launch_bounds__(kThreads) k_expand_lists(const __grid_constant__ DevParams P,
                                                           const __grid_constant__ DevBuffers B) {
    const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
    const uint32_t lst = t < B.cstart[P.G] ? B.nbr_cnt[t] : 0u;
    const bool mine = (lst & kMaskList) != 0;  // else boundary, index list or cell search already
    const uint32_t* __restrict__ tab = B.btab + (size_t)(mine ? lst & ~kMaskList : 0u) * kTabStride;
    const uint32_t nw = mine ? (__ldg(&tab[18]) + 31u) >> 5 : 0u;
    const size_t cap = (size_t)P.cap;
    const uint32_t* __restrict__ mw = B.nmask + t;
    // hits of this particle, then of the warp's busiest lane (the loop bound)
    uint32_t cnt = 0;
    for (uint32_t wd = 0; wd < nw; wd++) cnt += __popc(__ldg(mw + (size_t)wd * cap));
    const bool over = cnt > (uint32_t)kMaxNbr;  // keeps its mask list: nothing to write
    if (over) cnt = 0;
    uint32_t rounds = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rounds = max(rounds, __shfl_xor_sync(0xffffffffu, rounds, o));
    uint4* __restrict__ grp = reinterpret_cast<uint4*>(B.nbr) + t;
    uint32_t q0 = 0, q1 = 0, q2 = 0, q3 = 0;  // the list group being filled
    // the next mask word and the next range of the table are loaded one ahead, so
    // that the lockstep rounds wait on neither (only on a run of empty words or ranges)
    int r = 0;
    uint32_t end = 0, delta = 0, endn = 0, deltan = 0;
    if (mine) {
        end = __ldg(&tab[1]);
        delta = __ldg(&tab[20]);
        endn = __ldg(&tab[2]);
        deltan = __ldg(&tab[21]);
    }
    uint32_t wd = 0, m = nw > 0u ? __ldg(mw) : 0u, mn = nw > 1u ? __ldg(mw + cap) : 0u;
    for (uint32_t n = 0; n < rounds; n++) {
        if (n < cnt) {
            while (m == 0u) {
                m = mn;
                ++wd;
                mn = wd + 1u < nw ? __ldg(mw + (size_t)(wd + 1u) * cap) : 0u;
            }
            const uint32_t e = (wd << 5) + (uint32_t)(__ffs(m) - 1);
            m &= m - 1u;
            while (e >= end) {  // ends at tab[18] = the sequence length > e; reads stay below tab[39]
                r++;
                end = endn;
                delta = deltan;
                endn = __ldg(&tab[r + 2]);
                deltan = __ldg(&tab[21 + r]);
            }
            const uint32_t v = e + delta, u = n & 3u;
            q0 = u == 0u ? v : q0;
            q1 = u == 1u ? v : q1;
            q2 = u == 2u ? v : q2;
            q3 = u == 3u ? v : q3;
            if (u == 3u || n + 1u == cnt) grp[(size_t)(n >> 2) * cap] = make_uint4(q0, q1, q2, q3);
        }
    }
    const bool heavy = (mine && (over || cnt > P.heavy)) || lst == kRescan;
    if (mine && !over) B.nbr_cnt[t] = heavy ? (cnt | kHeavyFlag) : cnt;
    const uint32_t hb = __ballot_sync(0xffffffffu, heavy);
    if (hb) {
        const unsigned lane = lane_id();
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(B.hq_n, (uint32_t)__popc(hb));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (heavy) B.hq[base + __popc(hb & lanemask_lt())] = t;
    }
}

__global__ void __launch_bounds__(kThreads) k_density(const __grid_constant__ DevParams P,
                                                      const __grid_constant__ DevBuffers B,
                                                      const float4* __restrict__ pos4,
                                                      const float4* __restrict__ alpha4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B) || B.mgcell[s] == kUndef) return;
    const float4 pi = pos4[s];
    if (pi.w < 0.f) {  // boundary: carries its volume, no pressure, needs no list
        B.densp[s] = make_float2(-pi.w, 0.f);
        B.nbr_cnt[s] = 0;
        return;
    }
    const float rho0 = alpha4[s].w;
    Kahan sum;
    uint32_t cnt = 0;
    for_candidates(P, B, B.mgcell[s], pi.x, pi.y, pi.z, [&](uint32_t j) {
        const float4 pj = __ldg(&pos4[j]);
        const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
        const float dsq = dx * dx + dy * dy + dz * dz;
        if (dsq < P.r2) {
            const float c = P.r2 - dsq;
            const float m = pj.w > 0.f ? pj.w : rho0 * (-pj.w);
            sum.add(c * c * c * m);
        }
        if (dsq > 0.f && dsq < P.r2list) {
            if (cnt < (uint32_t)kMaxNbr) B.nbr[nbr_at((size_t)P.cap, (uint32_t)s, cnt)] = j;
            cnt++;
        }
    });
    B.nbr_cnt[s] = cnt;
    B.densp[s] = density_result(P, sum.s, rho0);
}

// ---------------------------------------------------------------------------
// Force + drift velocity (MfComputeForceCUDA, MfComputeDriftVelCUDA)
// ---------------------------------------------------------------------------

// Force + drift of one in-grid fluid particle, neighbours gathered from global
// memory through its list (or the cell search).
template <bool FORCE, bool DRIFT, int NP>
__device__ __forceinline__ void force_drift_one(const DevParams& P, const DevBuffers& B,
                                                const float4* __restrict__ pos4, const float4* __restrict__ vel4,
                                                const float4* __restrict__ alpha4, const float4* __restrict__ aprev4,
                                                const float4* __restrict__ vev4, int s, const float4 pi) {
    ForceDrift<FORCE, DRIFT, NP> acc;
    acc.init(P, pi, vel4[s], B.densp[s], alpha4[s]);
    for_slot_list(P, B, s, pi.x, pi.y, pi.z, [&](uint32_t j) {
        // every load first (list entries are almost always neighbours), so that
        // consecutive neighbours' gathers overlap
        const float4 pj = __ldg(&pos4[j]);
        const float2 dpj = __ldg(&B.densp[j]);
        const float4 vj = FORCE ? __ldg(&vel4[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 aj = DRIFT ? __ldg(&alpha4[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
        acc.pair(P, pj, dpj, vj, aj);
    });
    acc.finish(P, B, s, DRIFT ? aprev4[s] : make_float4(0.f, 0.f, 0.f, 0.f),
               FORCE && DRIFT ? vev4[s] : make_float4(0.f, 0.f, 0.f, 0.f));
}

// Force + drift of heavy particle s by the whole warp (every lane calls with
// the same s): the lanes share its neighbours out, their partial sums are
// added, lane 0 stores.
template <bool FORCE, bool DRIFT, int NP>
__device__ __forceinline__ void force_drift_warp(const DevParams& P, const DevBuffers& B,
                                                 const float4* __restrict__ pos4, const float4* __restrict__ vel4,
                                                 const float4* __restrict__ alpha4, const float4* __restrict__ aprev4,
                                                 const float4* __restrict__ vev4, int s) {
    const float4 pi = pos4[s];
    ForceDrift<FORCE, DRIFT, NP> acc;
    acc.init(P, pi, vel4[s], B.densp[s], alpha4[s]);
    warp_for_slot_list(P, B, s, pi.x, pi.y, pi.z, [&](uint32_t j) {
        const float4 pj = __ldg(&pos4[j]);
        const float2 dpj = __ldg(&B.densp[j]);
        const float4 vj = FORCE ? __ldg(&vel4[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 aj = DRIFT ? __ldg(&alpha4[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
        acc.pair(P, pj, dpj, vj, aj);
    });
    acc.warp_reduce();
    if (lane_id() == 0)
        acc.finish(P, B, s, DRIFT ? aprev4[s] : make_float4(0.f, 0.f, 0.f, 0.f),
                   FORCE && DRIFT ? vev4[s] : make_float4(0.f, 0.f, 0.f, 0.f));
}

// Force + drift, one thread per particle; every warp first takes heavy
// particles from the queue (whole warp per particle) while any are left. With
// both, it also writes every in-grid particle's neighbour record for the fused
// alpha pass.
template <bool FORCE, bool DRIFT, int NP>
__global__ void __launch_bounds__(kThreads, 4) k_force_drift(const __grid_constant__ DevParams P,
                                                             const __grid_constant__ DevBuffers B,
                                                             const float4* __restrict__ pos4,
                                                             const float4* __restrict__ vel4,
                                                             const float4* __restrict__ alpha4,
                                                             const float4* __restrict__ aprev4,
                                                             const float4* __restrict__ vev4) {
    if (P.list_mode != 0) {
        const unsigned lane = lane_id();
        const uint32_t nh = *B.hq_n;
        for (uint32_t h = next_item(&B.hctr[0], nh, lane); h < nh; h = next_item(&B.hctr[0], nh, lane))
            force_drift_warp<FORCE, DRIFT, NP>(P, B, pos4, vel4, alpha4, aprev4, vev4, (int)B.hq[h]);
    }
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B) || B.mgcell[s] == kUndef) return;
    const float4 pi = pos4[s];
    if (pi.w < 0.f) {
        if (FORCE) B.accel4[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (FORCE && DRIFT) {
            const float a0[3] = {0.f, 0.f, 0.f};
            const float u0[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            write_nrec(B, s, pi, -1.f, make_float4(0.f, 0.f, 0.f, 0.f), a0, u0);
        }
        return;
    }
    if (is_heavy(P, B.nbr_cnt[s])) return;  // taken from the queue
    force_drift_one<FORCE, DRIFT, NP>(P, B, pos4, vel4, alpha4, aprev4, vev4, s, pi);
}

// Force + drift of a corrected large step: the same pass, also filling the
// corrector's features from the neighbours it gathers (alpha4 is gathered
// even without drift). Features and ids cover every particle; 128 registers.
template <bool DRIFT, int NP>
__global__ void __launch_bounds__(kThreads, 2) k_force_drift_feat(const __grid_constant__ DevParams P,
                                                                  const __grid_constant__ DevBuffers B,
                                                                  const float4* __restrict__ pos4,
                                                                  const float4* __restrict__ vel4,
                                                                  const float4* __restrict__ alpha4,
                                                                  const float4* __restrict__ aprev4,
                                                                  const float4* __restrict__ vev4, float* feat,
                                                                  int32_t* ids, float vs, float dt_large) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B)) return;
    float* row = feat + (size_t)s * kLearnedFeatures;
    if (B.mgcell[s] == kUndef) {
        store_no_features(row, &ids[s]);
        return;
    }
    const float4 pi = pos4[s];
    if (pi.w < 0.f) {
        B.accel4[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (DRIFT) {
            const float a0[3] = {0.f, 0.f, 0.f};
            const float u0[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            write_nrec(B, s, pi, -1.f, make_float4(0.f, 0.f, 0.f, 0.f), a0, u0);
        }
        store_no_features(row, &ids[s]);
        return;
    }
    const float4 vi = vel4[s], ai = alpha4[s], gi = aprev4[s];
    const float2 di = B.densp[s];
    ForceDrift<true, DRIFT, NP> acc;
    acc.init(P, pi, vi, di, ai);
    LearnedFeatures lf;
    lf.init(P, pi, vi, ai, di, gi, vs, dt_large);
    for_slot_list(P, B, s, pi.x, pi.y, pi.z, [&](uint32_t j) {
        const float4 pj = __ldg(&pos4[j]);
        const float2 dpj = __ldg(&B.densp[j]);
        const float4 vj = __ldg(&vel4[j]);
        const float4 aj = __ldg(&alpha4[j]);
        acc.pair(P, pj, dpj, vj, aj);
        lf.pair(P, pj, dpj, vj, aj);
    });
    acc.finish(P, B, s, DRIFT ? gi : make_float4(0.f, 0.f, 0.f, 0.f), DRIFT ? vev4[s] : make_float4(0.f, 0.f, 0.f, 0.f));
    lf.store(row);
    ids[s] = B.bornid[__float_as_uint(gi.w)];
}

// Surface tension (reference SurfaceTension, fluid_system_kern.cu:569-625): all
// 27 cells, squared distance compared with the radius K*h, added to accel.
__global__ void __launch_bounds__(kThreads) k_surface_tension(const __grid_constant__ DevParams P,
                                                              const __grid_constant__ DevBuffers B,
                                                              const float4* __restrict__ pos4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B)) return;
    const uint32_t gc = B.mgcell[s];
    if (gc == kUndef) return;
    const float4 pi = pos4[s];
    const float tR = sqrtf(P.st_K * P.st_K * (P.h * P.h));
    float rx = 0.f, ry = 0.f, rz = 0.f;
    for (int c = 0; c < 27; c++) {
        const uint32_t cell = gc + (uint32_t)P.neighborid[c];
        const uint32_t j0 = B.cstart[cell], j1 = B.cend[cell];
        for (uint32_t j = j0; j < j1; j++) {
            const float4 pj = __ldg(&pos4[j]);
            const float dx = (pi.x - pj.x) * P.ss, dy = (pi.y - pj.y) * P.ss, dz = (pi.z - pj.z) * P.ss;
            float dsq = dx * dx + dy * dy + dz * dz;
            if (dsq != 0.f && dsq <= tR) {
                dsq = sqrtf(dsq);
                const float fm = P.st_C * cosf(1.5f * 3.14159f * dsq / tR) / dsq;
                rx += dx * fm; ry += dy * fm; rz += dz * fm;
            }
        }
    }
    float4 a = B.accel4[s];
    a.x += rx; a.y += ry; a.z += rz;
    B.accel4[s] = a;
}

// Project-U force (ComputeForce_projectu, multiphase.cu:578-616), one thread
// per particle: writes accel (the reference's mforce) and the XSPH correction of
// every in-grid fluid particle. In-grid boundary particles get accel 0, as in the
// force pass; boundary and out-of-grid particles get a zero correction (the
// reference leaves both untouched for them).
template <int NP>
__global__ void __launch_bounds__(kThreads) k_force_projectu(const __grid_constant__ DevParams P,
                                                             const __grid_constant__ DevBuffers B,
                                                             const float4* __restrict__ pos4,
                                                             const float4* __restrict__ vel4,
                                                             const float4* __restrict__ vev4,
                                                             const float4* __restrict__ alpha_cur,
                                                             const float4* __restrict__ alpha_pre,
                                                             const float4* __restrict__ aprev4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B)) return;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 pi = pos4[s];
    if (B.mgcell[s] == kUndef || pi.w < 0.f) {
        if (B.mgcell[s] != kUndef) B.accel4[s] = zero;
        B.velxcor[s] = zero;
        return;
    }
    float3 um[NP];
#pragma unroll
    for (int k = 0; k < NP; k++) {
        const float4 u = B.drift4[(size_t)k * P.cap + s];
        um[k] = make_float3(u.x, u.y, u.z);
    }
    ProjectU<NP> acc;
    acc.init(pi, vev4[s], B.densp[s], vel4[s].w, alpha_cur[s].w, alpha_pre[s], um);
    for_slot_list(P, B, s, pi.x, pi.y, pi.z, [&](uint32_t j) {
        const float4 pj = __ldg(&pos4[j]);
        const float2 dpj = __ldg(&B.densp[j]);
        const float4 vej = __ldg(&vev4[j]);
        const float viscj = __ldg(&vel4[j].w);
        const float4 aj = __ldg(&alpha_pre[j]);
        float4 uj[NP];
#pragma unroll
        for (int k = 0; k < NP; k++) uj[k] = __ldg(&B.drift4[(size_t)k * P.cap + j]);
        float mj = pj.w, rho0j = 1.f;
        if (pj.w < 0.f) {  // boundary: raw mass (per origin) and rest density
            mj = __ldg(&B.mass_raw[__float_as_uint(__ldg(&aprev4[j].w))]);
            rho0j = __ldg(&alpha_cur[j].w);
        }
        acc.pair(P, pj, dpj, vej, viscj, rho0j, mj, aj, uj);
    });
    B.accel4[s] = make_float4(acc.fx, acc.fy, acc.fz, 0.f);
    B.velxcor[s] = make_float4(acc.xx, acc.xy, acc.xz, 0.f);
}

// ---------------------------------------------------------------------------
// Volume-fraction advance, correction, advection
// ---------------------------------------------------------------------------

// Alpha change of particle s with neighbours gathered from global memory (the
// separate alpha-advance pass of the reference call order).
template <int NP>
__device__ __forceinline__ void alpha_change_slot(const DevParams& P, const DevBuffers& B,
                                                  const float4* __restrict__ pos4, const float4* __restrict__ vev4,
                                                  const float4* __restrict__ alpha4, int s, const float4 pi,
                                                  const float4 vei, const float4 ai, float (&out)[3]) {
    AlphaChange<NP> acc;
    acc.init(pi, vei, ai, B.drift4 + s, (size_t)P.cap);
    for_slot_list(P, B, s, pi.x, pi.y, pi.z, [&](uint32_t j) {
        // every load first, so that consecutive neighbours' gathers overlap
        const float4 pj = __ldg(&pos4[j]);
        const float2 dpj = __ldg(&B.densp[j]);
        const float4 vej = __ldg(&vev4[j]);
        const float4 aj = __ldg(&alpha4[j]);
        float4 uj[NP];
#pragma unroll
        for (int k = 0; k < NP; k++) uj[k] = __ldg(&B.drift4[(size_t)k * P.cap + j]);
        acc.pair(P, pj, pj.w * dpj.x, vej, aj, uj);
    });
    acc.result(P, out);
}

// Separate alpha advance: new fractions into alpha4 out (restdens copied).
template <int NP>
__global__ void __launch_bounds__(kThreads) k_alpha_advance(const __grid_constant__ DevParams P,
                                                            const __grid_constant__ DevBuffers B,
                                                            const float4* __restrict__ pos4,
                                                            const float4* __restrict__ vev4,
                                                            const float4* __restrict__ alpha_in,
                                                            float4* __restrict__ alpha_out) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B)) return;
    const float4 ai = alpha_in[s];
    const float4 pi = pos4[s];
    if (B.mgcell[s] == kUndef || pi.w < 0.f) {
        alpha_out[s] = ai;
        return;
    }
    float na[3] = {ai.x, ai.y, ai.z};
    alpha_change_slot<NP>(P, B, pos4, vev4, alpha_in, s, pi, vev4[s], ai, na);
    alpha_out[s] = make_float4(na[0], na[1], na[2], ai.w);
}

// Separate correction, in place: fractions in alpha_cur, start-of-step in alpha_pre.
template <int NP>
__global__ void __launch_bounds__(kThreads) k_correction(const __grid_constant__ DevParams P,
                                                         const __grid_constant__ DevBuffers B,
                                                         float4* alpha_cur, const float4* alpha_pre,
                                                         float4* __restrict__ vel4,
                                                         const float4* __restrict__ pos4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B)) return;
    if (B.mgcell[s] == kUndef || pos4[s].w < 0.f) return;
    const float4 ac = alpha_cur[s];
    const float4 ap = alpha_pre[s];
    float a[3] = {ac.x, ac.y, ac.z};
    const float apre[3] = {ap.x, ap.y, ap.z};
    float pmod, nr, nv;
    correct<NP>(P, a, apre, B.densp[s].x, ac.w, pmod, nr, nv);
    alpha_cur[s] = make_float4(a[0], a[1], a[2], nr);
    float4 v = vel4[s];
    v.w = nv;
    vel4[s] = v;
    B.pmod[s] = pmod;
}

// Separate advance, in place.
__global__ void __launch_bounds__(kThreads) k_advance(const __grid_constant__ DevParams P,
                                                      const __grid_constant__ DevBuffers B, float4* pos4,
                                                      float4* vel4, float4* vev4, float4* aprev4) {
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B)) return;
    float4 p = pos4[s];
    if (p.w < 0.f) return;
    float4 v = vel4[s];
    if (B.mgcell[s] == kUndef) {
        p.x = -1000.f; p.y = -1000.f; p.z = -1000.f;
        v.x = 0.f; v.y = 0.f; v.z = 0.f;
        pos4[s] = p;
        vel4[s] = v;
        return;
    }
    float4 ve = vev4[s], ap = aprev4[s];
    advance_one(P, p, v, ve, ap, B.accel4[s]);
    pos4[s] = p;
    vel4[s] = v;
    vev4[s] = ve;
    aprev4[s] = ap;
}

// Alpha change of in-grid particle s with its neighbours' data from the
// neighbour records the force + drift pass of this step wrote (five 16-byte
// loads per neighbour instead of seven separate gathers).
template <int NP>
__device__ __forceinline__ void alpha_change_nrec(const DevParams& P, const DevBuffers& B, int s, const float4 pi,
                                                  const float4 vei, const float4 ai, float (&out)[3]) {
    AlphaChange<NP> acc;
    acc.init(pi, vei, ai, B.drift4 + s, (size_t)P.cap);
    for_slot_list(P, B, s, pi.x, pi.y, pi.z, [&](uint32_t j) {
        float4 q[5];
        read_nrec<NP>(B, j, q);
        const float4 r0 = q[0], r1 = q[1], r2 = q[2], r3 = q[3], r4 = q[4];
        float4 uj[NP];
        uj[0] = make_float4(r2.z, r2.w, r3.x, 0.f);
        if (NP > 1) uj[NP > 1 ? 1 : 0] = make_float4(r3.y, r3.z, r3.w, 0.f);
        if (NP > 2) uj[NP > 2 ? 2 : 0] = make_float4(r4.x, r4.y, r4.z, 0.f);
        acc.pair(P, r0, r0.w, make_float4(r1.x, r1.y, r1.z, 0.f), make_float4(r1.w, r2.x, r2.y, 0.f), uj);
    });
    acc.result(P, out);
}

// Alpha change of heavy particle s by the whole warp (every lane calls with the
// same s and gets the result).
template <int NP>
__device__ __forceinline__ void alpha_change_nrec_warp(const DevParams& P, const DevBuffers& B, const F4Set& S, int s,
                                                       float (&out)[3]) {
    const float4 pi = S.in[POS][s], vei = S.in[VEV][s], ai = S.in[ALPHA][s];
    AlphaChange<NP> acc;
    acc.init(pi, vei, ai, B.drift4 + s, (size_t)P.cap);
    warp_for_slot_list(P, B, s, pi.x, pi.y, pi.z, [&](uint32_t j) {
        float4 q[5];
        read_nrec<NP>(B, j, q);
        const float4 r0 = q[0], r1 = q[1], r2 = q[2], r3 = q[3], r4 = q[4];
        float4 uj[NP];
        uj[0] = make_float4(r2.z, r2.w, r3.x, 0.f);
        if (NP > 1) uj[NP > 1 ? 1 : 0] = make_float4(r3.y, r3.z, r3.w, 0.f);
        if (NP > 2) uj[NP > 2 ? 2 : 0] = make_float4(r4.x, r4.y, r4.z, 0.f);
        acc.pair(P, r0, r0.w, make_float4(r1.x, r1.y, r1.z, 0.f), make_float4(r1.w, r2.x, r2.y, 0.f), uj);
    });
    acc.warp_reduce();
    acc.result(P, out);
}

// Alpha + correction + advance of one slot whose alpha sum (in-grid fluid
// particles) is `anew`; writes the five float4 fields to the other buffer.
template <int NP, bool MP>
__device__ __forceinline__ void pass_c_finish(const DevParams& P, const DevBuffers& B, const F4Set& S, int s,
                                              bool undef, float4 p, float4 ve, float4 al, const float (&anew)[3]) {
    float4 v = S.in[VEL][s], ap = S.in[APREV][s];
    pass_c_slot<NP, MP>(P, B, s, undef, p, v, ve, al, ap, [&](float (&a)[3]) {
        a[0] = anew[0];
        a[1] = anew[1];
        a[2] = anew[2];
    });
    S.out[POS][s] = p;
    S.out[VEL][s] = v;
    S.out[VEV][s] = ve;
    S.out[ALPHA][s] = al;
    S.out[APREV][s] = ap;
}

// Fused alpha advance + correction + advance, one thread per particle: reads the
// cur buffers, writes every float4 field of every particle into the other
// buffer. Every warp first takes heavy particles from the queue (whole warp per
// alpha sum, lane 0 finishes the particle) while any are left.
template <int NP, bool MP>
__global__ void __launch_bounds__(kThreads, 4) k_pass_c(const __grid_constant__ DevParams P,
                                                        const __grid_constant__ DevBuffers B,
                                                        const __grid_constant__ F4Set S) {
    if (MP && P.list_mode != 0) {
        const unsigned lane = lane_id();
        const uint32_t nh = *B.hq_n;
        for (uint32_t h = next_item(&B.hctr[1], nh, lane); h < nh; h = next_item(&B.hctr[1], nh, lane)) {
            const int sh = (int)B.hq[h];
            float a[3];
            alpha_change_nrec_warp<NP>(P, B, S, sh, a);
            if (lane == 0) pass_c_finish<NP, MP>(P, B, S, sh, false, S.in[POS][sh], S.in[VEV][sh], S.in[ALPHA][sh], a);
        }
    }
    const int s = blockIdx.x * kThreads + threadIdx.x;
    if (s >= active_n(B)) return;
    const float4 p = S.in[POS][s], ve = S.in[VEV][s], al = S.in[ALPHA][s];
    const bool undef = B.mgcell[s] == kUndef;
    // the alpha sum is needed for in-grid fluid particles (pass_c_slot)
    const bool walk = MP && !undef && !(p.w < 0.f);
    if (walk && is_heavy(P, B.nbr_cnt[s])) return;  // taken from the queue
    float anew[3] = {al.x, al.y, al.z};
    if (walk) alpha_change_nrec<NP>(P, B, s, p, ve, al, anew);
    pass_c_finish<NP, MP>(P, B, S, s, undef, p, ve, al, anew);
}

// ---------------------------------------------------------------------------
// FP64 conservation sums
// ---------------------------------------------------------------------------

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kThreads) k_conservation(const __grid_constant__ DevParams P,
                                                           const __grid_constant__ DevBuffers B,
                                                           const float4* __restrict__ pos4,
                                                           const float4* __restrict__ alpha4) {
    __shared__ double sh[6][kThreads / 32];
    double acc[6] = {0, 0, 0, 0, 0, 0};  // mass, volume, vol_k (3), max |sum alpha - 1|
    const int n = active_n(B);
    for (int s = blockIdx.x * kThreads + threadIdx.x; s < n; s += gridDim.x * kThreads) {
        if (B.mgcell[s] == kUndef) continue;
        const float4 p = pos4[s];
        if (p.w < 0.f) continue;
        const double m = p.w;
        const double vol = m * (double)B.densp[s].x;
        const float4 a = alpha4[s];
        const float al[3] = {a.x, a.y, a.z};
        acc[0] += m;
        acc[1] += vol;
        double sa = 0.0;
        for (int k = 0; k < P.nphase; k++) {
            acc[2 + k] += (double)al[k] * vol;
            sa += (double)al[k];
        }
        acc[5] = fmax(acc[5], fabs(sa - 1.0));
    }
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 5; q++) {
        const double v = warp_sum_d(acc[q]);
        if (lane == 0) sh[q][warp] = v;
    }
    double mx = acc[5];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) sh[5][warp] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < 5; q++) {
            double t = 0.0;
            for (int w = 0; w < kThreads / 32; w++) t += sh[q][w];
            atomicAdd(&B.red[q], t);
        }
        double m = 0.0;
        for (int w = 0; w < kThreads / 32; w++) m = fmax(m, sh[5][w]);
        atomicMax(reinterpret_cast<unsigned long long*>(&B.red[5]), (unsigned long long)__double_as_longlong(m));
    }
}

// ---------------------------------------------------------------------------
// Active count and device-side emission
// ---------------------------------------------------------------------------

__global__ void k_set_count(const __grid_constant__ DevBuffers B, int n) { *B.nact = n; }

// FluidSystem::EmitParticles (SPH_Solver/fluids/fluid_system.cpp:619-641) on the
// device, one block: at every frame that is a multiple of E.interval, the sites
// of `layers` disks (EmitImmediate, :644-673; InsertParticles, :676-700) are
// appended after the active slots and the device count grows; at capacity the
// remaining sites are dropped (AddParticle returns -1 there) and the capacity
// error bit is set. The sites, their jitter (stream E.seed + frame, two draws
// per site in (layer, i, j) order) and every record field are computed with the
// operations of the host generator sphmp_emit_disk in the same order, without
// contraction, so the records are the ones sphmp_emit_disk + sphmp_emit_aos
// would upload; a block-wide scan keeps the slot order of the accepted sites.
__global__ void __launch_bounds__(kScanBlock) k_emit(const __grid_constant__ DevParams P,
                                                     const __grid_constant__ DevBuffers B,
                                                     const __grid_constant__ F4Set S,
                                                     const __grid_constant__ DevEmitter E) {
    __shared__ int sh_frame, sh_base;
    if (threadIdx.x == 0) {
        sh_frame = *B.frame;
        sh_base = *B.nact;
    }
    __syncthreads();
    const int f = sh_frame;
    if (E.interval <= 0 || f % E.interval != 0) {
        if (threadIdx.x == 0) *B.frame = f + 1;
        return;
    }
    const uint32_t base = (uint32_t)sh_base;
    const uint32_t room = (uint32_t)P.cap - base;
    const int side = 2 * E.res + 1;
    const uint32_t per_layer = (uint32_t)(side * side);
    const uint32_t m = per_layer * (uint32_t)E.layers;
    const uint64_t seed = E.seed + (uint64_t)f;
    const float js = __fmul_rn(E.jitter, E.spacing);
    const float jh = __fmul_rn(js, 0.5f);
    const float r2 = __fmul_rn(E.radius, E.radius);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t written = 0;
    for (uint32_t c0 = 0; c0 < m; c0 += kScanBlock) {
        const uint32_t k = c0 + threadIdx.x;
        bool ok = false;
        float t0 = 0.f, t2 = 0.f;
        int layer = 0;
        if (k < m) {
            layer = (int)(k / per_layer);
            const uint32_t rem = k - (uint32_t)layer * per_layer;
            const int i = (int)(rem / (uint32_t)side) - E.res;
            const int j = (int)(rem % (uint32_t)side) - E.res;
            const float jx = __fsub_rn(__fmul_rn(__fmul_rn(uniform01(seed, 2ull * k), E.jitter), E.spacing), jh);
            const float jz = __fsub_rn(__fmul_rn(__fmul_rn(uniform01(seed, 2ull * k + 1ull), E.jitter), E.spacing), jh);
            t0 = __fadd_rn(__fmul_rn((float)i, E.spacing), jx);
            t2 = __fadd_rn(__fmul_rn((float)j, E.spacing), jz);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(t0, t0), __fmul_rn(0.f, 0.f)), __fmul_rn(t2, t2));
            ok = !(d2 > r2);
        }
        uint32_t total;
        const uint32_t off = block_excl_scan(ok ? 1u : 0u, &total);
        const uint32_t q = written + off;
        if (ok && q < room) {
            const uint32_t idx = base + q;
            const float centre[3] = {E.pos[0], __fadd_rn(E.pos[1], __fmul_rn((float)layer, E.spacing)), E.pos[2]};
            float x[3], v[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                x[a] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(E.rot[a][0], t0), __fmul_rn(E.rot[a][1], 0.f)),
                                           __fmul_rn(E.rot[a][2], t2)),
                                 centre[a]);
                v[a] = __fmul_rn(E.dir[a], E.vel);
            }
            S.out[POS][idx] = make_float4(x[0], x[1], x[2], E.mass);
            S.out[VEL][idx] = make_float4(v[0], v[1], v[2], E.visc);
            S.out[VEV][idx] = make_float4(v[0], v[1], v[2], 0.f);
            S.out[ALPHA][idx] = make_float4(E.onehot == 0 ? 1.f : 0.f, E.onehot == 1 ? 1.f : 0.f,
                                            E.onehot == 2 ? 1.f : 0.f, E.restdens);
            S.out[APREV][idx] = make_float4(0.f, 0.f, 0.f, __uint_as_float(idx));
            B.opos[idx] = idx;
            B.oidx[idx] = idx;
            B.densp[idx] = make_float2(0.f, 0.f);
            B.accel4[idx] = zero;
            B.color[idx] = make_float4(__fdiv_rn((float)f, 200.0f), 0.5f, 0.8f, 0.5f);
            B.bornid[idx] = (int32_t)idx;
            B.mass_raw[idx] = E.mass;
        }
        written += total;
    }
    if (threadIdx.x == 0) {
        if (written > room) set_err(B, kErrCapacity);
        *B.nact = (int)(base + min(written, room));
        *B.frame = f + 1;
    }
}

// ---------------------------------------------------------------------------
// Transfers
// ---------------------------------------------------------------------------

__device__ __forceinline__ bool finite3(float x, float y, float z) { return isfinite(x) && isfinite(y) && isfinite(z); }

__global__ void __launch_bounds__(kThreads) k_unpack_aos(const __grid_constant__ DevParams P,
                                                         const __grid_constant__ DevBuffers B,
                                                         const __grid_constant__ F4Set S,
                                                         const sphmp_display_pack* __restrict__ disp,
                                                         const sphmp_calc_pack* __restrict__ calc, int start,
                                                         int end) {
    const int i = start + blockIdx.x * kThreads + threadIdx.x;
    if (i >= end) return;
    const sphmp_display_pack d = disp[i - start];
    const sphmp_calc_pack& c = calc[i - start];
    int type = d.type;
    if (type != SPHMP_TYPE_FLUID && type != SPHMP_TYPE_BOUNDARY) {
        set_err(B, kErrType);
        type = SPHMP_TYPE_FLUID;
    }
    if (!finite3(d.pos[0], d.pos[1], d.pos[2])) set_err(B, kErrNotFinite);
    float w;
    if (type == SPHMP_TYPE_BOUNDARY) {
        w = -fabsf(c.dens);
        if (!(w < 0.f)) w = -1.f;  // a boundary needs a negative tag; the volume pass sets the value
    } else {
        w = c.mass;
        if (!(w > 0.f) || !isfinite(w)) {
            set_err(B, kErrBadMass);
            w = 1.f;
        }
    }
    S.out[POS][i] = make_float4(d.pos[0], d.pos[1], d.pos[2], w);
    S.out[VEL][i] = make_float4(c.vel[0], c.vel[1], c.vel[2], c.visc);
    S.out[VEV][i] = make_float4(c.veleval[0], c.veleval[1], c.veleval[2], 0.f);
    // one-hot volume fraction at the first phase whose rest density matches
    int ph = 0;
    for (int k = 0; k < P.nphase; k++)
        if (P.dens_k[k] == c.restdens) { ph = k; break; }
    S.out[ALPHA][i] = make_float4(ph == 0 ? 1.f : 0.f, ph == 1 ? 1.f : 0.f, ph == 2 ? 1.f : 0.f, c.restdens);
    S.out[APREV][i] = make_float4(0.f, 0.f, 0.f, __uint_as_float((uint32_t)i));
    B.opos[i] = (uint32_t)i;  // freshly written slots sit at their own internal index
    B.oidx[i] = (uint32_t)i;
    B.densp[i] = make_float2(c.dens, c.pressure);
    B.accel4[i] = make_float4(c.accel[0], c.accel[1], c.accel[2], 0.f);
    B.color[i] = make_float4(d.color[0], d.color[1], d.color[2], d.color[3]);
    B.bornid[i] = c.bornid;
    B.mass_raw[i] = c.mass;
}

__global__ void __launch_bounds__(kThreads) k_pack_aos(const __grid_constant__ DevParams P,
                                                       const __grid_constant__ DevBuffers B,
                                                       const __grid_constant__ F4Set S, sphmp_display_pack* disp,
                                                       sphmp_calc_pack* calc, int n) {
    const int slot = blockIdx.x * kThreads + threadIdx.x;
    if (slot >= n) return;
    const int i = (int)B.opos[slot];
    const float4 p = S.in[POS][i];
    const uint32_t o = __float_as_uint(S.in[APREV][i].w);
    const bool bnd = p.w < 0.f;
    const float4 col = B.color[o];
    sphmp_display_pack d;
    d.pos[0] = p.x; d.pos[1] = p.y; d.pos[2] = p.z;
    d.color[0] = col.x; d.color[1] = col.y; d.color[2] = col.z; d.color[3] = col.w;
    d.type = bnd ? SPHMP_TYPE_BOUNDARY : SPHMP_TYPE_FLUID;
    disp[slot] = d;
    if (calc == nullptr) return;
    const float4 v = S.in[VEL][i], ve = S.in[VEV][i], al = S.in[ALPHA][i];
    const float2 dp = B.densp[i];
    const float4 ac = B.accel4[i];
    sphmp_calc_pack c;
    float* raw = reinterpret_cast<float*>(&c);
    for (int k = 0; k < (int)(sizeof(sphmp_calc_pack) / 4); k++) raw[k] = 0.f;
    c.vel[0] = v.x; c.vel[1] = v.y; c.vel[2] = v.z;
    c.veleval[0] = ve.x; c.veleval[1] = ve.y; c.veleval[2] = ve.z;
    c.pressure = bnd ? 0.f : dp.y;
    c.dens = bnd ? -p.w : dp.x;
    c.restdens = al.w;
    c.mass = B.mass_raw[o];
    c.visc = v.w;
    c.bornid = B.bornid[o];
    c.accel[0] = ac.x; c.accel[1] = ac.y; c.accel[2] = ac.z;
    calc[slot] = c;
}

__global__ void __launch_bounds__(kThreads) k_pack_field(const __grid_constant__ DevParams P,
                                                         const __grid_constant__ DevBuffers B,
                                                         const __grid_constant__ F4Set S, int field,
                                                         const float4* __restrict__ alpha_c,
                                                         const float4* __restrict__ alpha_p, void* stage, int n) {
    const int t = blockIdx.x * kThreads + threadIdx.x;  // slot (stage index)
    if (t >= n) return;
    const int i = (int)B.opos[t];                         // internal index
    float* f = reinterpret_cast<float*>(stage);
    int32_t* q = reinterpret_cast<int32_t*>(stage);
    const float4 p = S.in[POS][i];
    const uint32_t o = __float_as_uint(S.in[APREV][i].w);
    switch (field) {
        case SPHMP_F_POS: f[3 * t] = p.x; f[3 * t + 1] = p.y; f[3 * t + 2] = p.z; break;
        case SPHMP_F_VEL: { const float4 v = S.in[VEL][i]; f[3 * t] = v.x; f[3 * t + 1] = v.y; f[3 * t + 2] = v.z; } break;
        case SPHMP_F_VELEVAL: { const float4 v = S.in[VEV][i]; f[3 * t] = v.x; f[3 * t + 1] = v.y; f[3 * t + 2] = v.z; } break;
        case SPHMP_F_PRESSURE: f[t] = p.w < 0.f ? 0.f : B.densp[i].y; break;
        case SPHMP_F_DENS: f[t] = p.w < 0.f ? -p.w : B.densp[i].x; break;
        case SPHMP_F_RESTDENS: f[t] = alpha_c[i].w; break;
        case SPHMP_F_VISC: f[t] = S.in[VEL][i].w; break;
        case SPHMP_F_ACCEL: { const float4 a = B.accel4[i]; f[3 * t] = a.x; f[3 * t + 1] = a.y; f[3 * t + 2] = a.z; } break;
        case SPHMP_F_ALPHA: { const float4 a = alpha_c[i]; f[3 * t] = a.x; f[3 * t + 1] = a.y; f[3 * t + 2] = a.z; } break;
        case SPHMP_F_ALPHA_PRE: { const float4 a = alpha_p[i]; f[3 * t] = a.x; f[3 * t + 1] = a.y; f[3 * t + 2] = a.z; } break;
        case SPHMP_F_DRIFT:
            for (int k = 0; k < 3; k++) {
                const float4 u = B.drift4[(size_t)k * P.cap + i];
                f[9 * t + 3 * k] = u.x; f[9 * t + 3 * k + 1] = u.y; f[9 * t + 3 * k + 2] = u.z;
            }
            break;
        case SPHMP_F_APREV: { const float4 a = S.in[APREV][i]; f[3 * t] = a.x; f[3 * t + 1] = a.y; f[3 * t + 2] = a.z; } break;
        case SPHMP_F_PMOD: f[t] = B.pmod[i]; break;
        case SPHMP_F_VELXCOR: { const float4 x = B.velxcor[i]; f[3 * t] = x.x; f[3 * t + 1] = x.y; f[3 * t + 2] = x.z; } break;
        case SPHMP_F_TYPE: q[t] = p.w < 0.f ? SPHMP_TYPE_BOUNDARY : SPHMP_TYPE_FLUID; break;
        case SPHMP_F_MASS: f[t] = B.mass_raw[o]; break;
        case SPHMP_F_BORNID: q[t] = B.bornid[o]; break;
        default: break;
    }
}

__global__ void __launch_bounds__(kThreads) k_unpack_field(const __grid_constant__ DevParams P,
                                                           const __grid_constant__ DevBuffers B,
                                                           const __grid_constant__ F4Set S, int field,
                                                           float4* alpha_c, float4* alpha_p, const void* stage,
                                                           int n) {
    const int t = blockIdx.x * kThreads + threadIdx.x;  // slot (stage index)
    if (t >= n) return;
    const int i = (int)B.opos[t];                         // internal index
    const float* f = reinterpret_cast<const float*>(stage);
    float4* const __restrict__* out = S.out;
    switch (field) {
        case SPHMP_F_POS: { float4 p = out[POS][i]; p.x = f[3 * t]; p.y = f[3 * t + 1]; p.z = f[3 * t + 2]; out[POS][i] = p; } break;
        case SPHMP_F_VEL: { float4 v = out[VEL][i]; v.x = f[3 * t]; v.y = f[3 * t + 1]; v.z = f[3 * t + 2]; out[VEL][i] = v; } break;
        case SPHMP_F_VELEVAL: { float4 v = out[VEV][i]; v.x = f[3 * t]; v.y = f[3 * t + 1]; v.z = f[3 * t + 2]; out[VEV][i] = v; } break;
        case SPHMP_F_PRESSURE: { float2 d = B.densp[i]; d.y = f[t]; B.densp[i] = d; } break;
        case SPHMP_F_RESTDENS: { float4 a = alpha_c[i]; a.w = f[t]; alpha_c[i] = a; } break;
        case SPHMP_F_VISC: { float4 v = out[VEL][i]; v.w = f[t]; out[VEL][i] = v; } break;
        case SPHMP_F_ACCEL: B.accel4[i] = make_float4(f[3 * t], f[3 * t + 1], f[3 * t + 2], 0.f); break;
        case SPHMP_F_ALPHA: { float4 a = alpha_c[i]; a.x = f[3 * t]; a.y = f[3 * t + 1]; a.z = f[3 * t + 2]; alpha_c[i] = a; } break;
        case SPHMP_F_ALPHA_PRE: { float4 a = alpha_p[i]; a.x = f[3 * t]; a.y = f[3 * t + 1]; a.z = f[3 * t + 2]; alpha_p[i] = a; } break;
        case SPHMP_F_DRIFT:
            for (int k = 0; k < 3; k++)
                B.drift4[(size_t)k * P.cap + i] = make_float4(f[9 * t + 3 * k], f[9 * t + 3 * k + 1], f[9 * t + 3 * k + 2], 0.f);
            break;
        case SPHMP_F_APREV: { float4 a = out[APREV][i]; a.x = f[3 * t]; a.y = f[3 * t + 1]; a.z = f[3 * t + 2]; out[APREV][i] = a; } break;
        case SPHMP_F_PMOD: B.pmod[i] = f[t]; break;
        default: break;
    }
}

inline int blocks_for(int n, int t = kThreads) { return (n + t - 1) / t; }

// Blocks of kThreads that are resident at once on the whole device (for
// kernels that loop over a device-side work count).
template <class K>
int resident_grid(K kernel) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kThreads, 0);
    if (sms <= 0) sms = 1;
    if (per <= 0) per = 1;
    return sms * per;
}

F4Set make_set(const DevBuffers& B, const int* cur, bool to_alt) {
    F4Set S;
    for (int f = 0; f < kNumFloat4Fields; f++) {
        S.in[f] = B.f4[f][cur[f]];
        S.out[f] = B.f4[f][to_alt ? cur[f] ^ 1 : cur[f]];
    }
    return S;
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

void launch_hash(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    cudaMemsetAsync(B.ccount, 0, sizeof(uint32_t) * (size_t)(P.G + 1), s);
    if (P.n <= 0) return;
    k_hash<<<blocks_for(P.n, kHashBlock), kHashBlock, 0, s>>>(P, B, B.f4[POS][cur[POS]]);
}

void launch_cell_starts(const DevParams& P, const DevBuffers& B, cudaStream_t s) {
    const int per = kScanBlock * kScanItems;
    const int nb = (P.G + per - 1) / per;
    const int nchunks = blocks_for(P.n, kHashBlock);
    k_scan_reduce<<<nb, kScanBlock, 0, s>>>(P, B);
    k_scan_top<<<1, kScanBlock, 0, s>>>(P, B, nb, nchunks);
    k_scan_apply<<<nb, kScanBlock, 0, s>>>(P, B);
}

void launch_cell_order(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    const float4* pos_in = B.f4[POS][cur[POS]];
    k_scatter<<<blocks_for(P.n), kThreads, 0, s>>>(P, B);
    const int grid = min(blocks_for(P.G * 32), 152 * 16);
    k_cell_sort<<<grid, kThreads, 0, s>>>(P, B, pos_in);
    k_big_cell_sort<<<64, 1024, 0, s>>>(P, B, pos_in);
}

void launch_grid_list(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    launch_cell_starts(P, B, s);
    launch_cell_order(P, B, cur, s);
}

void launch_rearrange(const DevParams& P, const DevBuffers& B, const int* cur, bool slot_order, cudaStream_t s) {
    if (P.n <= 0) return;
    if (slot_order) k_slot_order<<<blocks_for(P.n), kThreads, 0, s>>>(P, B);
    k_rearrange<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, make_set(B, cur, true));
}

void launch_boundary_volume(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    k_boundary_volume<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]]);
    k_boundary_volume_store<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]]);
}

void launch_density(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    k_density<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]], B.f4[ALPHA][cur[ALPHA]]);
}

void launch_density_oct(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    const float4* pos = B.f4[POS][cur[POS]];
    const float4* alpha = B.f4[ALPHA][cur[ALPHA]];
    cudaMemsetAsync(B.dctr, 0, sizeof(uint32_t), s);
    if (P.ss == 1.0f)
        k_density_bucket<true><<<resident_grid(k_density_bucket<true>), kThreads, 0, s>>>(P, B, pos, alpha);
    else
        k_density_bucket<false><<<resident_grid(k_density_bucket<false>), kThreads, 0, s>>>(P, B, pos, alpha);
    k_expand_lists<<<blocks_for(P.n), kThreads, 0, s>>>(P, B);
}

template <bool F, bool D>
static void fd_dispatch(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    cudaMemsetAsync(&B.hctr[0], 0, sizeof(uint32_t), s);  // the heavy-particle queue's work counter
    const float4* pos = B.f4[POS][cur[POS]];
    const float4* vel = B.f4[VEL][cur[VEL]];
    const float4* al = B.f4[ALPHA][cur[ALPHA]];
    const float4* ap = B.f4[APREV][cur[APREV]];
    const float4* ve = B.f4[VEV][cur[VEV]];
    const int g = blocks_for(P.n);
    if (!D) {
        k_force_drift<F, false, 0><<<g, kThreads, 0, s>>>(P, B, pos, vel, al, ap, ve);
        return;
    }
    switch (P.nphase) {
        case 1: k_force_drift<F, true, 1><<<g, kThreads, 0, s>>>(P, B, pos, vel, al, ap, ve); break;
        case 2: k_force_drift<F, true, 2><<<g, kThreads, 0, s>>>(P, B, pos, vel, al, ap, ve); break;
        default: k_force_drift<F, true, 3><<<g, kThreads, 0, s>>>(P, B, pos, vel, al, ap, ve); break;
    }
}

void launch_force_drift(const DevParams& P, const DevBuffers& B, const int* cur, bool force, bool drift,
                        cudaStream_t s) {
    if (P.n <= 0 || (!force && !drift)) return;
    if (force && drift) fd_dispatch<true, true>(P, B, cur, s);
    else if (force) fd_dispatch<true, false>(P, B, cur, s);
    else fd_dispatch<false, true>(P, B, cur, s);
}

void launch_force_drift_features(const DevParams& P, const DevBuffers& B, const int* cur, float* feat, int32_t* ids,
                                 float vs, float dt_large, cudaStream_t s) {
    if (P.n <= 0) return;
    const float4* pos = B.f4[POS][cur[POS]];
    const float4* vel = B.f4[VEL][cur[VEL]];
    const float4* al = B.f4[ALPHA][cur[ALPHA]];
    const float4* ap = B.f4[APREV][cur[APREV]];
    const float4* ve = B.f4[VEV][cur[VEV]];
    const int g = blocks_for(P.n);
    if (!P.multiphase) {
        k_force_drift_feat<false, 0><<<g, kThreads, 0, s>>>(P, B, pos, vel, al, ap, ve, feat, ids, vs, dt_large);
        return;
    }
    switch (P.nphase) {
        case 1: k_force_drift_feat<true, 1><<<g, kThreads, 0, s>>>(P, B, pos, vel, al, ap, ve, feat, ids, vs, dt_large); break;
        case 2: k_force_drift_feat<true, 2><<<g, kThreads, 0, s>>>(P, B, pos, vel, al, ap, ve, feat, ids, vs, dt_large); break;
        default: k_force_drift_feat<true, 3><<<g, kThreads, 0, s>>>(P, B, pos, vel, al, ap, ve, feat, ids, vs, dt_large); break;
    }
}

void launch_surface_tension(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    k_surface_tension<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]]);
}

void launch_force_projectu(const DevParams& P, const DevBuffers& B, const int* cur, int pre, cudaStream_t s) {
    if (P.n <= 0) return;
    const float4* pos = B.f4[POS][cur[POS]];
    const float4* vel = B.f4[VEL][cur[VEL]];
    const float4* vev = B.f4[VEV][cur[VEV]];
    const float4* ac = B.f4[ALPHA][cur[ALPHA]];
    const float4* ap = B.f4[ALPHA][pre];
    const float4* apv = B.f4[APREV][cur[APREV]];
    const int g = blocks_for(P.n);
    switch (P.nphase) {
        case 1: k_force_projectu<1><<<g, kThreads, 0, s>>>(P, B, pos, vel, vev, ac, ap, apv); break;
        case 2: k_force_projectu<2><<<g, kThreads, 0, s>>>(P, B, pos, vel, vev, ac, ap, apv); break;
        default: k_force_projectu<3><<<g, kThreads, 0, s>>>(P, B, pos, vel, vev, ac, ap, apv); break;
    }
}

void launch_alpha_advance(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    const float4* pos = B.f4[POS][cur[POS]];
    const float4* vev = B.f4[VEV][cur[VEV]];
    const float4* ain = B.f4[ALPHA][cur[ALPHA]];
    float4* aout = B.f4[ALPHA][cur[ALPHA] ^ 1];
    const int g = blocks_for(P.n);
    switch (P.nphase) {
        case 1: k_alpha_advance<1><<<g, kThreads, 0, s>>>(P, B, pos, vev, ain, aout); break;
        case 2: k_alpha_advance<2><<<g, kThreads, 0, s>>>(P, B, pos, vev, ain, aout); break;
        default: k_alpha_advance<3><<<g, kThreads, 0, s>>>(P, B, pos, vev, ain, aout); break;
    }
}

void launch_correction(const DevParams& P, const DevBuffers& B, const int* cur, int pre, cudaStream_t s) {
    if (P.n <= 0) return;
    float4* ac = B.f4[ALPHA][cur[ALPHA]];
    const float4* ap = B.f4[ALPHA][pre];
    float4* vel = B.f4[VEL][cur[VEL]];
    const float4* pos = B.f4[POS][cur[POS]];
    const int g = blocks_for(P.n);
    switch (P.nphase) {
        case 1: k_correction<1><<<g, kThreads, 0, s>>>(P, B, ac, ap, vel, pos); break;
        case 2: k_correction<2><<<g, kThreads, 0, s>>>(P, B, ac, ap, vel, pos); break;
        default: k_correction<3><<<g, kThreads, 0, s>>>(P, B, ac, ap, vel, pos); break;
    }
}

void launch_advance(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    k_advance<<<blocks_for(P.n), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]], B.f4[VEL][cur[VEL]],
                                                    B.f4[VEV][cur[VEV]], B.f4[APREV][cur[APREV]]);
}

void launch_pass_c(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    if (P.n <= 0) return;
    const F4Set S = make_set(B, cur, true);
    const int g = blocks_for(P.n);
    cudaMemsetAsync(&B.hctr[1], 0, sizeof(uint32_t), s);  // the heavy-particle queue's work counter
    if (!P.multiphase) {
        k_pass_c<1, false><<<g, kThreads, 0, s>>>(P, B, S);
        return;
    }
    switch (P.nphase) {
        case 1: k_pass_c<1, true><<<g, kThreads, 0, s>>>(P, B, S); break;
        case 2: k_pass_c<2, true><<<g, kThreads, 0, s>>>(P, B, S); break;
        default: k_pass_c<3, true><<<g, kThreads, 0, s>>>(P, B, S); break;
    }
}

void launch_conservation(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s) {
    cudaMemsetAsync(B.red, 0, sizeof(double) * 16, s);
    if (P.n <= 0) return;
    k_conservation<<<min(blocks_for(P.n), 152 * 8), kThreads, 0, s>>>(P, B, B.f4[POS][cur[POS]],
                                                                      B.f4[ALPHA][cur[ALPHA]]);
}

void launch_set_count(const DevBuffers& B, int n, cudaStream_t s) { k_set_count<<<1, 1, 0, s>>>(B, n); }

void launch_emit(const DevParams& P, const DevBuffers& B, const int* cur, const DevEmitter& E, cudaStream_t s) {
    k_emit<<<1, kScanBlock, 0, s>>>(P, B, make_set(B, cur, false), E);
}

void launch_unpack_aos(const DevParams& P, const DevBuffers& B, const int* cur, const sphmp_display_pack* d,
                       const sphmp_calc_pack* c, int start, int end, cudaStream_t s) {
    if (end <= start) return;
    k_unpack_aos<<<blocks_for(end - start), kThreads, 0, s>>>(P, B, make_set(B, cur, false), d, c, start, end);
}

void launch_pack_aos(const DevParams& P, const DevBuffers& B, const int* cur, sphmp_display_pack* d,
                     sphmp_calc_pack* c, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_pack_aos<<<blocks_for(n), kThreads, 0, s>>>(P, B, make_set(B, cur, false), d, c, n);
}

void launch_pack_field(const DevParams& P, const DevBuffers& B, const int* cur, int field, int alpha_cur,
                       int alpha_pre, void* stage, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_pack_field<<<blocks_for(n), kThreads, 0, s>>>(P, B, make_set(B, cur, false), field,
                                                     B.f4[ALPHA][alpha_cur], B.f4[ALPHA][alpha_pre], stage, n);
}

void launch_unpack_field(const DevParams& P, const DevBuffers& B, const int* cur, int field, int alpha_cur,
                         int alpha_pre, const void* stage, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_unpack_field<<<blocks_for(n), kThreads, 0, s>>>(P, B, make_set(B, cur, false), field,
                                                       B.f4[ALPHA][alpha_cur], B.f4[ALPHA][alpha_pre], stage, n);
}

}  // namespace sphmp
