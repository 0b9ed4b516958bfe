// sphmp_internal.h — device-side data layout and kernel launchers of the
// GB300 multiphase SPH step (shared by sphmp_kernels.cu and sphmp_api.cu).
//
// Particle state lives in HBM as structure-of-arrays in an internal order: the
// in-grid particles grouped by the reference's 2h cell (cell c occupies the same
// index range [cstart[c], cstart[c+1]) as its slots in the reference's sorted
// order) and, inside a cell, by h-subcell (octant); out-of-grid particles follow
// in slot order. opos[slot] and oidx[index] map between the reference's slots
// and internal indices; every reference-facing array (mgcell, midsort, mgndx,
// mgridoff, mgridcnt) and every transfer is in slot order. Every per-particle
// array that survives a step is a float4 so neighbour gathers are single
// 16-byte loads, and each is double-buffered: a pass that moves or advances
// particles reads buffer `cur` and writes buffer `cur ^ 1`.
//
//   pos4   : x, y, z (sim units), w = mass (fluid) or -V_b (boundary volume)
//   vel4   : vx, vy, vz, visc
//   vev4   : veleval x, y, z, (unused)
//   alpha4 : alpha_0, alpha_1, alpha_2, restdens
//   aprev4 : gravity - total accel of the last advance (x, y, z), w = origin slot
//            (bits of a uint32: the slot the particle was uploaded to)
//
// Per-step arrays (single buffer): densp (1/rho or V_b, pressure), accel4,
// drift4 (phase-major: drift of phase k for slot i at [k * cap + i]), pmod,
// velxcor (XSPH correction of the project-U force).
// Per-origin arrays (never moved): color, bornid, raw calc mass.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sphmp.h"
#include "sphmp_learned.h"

namespace sphmp {

constexpr uint32_t kUndef = 0xFFFFFFFFu;
constexpr int kHashBlock = 256;       // threads per hash block (= one chunk for out-of-grid ranks)
constexpr int kScanBlock = 1024;      // threads per scan block
constexpr int kScanItems = 4;         // items per thread in the scan
constexpr int kWarpSortMax = 256;     // cells up to this size are sorted by one warp
constexpr int kCtaSortMax = 8192;     // larger cells up to this size are sorted by one CTA
constexpr int kNumFloat4Fields = 5;   // pos4, vel4, vev4, alpha4, aprev4
constexpr int kMaxNbr = 256;          // index-list capacity per particle (more: the passes rescan)
constexpr int kNrecFloat4 = 5;        // float4 per neighbour record of the alpha pass
// Bucket neighbour lists: a bitmask over the bucket's candidate sequence (the 27
// h-subcells around it as 18 index ranges), one word per 32 candidates.
constexpr int kMaskWords = 64;        // mask words per particle (more candidates: the passes rescan)
constexpr int kTabStride = 40;        // per bucket: [0..18] range ends in the sequence, [20..37] index - sequence
constexpr uint32_t kBucketWindow = 32;  // largest member window of one density work item (one member per lane)
constexpr uint32_t kBucketWindowMin = 8;
constexpr uint32_t kMaskList = 0x80000000u;  // nbr_cnt flag: bucket mask list, low bits = bucket (cell * 8 + octant)
constexpr uint32_t kRescan = 0x7fffffffu;    // nbr_cnt value: no list, search the cells
// Heavy particles (long lists, overflowed lists, cell searches) are queued in hq by
// the list expansion and taken by whole warps in the force and alpha passes; an
// index list of a heavy particle carries this flag over its length.
constexpr uint32_t kHeavyFlag = 0x40000000u;
constexpr uint32_t kHeavyList = 128;         // default: index lists longer than this are heavy

// Error bits accumulated in the device error word (1 << sphmp_status).
constexpr uint32_t kErrCellOverflow = 1u << SPHMP_ERR_CELL_OVERFLOW;
constexpr uint32_t kErrType = 1u << SPHMP_ERR_UNSUPPORTED_TYPE;
constexpr uint32_t kErrNotFinite = 1u << SPHMP_ERR_NOT_FINITE;
constexpr uint32_t kErrBadMass = 1u << SPHMP_ERR_BAD_MASS;
constexpr uint32_t kErrCapacity = 1u << SPHMP_ERR_CAPACITY;

// Scalars every kernel needs, passed by value.
struct DevParams {
    int n;           // launch size: the active slots, or the capacity while a device emitter runs
                     // (kernels bound themselves by the device counter, active_n)
    int cap;         // capacity (stride of phase-major arrays)
    int G;           // grid cells
    int rx, ry, rz;  // grid resolution
    float gmin[3];
    float fac[3];    // gridIdfac
    float srad[3];   // search radius h/simscale in cell units per axis, plus a rounding margin
    float ss;        // simscale
    float h, r2;     // smoothing radius and its square
    float r2list;    // squared radius of the neighbour list (r2 plus a rounding margin)
    int list_mode;   // 0: no list, 1: index lists in nbr (written by the last density pass)
    int narrow;      // 1: positions are the ones the cell lists were built from (the cell
                     // search may skip the cells beyond h of the current position)
    float dt;
    float kpoly6, kspikydiff;
    float kspline;   // 1 / (pi h^3), the cubic spline of the IISPH step
    float bvisc;
    float grav[3];
    int nphase;
    int multiphase;
    float dens_k[3], visc_k[3];
    float relax, sigma, cont, cont1, cont2, pintstiff;
    float omega, visc_factor;  // boundary factors of the project-U force
    int eos;
    float eos_k;
    int st_on;
    float st_K, st_C;
    int neighborid[27];
    int morton;      // 1: cells in Z-order in the sorted arrays (corder), 0: the reference's linear order
    int bwin;        // members per work item of the bucket density pass (8..32)
    uint32_t heavy;  // index lists longer than this are heavy (queued in hq)
};

struct DevBuffers {
    float4* f4[kNumFloat4Fields][2];  // pos4, vel4, vev4, alpha4, aprev4 double buffers
    float2* densp;
    float4* accel4;
    float4* drift4;   // [3 * cap]
    float4* velxcor;  // [cap] XSPH velocity correction of the project-U force
    float* pmod;
    uint32_t* mgcell;   // sorted cell id per slot (unsorted key after the hash)
    uint32_t* midsort;  // pre-sort slot of each sorted slot
    uint32_t* mgndx;    // rank in cell
    int32_t* mgridoff;  // [G]
    int32_t* mgridcnt;  // [G]
    uint32_t* key;      // [cap] unsorted cell key per slot
    uint8_t* octk;      // [cap] octant (h-subcell inside the cell) per slot, in-grid slots only
    uint32_t* arank;    // [cap] rank inside the bin (atomic order; exact for out-of-grid)
    uint32_t* sidx;     // [cap] scatter target (pre-sort slots grouped by cell)
    uint32_t* ccount;   // [G + 1] histogram, bin G = out-of-grid
    uint32_t* cstart;   // [G + 2] exclusive scan of ccount in the cell order; cstart[G] = in-grid count,
                        // cstart[G+1] = n
    uint32_t* cend;     // [G] end of each cell's range (cstart[c + 1] in the linear order only)
    uint32_t* corder;   // [G] cells in Z-order (the scan order of the Morton mode)
    uint32_t* bsum;     // [nblocks] scan block sums
    uint32_t* uchunk;   // [cap / kHashBlock + 1] out-of-grid count per hash chunk, scanned in place
    uint32_t* big;      // [cap / (kWarpSortMax+1) + 2]: big[0] = count, then big cell ids
    float4* color;      // [cap] per origin
    int32_t* bornid;    // [cap] per origin
    float* mass_raw;    // [cap] per origin
    uint32_t* err;      // device error word
    double* red;        // [16] FP64 reduction results
    float* vtmp;        // [cap] scratch (boundary volumes)
    uint32_t* nbr;      // [kMaxNbr * cap] neighbour indices, groups of 4 column-major: entry k of s at ((k / 4) * cap + s) * 4 + k % 4
    uint32_t* nbr_cnt;  // [cap] list of particle s: kMaskList | bucket, index count (<= kMaxNbr) or kRescan
    uint32_t* nmask;    // [kMaskWords * cap] bucket mask lists, column-major: word k of particle s at k * cap + s
    uint32_t* btab;     // [8 * G * kTabStride] candidate ranges of each bucket with a mask list
    uint32_t* dctr;     // [1] work counter of the bucket density kernel
    uint2* wq;          // [cap / kBucketWindowMin + 16] member windows after the first of large buckets:
                        // x = bucket (cell * 8 + octant), y = first member (internal index)
    uint32_t* wq_n;     // [1] entries in wq (cleared by the scan, filled by the cell sort)
    uint32_t* hq;       // [cap] heavy particles (internal index), filled by the list expansion
    uint32_t* hq_n;     // [1] entries in hq (cleared by the scan)
    uint32_t* hctr;     // [2] work counters over hq of the force and the alpha pass
    // IISPH step (sphmp_iisph.cu): d_ii, sum_j d_ij p_j (float4, w unused), a_ii, the
    // predicted density, the pressure iterates p_l and p_l+1, the density residue
    float4* iis_dii;
    float4* iis_dijpj;
    float* iis_aii;
    float* iis_rho_adv;
    float* iis_pl;
    float* iis_pl1;
    float* iis_res;
    float4* nrec;       // [kNrecFloat4 * cap] neighbour records of the alpha pass (written by force + drift)
    // Internal order: inside every 2h cell, members grouped by the h-subcell
    // (octant) they occupy, octant index (oy * 2 + oz) * 2 + ox.
    uint32_t* opos;     // [cap] internal index of each reference slot
    uint32_t* oidx;     // [cap] reference slot of each internal index (after the last sort)
    uint32_t* osrc;     // [cap] previous internal index of each new internal index (sort -> rearrange)
    uint32_t* oct_start;// [8 * G] first internal index of bucket (cell, octant)
    uint32_t* act;      // [G] cells with members (any order)
    uint32_t* act_n;    // [1] number of entries in act
    int32_t* nact;      // [1] active slots (device-side emission grows it inside a step)
    int32_t* frame;     // [1] steps since the device emitter was set
    uint32_t* esum;     // [1] scratch of the emission kernel
};

// Device-side disk emitter (the reference's EmitParticles, run before the sort
// of every step whose frame is a multiple of `interval`).
struct DevEmitter {
    float rot[3][3];   // columns (newx, dir, newz) of EmitImmediate's rotation
    float pos[3];
    float dir[3];
    float vel, radius, spacing, jitter;
    float mass, restdens, visc;  // of the emitted phase (massArr, densArr, viscArr)
    unsigned long long seed;
    int res;           // sites per half axis: int(radius / spacing)
    int layers, interval;
    int onehot;        // volume-fraction phase: the first whose rest density is `restdens`
};

#ifdef __CUDACC__
// The active slot count every kernel bounds itself by.
__device__ __forceinline__ int active_n(const DevBuffers& B) { return *B.nact; }
#endif

enum Field4 { POS = 0, VEL = 1, VEV = 2, ALPHA = 3, APREV = 4 };

// Input and output buffers of the five float4 fields for one kernel launch.
struct F4Set {
    const float4* __restrict__ in[kNumFloat4Fields];
    float4* __restrict__ out[kNumFloat4Fields];
};

// Record the text returned by sphmp_last_error on the calling thread (sphmp_api.cu).
sphmp_status record_error(sphmp_status st, const char* msg);

// ---- launchers (sphmp_kernels.cu) ----
// All take the current double-buffer selectors in `cur` (one per Field4).
void launch_hash(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
// (reads the pre-sort positions pos4[cur[POS]] to build the next internal order)
void launch_grid_list(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
// the two halves of launch_grid_list: cell starts (histogram scan), then the
// scatter, the per-cell stable ordering and the per-cell octant order
void launch_cell_starts(const DevParams& P, const DevBuffers& B, cudaStream_t s);
void launch_cell_order(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
// move every particle to its new internal index (osrc) and update opos; with
// `slot_order`, the new internal order is the reference's sorted slot order
// (for a rearrange that did not follow this library's grid list)
void launch_rearrange(const DevParams& P, const DevBuffers& B, const int* cur, bool slot_order, cudaStream_t s);
void launch_boundary_volume(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
void launch_density(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
// octant-order density (needs the octant order of this sort); writes slot lists
void launch_density_oct(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
void launch_force_drift(const DevParams& P, const DevBuffers& B, const int* cur, bool force, bool drift,
                        cudaStream_t s);
void launch_surface_tension(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
// project-U force: start-of-step fractions in alpha4[pre], rest densities in alpha4[cur[ALPHA]]
void launch_force_projectu(const DevParams& P, const DevBuffers& B, const int* cur, int pre, cudaStream_t s);
// alpha advance: reads alpha4[cur], writes alpha4[cur^1] (new fractions, same restdens)
void launch_alpha_advance(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
// correction: fractions in alpha4[cur[ALPHA]], start-of-step fractions in alpha4[pre]; in place
void launch_correction(const DevParams& P, const DevBuffers& B, const int* cur, int pre, cudaStream_t s);
// advance in place on the cur buffers
void launch_advance(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
// fused alpha + correction + advance: reads cur, writes cur^1 for all five float4 fields
void launch_pass_c(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
void launch_conservation(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
// IISPH step (sphmp_iisph.cu): density (densp.x = rho), PredictAdvection (veleval,
// d_ii, rho_adv, p_l = p / 2, a_ii), one pressure iteration (dijpj, p_l1, residue,
// accel, pressure, then p_l = p_l1; FP64 residue sums in red[8..10]), integration
void launch_iisph_density(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
void launch_iisph_predict(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
void launch_iisph_iteration(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
void launch_iisph_integrate(const DevParams& P, const DevBuffers& B, const int* cur, cudaStream_t s);
// set the device counter of active slots
void launch_set_count(const DevBuffers& B, int n, cudaStream_t s);
// device-side emission into the current buffers (one block)
void launch_emit(const DevParams& P, const DevBuffers& B, const int* cur, const DevEmitter& E, cudaStream_t s);

// learned large step: the force (+ drift) pass that also fills the corrector's
// features of every particle (feat [n][48], ids = bornid, -1 without features;
// sphmp_kernels.cu), and the correction of the step's result by the network
// outputs y [n][4] (sphmp_learned.cu)
void launch_force_drift_features(const DevParams& P, const DevBuffers& B, const int* cur, float* feat, int32_t* ids,
                                 float vs, float dt_large, cudaStream_t s);
void launch_apply_correction(const DevParams& P, const DevBuffers& B, const int* cur, const float* y,
                             const float* out_scale, const int32_t* ids, float dt_large, float* corr, cudaStream_t s);

// differences of state b against state a (see sphmp_compare_states); map: scratch of map_size
// entries (bornid -> index of a), out: 7 doubles (6 sums, then the maximum)
void launch_compare(const DevParams& Pa, const DevBuffers& Ba, const int* cur_a, const DevParams& Pb,
                    const DevBuffers& Bb, const int* cur_b, int32_t* map, int map_size, double* out, cudaStream_t s);

// transfers (staging buffers hold reference records)
void launch_unpack_aos(const DevParams& P, const DevBuffers& B, const int* cur, const sphmp_display_pack* d,
                       const sphmp_calc_pack* c, int start, int end, cudaStream_t s);
void launch_pack_aos(const DevParams& P, const DevBuffers& B, const int* cur, sphmp_display_pack* d,
                     sphmp_calc_pack* c, int n, cudaStream_t s);
// field pack/unpack through a float/uint32 staging array; `aux` = alpha_pre buffer selector
void launch_pack_field(const DevParams& P, const DevBuffers& B, const int* cur, int field, int alpha_cur,
                       int alpha_pre, void* stage, int n, cudaStream_t s);
void launch_unpack_field(const DevParams& P, const DevBuffers& B, const int* cur, int field, int alpha_cur,
                         int alpha_pre, const void* stage, int n, cudaStream_t s);

// the corrector network as the large step uses it (sphmp_learned.cu)
cudaError_t corrector_forward_on(sphmp_corrector* c, const float* x, int n, float* y, uint32_t* err, cudaStream_t s);
const float* corrector_out_scale(const sphmp_corrector* c);  // device [4]
int corrector_device(const sphmp_corrector* c);

}  // namespace sphmp
