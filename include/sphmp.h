/*
 * sphmp.h — C ABI of the GB300-native multiphase SPH step.
 *
 * This is the drop-in boundary for the per-step particle pipeline of
 * ZP-Z/sph-multiphase: uniform-grid hashing, stable counting sort, reorder,
 * density + equation-of-state pressure, pressure/viscosity/boundary (and
 * optional surface-tension) forces, drift-flux drift velocity, volume-fraction
 * advance and correction, and symplectic-Euler advection.
 *
 * Two layers are exported:
 *   1. a handle-based API (sphmp_*) that owns device buffers per context and
 *      returns a status code from every call;
 *   2. the reference's own entry-point names (GetParticleIndexCUDA, ...) as
 *      thin `void` wrappers over one default context, declared in
 *      sphmp_legacy.h.
 *
 * All pointers in this header are host pointers unless stated otherwise.
 * No CUDA or torch types appear in the signatures; a CUDA stream is passed as
 * an opaque `void*` (a cudaStream_t).
 */
#ifndef SPHMP_H
#define SPHMP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHMP_MAX_PHASES 3        /* reference MAX_FLUIDNUM, SPH_Solver/common_header.h:17 */
#define SPHMP_GRID_UNDEF 0xFFFFFFFFu /* reference GRID_UNDEF, SPH_Solver/fluids/fluid_system_kern.cuh:18 */

#define SPHMP_TYPE_FLUID 0        /* SPH_Solver/common_header.h:20 */
#define SPHMP_TYPE_BOUNDARY 1     /* SPH_Solver/common_header.h:21 */

typedef enum sphmp_status {
    SPHMP_OK = 0,
    SPHMP_ERR_INVALID_ARG = 1,     /* null pointer, bad size, bad enum */
    SPHMP_ERR_CAPACITY = 2,        /* n > capacity fixed at create */
    SPHMP_ERR_CUDA = 3,            /* a CUDA runtime call failed */
    SPHMP_ERR_UNSUPPORTED_TYPE = 4,/* particle type other than fluid(0)/boundary(1) */
    SPHMP_ERR_NOT_FINITE = 5,      /* NaN/Inf in uploaded positions or params */
    SPHMP_ERR_CELL_OVERFLOW = 6,   /* one grid cell holds more particles than the sort supports */
    SPHMP_ERR_STATE = 7,           /* call order violated (e.g. force before sort) */
    SPHMP_ERR_NO_DEVICE = 8,       /* no CUDA device / extension not loadable */
    SPHMP_ERR_BAD_MASS = 9,        /* fluid particle with mass <= 0 */
    SPHMP_ERR_GRID = 10,           /* grid parameters inconsistent (res < 3, total overflow) */
    SPHMP_ERR_TIMEOUT = 11         /* a bounded device wait ran out (a tensor-core chain did not complete) */
} sphmp_status;

/* Equation of state used by the density pass. */
typedef enum sphmp_eos {
    SPHMP_EOS_TAIT = 0,   /* p = 2.5*rho0*((rho/rho0)^7 - 1), clamped >= 0
                             (SPH_Solver/fluids/fluid_system_kern.cu:310-313) */
    SPHMP_EOS_LINEAR = 1  /* p = k*(rho - rho0), clamped >= 0 (the commented
                             linear form at fluid_system_kern.cu:308, k = eos_stiffness) */
} sphmp_eos;

/* Order in which one step composes the per-pass functions. */
typedef enum sphmp_schedule {
    /* sort, density, [drift, alpha, correction], force, advance: the reference's
       call order (legacy multiphase step SPH_Solver/fluids/fluid_system.cpp:375-420,
       plain step :514-539), one kernel per function. */
    SPHMP_SCHEDULE_REFERENCE = 0,
    /* sort, density+pressure, force+drift, alpha+correction+advance: three
       neighbour passes. The force reads the mixture rest density and viscosity
       from before this step's correction (the correction lands one step later
       in the force); everything else is identical to the reference order. */
    SPHMP_SCHEDULE_FUSED = 1,
    /* the legacy multiphase step as RunSimulateMultiCUDAFull writes it
       (SPH_Solver/fluids/fluid_system.cpp:375-420): sort, density, drift, alpha
       advance, correction, then the project-U force (ComputeForce_projectu,
       SPH_Solver/fluids/multiphase.cu:488-616) in place of MfComputeForce, then
       the advance; needs `multiphase` = 1. */
    SPHMP_SCHEDULE_PROJECTU = 2
} sphmp_schedule;

/*
 * Parameters. The first 464 bytes are byte-compatible with the reference's
 * `ParamCarrier` (SPH_Solver/common_header.h:28-109), so a caller holding a
 * ParamCarrier can copy it over the prefix. The fields after `fBlending` are
 * extensions for the multiphase kernels (whose constants lived in the removed
 * legacy `FluidParams simData`) and for this implementation.
 */
/* Order of the cells in the sorted particle arrays. LINEAR is the reference's
   key order, (gy * rz + gz) * rx + gx (fluid_system_kern.cu:55), and is the only
   order whose midsort / mgridoff are bit-identical to GetGridListCUDA's. MORTON
   sorts the same cells by the Z-order (bit-interleaved) code of (gx, gy, gz):
   every cell holds the same particles in the same order as in LINEAR mode
   (mgcell per particle, mgridcnt and mgndx are unchanged), only the sequence of
   the cells in the sorted arrays differs, so that neighbouring cells sit close
   in memory along all three axes. Caller-supplied sort arrays (uploads of
   SPHMP_F_MIDSORT / SPHMP_F_MGRIDCNT) are refused in MORTON mode. */
typedef enum sphmp_cell_order {
    SPHMP_CELL_ORDER_LINEAR = 0,
    SPHMP_CELL_ORDER_MORTON = 1
} sphmp_cell_order;

typedef struct sphmp_params {
    /* environment */
    float acclimit;
    float vlimit;
    float gravity[3];
    float volmin[3];
    float volmax[3];
    float softminx[3];
    float softmaxx[3];
    /* case */
    int32_t num;        /* active particle slots */
    int32_t maxNum;     /* capacity */
    float dt;
    float simscale;
    /* fluid */
    float viscosity;
    float restdensity;
    float mass;
    float radius;
    float smoothradius;
    float scalep;
    float massArr[SPHMP_MAX_PHASES];
    float densArr[SPHMP_MAX_PHASES];  /* per-phase rest density (mf_dens) */
    float viscArr[SPHMP_MAX_PHASES];  /* per-phase viscosity (mf_visc) */
    float boundstiff;
    /* sph kernel constants (derived by sphmp_setup_constants) */
    float kpoly6;
    float kspiky;
    float kspikydiff;
    float klaplacian;
    float kspline;
    /* boundary particles */
    float bmass;
    float bRestdensity;
    float bvisc;
    /* index-sort grid (derived by sphmp_setup_grid) */
    float cellsize;
    int32_t searchnum;
    int32_t neighbornum;
    int32_t neighborid[27];
    float gridmin[3];
    float gridmax[3];
    float gridsize[3];
    float gridIdfac[3];
    int32_t gridres[3];
    int32_t gridtotal;
    /* MPM grid, solid, Drucker-Prager, FLIP: carried for layout only, unused */
    float mpmcellsize;
    float mpmXmin[3];
    float mpmXmax[3];
    int32_t mpmRes[3];
    int32_t mpmNodeNum;
    float solidK;
    float solidG;
    float a_phi;
    float a_psi;
    float k_c;
    float w_deltax;
    float fijn;
    float SFlipControl;
    float LFlipControl;
    int32_t mpmSplitNum;
    float collisionStiff;
    float surfaceTensionK;       /* tension radius factor K (radius = K*h) */
    float surfaceTensionFluidC;  /* cohesion coefficient C */
    float fBlending;
    /* ---- extensions (offset 464) ---- */
    int32_t nphase;              /* mf_catnum: number of phases, 1..3 */
    int32_t multiphase;          /* 1: run drift / alpha / correction in sphmp_step */
    int32_t surface_tension;     /* 1: add the reference SurfaceTension term in the force pass */
    int32_t eos;                 /* sphmp_eos */
    float eos_stiffness;         /* k for SPHMP_EOS_LINEAR */
    float mf_relax;              /* drift relaxation time coefficient (simData.relax) */
    float mf_diffusion;          /* alpha-gradient diffusion sigma (simData.mf_diffusion) */
    float mf_cont;               /* simData.cont */
    float mf_cont1;              /* simData.cont1 (diffusion term switch) */
    float mf_cont2;              /* simData.cont2 (pressure term switch) */
    float mf_pintstiff;          /* simData.pintstiff (pressure-correction stiffness) */
    float mf_omega;              /* simData.omega: boundary pressure factor of the project-U force */
    float mf_visc_factor;        /* simData.visc_factor: boundary viscosity factor of the project-U force */
    int32_t cell_order;          /* sphmp_cell_order: order of the cells in the sorted arrays */
    int32_t bucket_window;       /* members of one h-subcell per work item of the density pass, 8..32 (0: 32) */
    int32_t heavy_list;          /* neighbour lists longer than this are walked by a whole warp, 32..256 (0: 128) */
} sphmp_params;

/* Byte-compatible copies of the reference records (SPH_Solver/common_header.h:112-137). */
typedef struct sphmp_display_pack {
    float pos[3];
    float color[4];
    int32_t type;
} sphmp_display_pack; /* 32 bytes */

typedef struct sphmp_calc_pack {
    float vel[3];
    float veleval[3];
    float pressure;
    float dens;       /* fluid: 1/rho; boundary: particle volume V_b */
    float restdens;
    float mass;
    float visc;
    int32_t bornid;
    float accel[3];
    float deformGrad[9]; /* solid/MPM fields: carried for layout only */
    float stress[9];
    float B[9];
    float solidG;
    float solidK;
    float X[3];
    float invA[9];
} sphmp_calc_pack; /* 224 bytes */

/* Per-particle / per-cell arrays addressable by sphmp_upload_field / sphmp_download_field.
   Element layouts follow the reference: vectors are 3 consecutive floats per
   particle, phase arrays use the MAX_FLUIDNUM stride (3 floats per particle),
   drift velocities are 3 phases x 3 floats per particle (mf_vel_phrel[i*3+k]). */
typedef enum sphmp_field {
    SPHMP_F_POS = 0,       /* float[3n] */
    SPHMP_F_VEL = 1,       /* float[3n] */
    SPHMP_F_VELEVAL = 2,   /* float[3n] */
    SPHMP_F_PRESSURE = 3,  /* float[n]  */
    SPHMP_F_DENS = 4,      /* float[n]  1/rho (fluid) or V_b (boundary); download only */
    SPHMP_F_RESTDENS = 5,  /* float[n]  */
    SPHMP_F_VISC = 6,      /* float[n]  */
    SPHMP_F_ACCEL = 7,     /* float[3n] */
    SPHMP_F_ALPHA = 8,     /* float[3n] mf_alpha (after the alpha advance) */
    SPHMP_F_ALPHA_PRE = 9, /* float[3n] mf_alpha_pre (start-of-step fractions) */
    SPHMP_F_DRIFT = 10,    /* float[9n] mf_vel_phrel */
    SPHMP_F_APREV = 11,    /* float[3n] mforce: gravity - total accel of the last advance */
    SPHMP_F_PMOD = 12,     /* float[n]  mf_pressure_modify */
    SPHMP_F_TYPE = 13,     /* int32[n]  download only */
    SPHMP_F_MASS = 14,     /* float[n]  download only */
    SPHMP_F_BORNID = 15,   /* int32[n]  download only */
    SPHMP_F_MGCELL = 16,   /* uint32[n] cell id per slot */
    SPHMP_F_MIDSORT = 17,  /* uint32[n] pre-sort slot of each sorted slot */
    SPHMP_F_MGNDX = 18,    /* uint32[n] rank inside its cell (GRID_UNDEF for out-of-grid slots) */
    SPHMP_F_MGRIDOFF = 19, /* int32[gridtotal] first slot of each occupied cell, 0 if empty */
    SPHMP_F_MGRIDCNT = 20, /* int32[gridtotal] particle count per cell */
    SPHMP_F_VELXCOR = 21,  /* float[3n] mf_velxcor: XSPH velocity correction of the project-U force
                              (0 for boundary and out-of-grid slots); download only */
    SPHMP_F_COUNT = 22
} sphmp_field;

typedef struct sphmp_ctx sphmp_ctx;

/* ---- host-side setup (reference FluidSystem setup, SPH_Solver/fluids/fluid_system.cpp) ---- */

/* Fill every field with the defaults of a water-like single-phase scene. */
sphmp_status sphmp_params_default(sphmp_params* p);
/* SPH kernel constants from smoothradius, and cellsize = 2h
   (reference SetupSimpleSphCase, fluid_system.cpp:308-313). */
sphmp_status sphmp_setup_constants(sphmp_params* p);
/* Grid resolution, cell index factors and the 27-neighbour offsets from
   volmin/volmax/cellsize/simscale (reference SetupGrid, fluid_system.cpp:119-145). */
sphmp_status sphmp_setup_grid(sphmp_params* p);

/* Append a fluid block on a lattice (reference AddFluidVolume,
   fluid_system.cpp:719-762, with the jitter drawn from a seeded generator
   instead of rand()). Writes at most `cap - *count` particles into the host
   arrays starting at index *count and advances *count. */
sphmp_status sphmp_add_fluid_volume(const sphmp_params* p, const float vmin[3], const float vmax[3],
                                    float spacing, const float offs[3], int32_t phase, float jitter,
                                    uint64_t seed, sphmp_display_pack* disp, sphmp_calc_pack* calc,
                                    int32_t cap, int32_t* count);
/* Append a boundary wall lattice (reference SetupAddWall, SPH_Solver/fluids/AddShape.cpp:306-353). */
sphmp_status sphmp_add_wall(const sphmp_params* p, const float vmin[3], const float vmax[3],
                            sphmp_display_pack* disp, sphmp_calc_pack* calc, int32_t cap, int32_t* count);
/* Append an open box of five walls (reference SetupAddOpenBox, AddShape.cpp:355-366). */
sphmp_status sphmp_add_open_box(const sphmp_params* p, const float vmin[3], const float vmax[3],
                                float thickness, sphmp_display_pack* disp, sphmp_calc_pack* calc,
                                int32_t cap, int32_t* count);
/* A disk emitter (the reference's ParticleEmitter, SPH_Solver/fluids/fluid_system.h:30-40). */
typedef struct sphmp_emitter {
    float position[3];
    float dir[3];      /* unit emission direction */
    float vel;         /* emission speed */
    float radius;
    float spacing;
} sphmp_emitter;
/* Append `layers` emitted disks (FluidSystem::EmitParticles / EmitImmediate /
   InsertParticles, SPH_Solver/fluids/fluid_system.cpp:619-700) as fluid of `phase`:
   lattice sites within `radius` of the centre in the plane normal to dir, with
   a seeded in-plane jitter of +-jitter/2 spacings (the reference uses 1 and
   rand()), layer k shifted by k spacings along +y, velocity dir * vel, colour
   (frame/200, 0.5, 0.8, 0.5). Upload the new records with sphmp_emit_aos
   (EmitUpdateCUDA). */
sphmp_status sphmp_emit_disk(const sphmp_params* p, const sphmp_emitter* e, int32_t layers, int32_t phase,
                             int32_t frame, float jitter, uint64_t seed, sphmp_display_pack* disp,
                             sphmp_calc_pack* calc, int32_t cap, int32_t* count);
/* Device-side emission (FluidSystem::EmitParticles, SPH_Solver/fluids/fluid_system.cpp:619-641,
   where the host inserts particles every emitInterval frames and re-uploads them with
   EmitUpdateCUDA): from now on every sphmp_step starts by appending, when its frame
   (steps since this call, from 0) is a multiple of `interval`, the particles that
   sphmp_emit_disk(params, e, layers, phase, frame, jitter, seed + frame, ...) would
   produce, bit for bit, after the active slots, and the particle count grows on the
   device, inside the captured step graph (no host round trip, no re-capture). The
   kernels then run over the capacity and bound themselves by the device count;
   sphmp_num_particles, the transfers and sphmp_sync read the count back. At capacity
   the remaining sites are dropped, as the reference's AddParticle does, and
   sphmp_device_errors reports SPHMP_ERR_CAPACITY. `e` NULL or interval <= 0 turns
   the emitter off. */
sphmp_status sphmp_set_device_emitter(sphmp_ctx* ctx, const sphmp_emitter* e, int32_t layers, int32_t phase,
                                      int32_t interval, float jitter, uint64_t seed);
/* Boundary lattice spacing (bmass/bRestdensity)^(1/3)/simscale (AddShape.cpp:265-271). */
float sphmp_boundary_spacing(const sphmp_params* p);

/* ---- particle data formats (host only) ---- */

/* Text frame dump of the reference's FluidSystem::outputFile
   (SPH_Solver/fluids/FluidIOUtility.cpp:17-38): the count on the first line, then
   per record "x y z mass restdens type" in printf %f / %d form. */
sphmp_status sphmp_write_frame_text(const char* path, const sphmp_display_pack* disp,
                                    const sphmp_calc_pack* calc, int32_t n);

/* Header of a BINX-020 (.bi2) particle file (SPH_Solver/catpaw/BI2Reader.h:20-58). */
typedef struct sphmp_bi2_info {
    int32_t fmt, bitorder, full, data2d;
    float dp, h, b, rhop0, gamma, massbound, massfluid, time;
    int32_t np, nfixed, nmoving, nfloat, nfluidout, nbound, nfluid;
} sphmp_bi2_info;

/* Read a BINX-020 file as the reference's BI2Reader::GetInfo(false) does
   (SPH_Solver/catpaw/BI2Reader.cpp:19-106), converting the byte order when it
   differs from the host's. Fills `info`; when any of pos (3 floats per
   particle), vel (3 floats) or rhop (1 float) is non-NULL, also fills those
   arrays for info->np particles (cap >= np), with zero for particles the file
   does not carry (the fixed ones of a short file, fluid that left). Unlike the
   reference, a file that is not BINX-020 or has inconsistent counts is an error. */
sphmp_status sphmp_read_bi2(const char* path, sphmp_bi2_info* info, float* pos, float* vel, float* rhop,
                            int32_t cap);

/* Append the particles of a .bi2 shape as fluid of `phase` (the reference's
   FluidSystem::AddShape, SPH_Solver/fluids/fluid_system.cpp:809-835, which uses
   scale 0.005, velocity (0, -1.5, 0) and the third phase): position (x, y, z)
   of the file becomes (x, z, y) / scale + offs. */
sphmp_status sphmp_add_bi2_shape(const sphmp_params* p, const float* pos, int32_t np, float scale,
                                 const float offs[3], const float vel[3], int32_t phase,
                                 sphmp_display_pack* disp, sphmp_calc_pack* calc, int32_t cap, int32_t* count);

/* ---- context lifetime (reference FluidSetupCUDA / FluidClearCUDA, fluid_system_host.cu:79-144) ---- */

/* Allocate device buffers for p->maxNum particles and p->gridtotal cells on the
   current CUDA device. The params are copied (reference CarryParam). */
sphmp_status sphmp_create(const sphmp_params* p, sphmp_ctx** out);
sphmp_status sphmp_destroy(sphmp_ctx* ctx);
/* Replace the parameters (reference CarryParam, fluid_system_kern.cu:22-25).
   maxNum and the grid size may not grow beyond what create allocated. */
sphmp_status sphmp_set_params(sphmp_ctx* ctx, const sphmp_params* p);
sphmp_status sphmp_get_params(const sphmp_ctx* ctx, sphmp_params* p);
/* Run all later work of this context on `stream` (a cudaStream_t; NULL = the
   context's own stream). */
sphmp_status sphmp_set_stream(sphmp_ctx* ctx, void* stream);
/* Wait for the context's work; returns the first device error recorded since the
   last check (and clears it). */
sphmp_status sphmp_sync(sphmp_ctx* ctx);
/* Active particle slots (read back from the device after steps with a device
   emitter, which waits for the context's stream); 0 for NULL, -1 if that read fails. */
int32_t sphmp_num_particles(const sphmp_ctx* ctx);

/* ---- host transfers (reference TransferToCUDA / TransferFromCUDA / EmitUpdateCUDA,
        SPH_Solver/fluids/fluid_system.cpp:979-999) ---- */

/* Upload n reference records into slots [0, n) and set num = n. Multiphase
   arrays are initialised one-hot from `phase` = 0 unless uploaded later. */
sphmp_status sphmp_upload_aos(sphmp_ctx* ctx, const sphmp_display_pack* disp,
                              const sphmp_calc_pack* calc, int32_t n);
/* Download slots [0, n) in the current (sorted) slot order. `calc` may be NULL
   (the reference's per-frame TransferFromCUDA copies display records only). */
sphmp_status sphmp_download_aos(sphmp_ctx* ctx, sphmp_display_pack* disp,
                                sphmp_calc_pack* calc, int32_t n);
/* Asynchronous TransferFromCUDA: queue, after the work already on the context
   stream, a download of the n display records into `disp` and return at once.
   The copy runs on a separate stream, so it overlaps whatever is queued next
   (the following steps); `disp` must stay valid and unread until
   sphmp_download_wait (or sphmp_sync) returns, and should be pinned host memory
   (pageable memory makes the copy synchronous). Two downloads can be in flight;
   a third waits on the device for the first. No counterpart in the reference,
   whose TransferFromCUDA is synchronous. */
sphmp_status sphmp_download_display_async(sphmp_ctx* ctx, sphmp_display_pack* disp, int32_t n);
/* Wait for every asynchronous download of the context. */
sphmp_status sphmp_download_wait(sphmp_ctx* ctx);
/* Append records into slots [start, end) and set num = end (EmitUpdateCUDA). */
sphmp_status sphmp_emit_aos(sphmp_ctx* ctx, const sphmp_display_pack* disp,
                            const sphmp_calc_pack* calc, int32_t start, int32_t end);
/* Upload / download one array (sphmp_field) for n slots (gridtotal cells for the
   MGRIDOFF/MGRIDCNT fields). Fields marked "download only" reject uploads. */
sphmp_status sphmp_upload_field(sphmp_ctx* ctx, int32_t field, const void* host, int32_t n);
sphmp_status sphmp_download_field(sphmp_ctx* ctx, int32_t field, void* host, int32_t n);

/* ---- per-pass entry points (one per reference launch wrapper) ---- */

/* GetParticleIndexCUDA (fluid_system_host.cu:147-159): cell id of every slot. */
sphmp_status sphmp_get_particle_index(sphmp_ctx* ctx);
/* GetGridListCUDA (fluid_system_host.cu:161-185): stable key sort, cell
   offsets/counts and rank-in-cell. */
sphmp_status sphmp_get_grid_list(sphmp_ctx* ctx);
/* Allocation-free cell sort; no counterpart in the reference (its GetGridListCUDA
   sorts the context's own arrays). For callers that must not let a library
   allocate device memory (a host application owning the device through its own
   pool, a frame loop that cannot take cudaMalloc's implicit synchronisation):
   sorts n cell ids `cell` (GRID_UNDEF for out-of-grid particles) on `stream` (a
   cudaStream_t, NULL for the default stream) into caller-owned device buffers:
   midsort[n] (stable order), mgndx[n] (rank in cell, GRID_UNDEF out of grid),
   gridoff[gridtotal] and gridcnt[gridtotal], with the values GetGridListCUDA
   gives. Its only scratch is a 4.2 MB static device array, so n is limited to
   SPHMP_NOALLOC_MAX_PARTICLES, gridtotal to SPHMP_NOALLOC_MAX_CELLS and one cell
   to 4096 particles (larger inputs return SPHMP_ERR_CAPACITY or
   SPHMP_ERR_CELL_OVERFLOW; a key that is neither a cell id below gridtotal nor
   GRID_UNDEF returns SPHMP_ERR_INVALID_ARG). The first call in a CUDA context
   (the device's primary context, or one the caller made current) looks the
   scratch up with cudaGetSymbolAddress and keeps the address with the context's
   id, so a call after cudaDeviceReset looks it up again. Every call copies an
   error word to the host and synchronises `stream` before it returns, so no
   call may be made while `stream` is being captured into a CUDA graph. Calls on
   one device share the scratch: calls that overlap in time race and must be
   serialised. */
#define SPHMP_NOALLOC_MAX_PARTICLES 262144
#define SPHMP_NOALLOC_MAX_CELLS 262144
sphmp_status sphmp_sort_cells_noalloc(const uint32_t* cell, int32_t n, int32_t gridtotal,
                                      uint32_t* midsort, uint32_t* mgndx, int32_t* gridoff,
                                      int32_t* gridcnt, void* stream);
/* RearrageDataCUDA (fluid_system_host.cu:187-210): move every particle to its
   sorted slot; out-of-grid slots are parked at (-1000,-1000,-1000). */
sphmp_status sphmp_rearrange_data(sphmp_ctx* ctx);
/* ComputeBoundaryDensity (fluid_system_host.cu:510-513): boundary particle volumes. */
sphmp_status sphmp_compute_boundary_density(sphmp_ctx* ctx);
/* MfComputePressureCUDA (fluid_system_host.cu:337-348): density + EOS pressure. */
sphmp_status sphmp_compute_pressure(sphmp_ctx* ctx);
/* MfComputeDriftVelCUDA (decl fluid_system_host.cuh:62; kernel multiphase.cu:78-166). */
sphmp_status sphmp_compute_drift_vel(sphmp_ctx* ctx);
/* MfComputeAlphaAdvanceCUDA (decl fluid_system_host.cuh:63; kernel multiphase.cu:218-272). */
sphmp_status sphmp_compute_alpha_advance(sphmp_ctx* ctx);
/* MfComputeCorrectionCUDA (decl fluid_system_host.cuh:64; kernel multiphase.cu:275-349). */
sphmp_status sphmp_compute_correction(sphmp_ctx* ctx);
/* MfComputeForceCUDA (fluid_system_host.cu:421-438), plus the reference
   SurfaceTension term (fluid_system_kern.cu:605-625) when enabled. */
sphmp_status sphmp_compute_force(sphmp_ctx* ctx);
/* ComputeForce_projectu (kernel SPH_Solver/fluids/multiphase.cu:488-616; its host
   wrapper ComputeForceCUDA_ProjectU, fluid_system_host.cu:396-419, has the launch
   commented out): pressure with p_i + p_j, viscosity on veleval, boundary terms
   scaled by mf_omega / mf_visc_factor, the drift-velocity tensor term of every
   phase, written to accel; the XSPH velocity correction to SPHMP_F_VELXCOR. Reads
   the start-of-step fractions and this step's drift velocities. Adds the
   SurfaceTension term when enabled. */
sphmp_status sphmp_compute_force_projectu(sphmp_ctx* ctx);
/* MfAdvanceCUDA (fluid_system_host.cu:385-394). */
sphmp_status sphmp_advance(sphmp_ctx* ctx);

/* ---- the IISPH step (implicit incompressible SPH, RunIISPH,
   fluid_system.cpp:567-588; kernels fluid_system_kern.cu:637-1115) ----
   The reference's kernels as written: the cubic spline of support 2h and its
   gradient, the advection acceleration from the boundary's artificial
   viscosity within 2h plus gravity, every other gradient sum over fluid
   neighbours within h, relaxed Jacobi with omega = 0.1 starting from half the
   stored pressure. After sphmp_iisph_density, SPHMP_F_DENS reads the density
   itself (the reference stores it there), not its inverse. Each needs the cell
   lists of the current sort. */
/* ComputeDensityIISPH_CUDA (fluid_system_host.cu:505-508). */
sphmp_status sphmp_iisph_density(sphmp_ctx* ctx);
/* PredictAdvection (fluid_system_host.cu:515-524): ComputeDii then ComputeAii. */
sphmp_status sphmp_iisph_predict_advection(sphmp_ctx* ctx);
/* One pass of PressureSolve's loop (fluid_system_host.cu:529-540): Pressure_DP,
   Pressure_Iter (accel and pressure of the iterate), press_l = press_l1. With
   `residue`: residue[0] = the reference's quantity (the residues summed over
   every slot, boundary particles 0, divided by the slot count), residue[1] = the
   mean |residue| over in-grid fluid particles (kg/m^3). Synchronises the
   context stream. */
sphmp_status sphmp_iisph_pressure_iteration(sphmp_ctx* ctx, double* residue);
/* PressureSolve with a stopping rule of this library's own (the reference's
   loop never ends): iterate until residue[1] <= tol after at least min_iter
   iterations, or max_iter iterations; `iters` and `residue` (2 doubles) receive
   the count and the last residues. */
sphmp_status sphmp_iisph_pressure_solve(sphmp_ctx* ctx, float tol, int32_t min_iter, int32_t max_iter,
                                        int32_t* iters, double* residue);
/* Integration (IntegrateIISPH, fluid_system_host.cu:552-556): vel = veleval +
   accel dt, pos += vel dt / simscale. */
sphmp_status sphmp_iisph_integrate(sphmp_ctx* ctx);
/* ---- launch-shape autotuner; no counterpart in the reference (which runs one
   scene at a fixed 384-thread launch geometry, fluid_system_host.cu:70-76) ---- */
typedef struct sphmp_tuning {
    int32_t cell_order;     /* chosen sphmp_cell_order */
    int32_t bucket_window;  /* chosen members per density work item */
    int32_t heavy_list;     /* chosen heavy-list threshold */
    int32_t trials;         /* configurations timed */
    float ms_per_step;      /* fused step of the chosen configuration */
    float ms_before;        /* fused step of the configuration the context had */
} sphmp_tuning;
/* Times the fused step of the context's current state in a scratch context of
   the same capacity for each candidate configuration (members per density work
   item 16 or 32, heavy-list threshold 64, 128 or 256, and with allow_reorder the
   Morton cell order beside the linear one): a device copy of the state, one
   captured-graph step to warm, then trial_steps graph steps timed with CUDA
   events on the scratch stream. The fastest configuration is written into the
   context's parameters (its graph is re-captured at the next step); the
   context's own state does not move. The window and threshold change no result
   beyond the summation order of the heavy particles; the Morton order changes the
   order of the sorted arrays (not bit-exact with the reference's sort), hence
   the opt-in. Allocates the scratch context for the duration of the call. */
sphmp_status sphmp_autotune(sphmp_ctx* ctx, int32_t trial_steps, int32_t allow_reorder, sphmp_tuning* out);

/* nsteps IISPH steps: the sort, density, PredictAdvection, the pressure solve
   (tol, at least 2 and at most max_iter iterations) and the integration the
   reference comments out; iters[k] (if given) = the iterations of step k,
   residue (2 doubles, if given) = the last step's final residues. */
sphmp_status sphmp_step_iisph(sphmp_ctx* ctx, int32_t nsteps, float tol, int32_t max_iter, int32_t* iters,
                              double* residue);

/* nsteps full steps (sort ... advance) in the given sphmp_schedule. Steps run
   from a captured CUDA graph when `use_graph` is 1 (one step per graph for the
   fused schedule, two for the others, whose steps flip the double buffers an
   odd number of times; an odd remainder runs eagerly). */
sphmp_status sphmp_step(sphmp_ctx* ctx, int32_t nsteps, int32_t schedule, int32_t use_graph);

/* Run one step eagerly with a CUDA event recorded on the context stream between
   consecutive stages (hash, cell_starts, cell_order, rearrange, density, then the
   neighbour passes of the schedule). Writes the milliseconds of each stage into
   ms[i] and its name into names + 32*i (NUL-terminated, may be NULL); returns the
   number of stages, or minus a sphmp_status on error. */
int32_t sphmp_step_profile(sphmp_ctx* ctx, int32_t schedule, float* ms, char* names, int32_t nmax);

/* FP64 conservation sums over in-grid, non-boundary slots, computed on the GPU:
   out[0] = total mass, out[1] = total volume sum(m/rho), out[2+k] = phase-k volume
   sum(alpha_k m/rho) for k < nphase, out[2+nphase] = max |sum_k alpha_k - 1|. */
sphmp_status sphmp_conservation(sphmp_ctx* ctx, double* out, int32_t nout);

/* Binary state checkpoint of a context (no counterpart in the reference): the
   reference records of every particle plus its volume fractions and last-step
   (g - a), everything a following step reads, so a context loaded from a
   checkpoint continues bit for bit like the one that wrote it. Little-endian
   hosts; sphmp_load_state replaces the context's particles (the phase count
   must match, n must fit the capacity). */
sphmp_status sphmp_save_state(sphmp_ctx* ctx, const char* path);
sphmp_status sphmp_load_state(sphmp_ctx* ctx, const char* path);

/* Device-side error word accumulated by the kernels since the last call (bit set of
   (1 << sphmp_status)); reading it clears it. */
sphmp_status sphmp_device_errors(sphmp_ctx* ctx, uint32_t* bits);

/* Text of the last error raised on the calling thread ("" if none). */
const char* sphmp_last_error(void);
/* Library build identification, e.g. "sphmp 0.1 sm_103a". */
const char* sphmp_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SPHMP_H */
