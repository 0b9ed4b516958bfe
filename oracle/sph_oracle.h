/*
 * sph_oracle.h — CPU oracle for the multiphase SPH step. TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference kernels of ZP-Z/sph-multiphase
 * (SPH_Solver/fluids/fluid_system_kern.cu, SPH_Solver/fluids/multiphase.cu and
 * the launch wrappers in SPH_Solver/fluids/fluid_system_host.cu), one function per
 * reference launch wrapper, iterating the 27 neighbour cells and the particles
 * inside each cell in the reference order and reproducing the reference's
 * float/double promotions operation by operation.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * this code, and only as the checker / the timed CPU baseline. The product path
 * (the CUDA library) never calls it.
 *
 * The file sph_oracle.c is compiled twice: with ORC_F64 undefined it is the
 * FP32 oracle with the reference's mixed float/double arithmetic (functions
 * suffixed _f32); with ORC_F64 defined every quantity is double (suffix _f64),
 * which is the FP64 oracle the FP32 results are measured against.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>
#include "../include/sphmp.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_STATE_FIELDS(R)                                                       \
    int32_t n;          /* particle slots (reference fcuda.pnum) */               \
    R* pos;             /* [3n] displayPack.pos */                                \
    int32_t* type;      /* [n]  displayPack.type */                               \
    float* color;       /* [4n] displayPack.color (only moved by the sort) */     \
    R* vel;             /* [3n] */                                                \
    R* veleval;         /* [3n] */                                                \
    R* pressure;        /* [n] */                                                 \
    R* dens;            /* [n]  1/rho (fluid) or boundary volume */               \
    R* restdens;        /* [n] */                                                 \
    R* mass;            /* [n] */                                                 \
    R* visc;            /* [n] */                                                 \
    int32_t* bornid;    /* [n] */                                                 \
    R* accel;           /* [3n] */                                                \
    R* alpha;           /* [3n] mf_alpha */                                       \
    R* alpha_pre;       /* [3n] mf_alpha_pre */                                   \
    R* drift;           /* [9n] mf_vel_phrel */                                   \
    R* aprev;           /* [3n] mforce */                                         \
    R* pmod;            /* [n]  mf_pressure_modify */                             \
    uint32_t* mgcell;   /* [n] */                                                 \
    uint32_t* midsort;  /* [n] */                                                 \
    uint32_t* mgndx;    /* [n] */                                                 \
    int32_t* mgridoff;  /* [gridtotal] */                                         \
    int32_t* mgridcnt;  /* [gridtotal] */                                         \
    R* velxcor;         /* [3n] mf_velxcor (project-U force) */                   \
    R* dii;             /* [3n] IISPH d_ii */                                     \
    R* aii;             /* [n]  IISPH a_ii */                                     \
    R* rho_adv;         /* [n]  IISPH predicted density */                        \
    R* press_l;         /* [n]  IISPH pressure iterate */                         \
    R* press_l1;        /* [n]  IISPH next iterate */                             \
    R* dijpj;           /* [3n] IISPH sum_j d_ij p_j */                           \
    R* residue;         /* [n]  IISPH density residue */

typedef struct orc_state_f32 { ORC_STATE_FIELDS(float) } orc_state_f32;
typedef struct orc_state_f64 { ORC_STATE_FIELDS(double) } orc_state_f64;

#define ORC_DECLARE(SFX, ST)                                                         \
    void orc_get_particle_index##SFX(const sphmp_params* p, ST* s);                  \
    void orc_get_grid_list##SFX(const sphmp_params* p, ST* s);                       \
    int orc_rearrange_data##SFX(const sphmp_params* p, ST* s);                       \
    void orc_compute_boundary_volume##SFX(const sphmp_params* p, ST* s);             \
    void orc_compute_pressure##SFX(const sphmp_params* p, ST* s);                    \
    void orc_compute_force##SFX(const sphmp_params* p, ST* s);                       \
    void orc_surface_tension##SFX(const sphmp_params* p, ST* s);                     \
    void orc_advance##SFX(const sphmp_params* p, ST* s);                             \
    void orc_compute_drift_vel##SFX(const sphmp_params* p, ST* s);                   \
    void orc_compute_alpha_advance##SFX(const sphmp_params* p, ST* s);               \
    void orc_compute_correction##SFX(const sphmp_params* p, ST* s);                  \
    void orc_compute_force_projectu##SFX(const sphmp_params* p, ST* s);              \
    int orc_step##SFX(const sphmp_params* p, ST* s, int schedule, int nsteps);       \
    int orc_before_first_step##SFX(const sphmp_params* p, ST* s);                 \
    void orc_iisph_density##SFX(const sphmp_params* p, ST* s);                     \
    void orc_iisph_predict##SFX(const sphmp_params* p, ST* s);                     \
    double orc_iisph_iteration##SFX(const sphmp_params* p, ST* s);                 \
    void orc_iisph_integrate##SFX(const sphmp_params* p, ST* s);

ORC_DECLARE(_f32, orc_state_f32)
ORC_DECLARE(_f64, orc_state_f64)

/* Kernel constants and grid exactly as the reference host derives them
   (fluid_system.cpp:308-313 and :119-145). Returns 0 on success. */
int orc_setup_constants(sphmp_params* p);
int orc_setup_grid(sphmp_params* p);

/* Scene generation restated from the reference's AddFluidVolume, SetupAddWall and
   SetupAddOpenBox (fluid_system.cpp:719-762, AddShape.cpp:265-366) with the
   library's seeded jitter stream, and the library's parameter defaults: a CPU
   run builds the same records as the CUDA library's generators without loading
   it. The generators return 0, or -1 when `cap` records are not enough. */
void orc_params_default(sphmp_params* p);
int orc_add_fluid_volume(const sphmp_params* p, const float vmin[3], const float vmax[3], float spacing,
                         const float offs[3], int32_t phase, float jitter, uint64_t seed,
                         sphmp_display_pack* disp, sphmp_calc_pack* calc, int32_t cap, int32_t* count);
int orc_add_wall(const sphmp_params* p, const float vmin[3], const float vmax[3], sphmp_display_pack* disp,
                 sphmp_calc_pack* calc, int32_t cap, int32_t* count);
int orc_add_open_box(const sphmp_params* p, const float mn[3], const float mx[3], float t, sphmp_display_pack* disp,
                     sphmp_calc_pack* calc, int32_t cap, int32_t* count);

void orc_set_num_threads(int n);
int orc_get_num_threads(void);

#ifdef __cplusplus
}
#endif

#endif
