/* fluid_system_kern.cuh stand-in for the oracle host build of the reference's
 * SPH_Solver/fluids/multiphase.cu (oracle/ref).
 *
 * multiphase.cu was written against the older Fluids-v3 multi-fluid buffer
 * layout (`simData`, `buf.mpos`, `buf.mf_alpha`, `buf.mgrid`, ...), which the
 * current fluid_system_kern.cuh no longer declares. This header declares that
 * older layout under distinct type names (so it can coexist with the current
 * layout in the same library) plus the vector helpers the legacy code expects
 * (make_cfloat3, scalar * vector). */
#pragma once
#include "../common_header.h"

#ifndef MAX_FLUIDNUM
#define MAX_FLUIDNUM 3
#endif
#define GRID_UNDEF 4294967295
#define EPSILON 0.00001f

#define bufList legacy_bufList
#define FluidParams legacy_FluidParams

struct legacy_FluidParams {
    /* fields read by the multiphase kernels */
    float psimscale, r2, psmoothradius, spikykern, poly6kern;
    int mf_catnum;
    float mf_dens[MAX_FLUIDNUM], mf_visc[MAX_FLUIDNUM];
    float relax, mf_diffusion, cont, cont1, cont2;
    cint3 gridRes;
    int gridAdjCnt;
    int gridAdj[64];
    float mf_dt, tohydro, pintstiff, visc_factor, omega;
    /* fields read only by the granular / project-U code in the same file */
    float Yradius, boundaryVisc, coA, coB, coD, coD0, coG, coLambdaK, coN, cohesion;
    float fsa, fsb, initspacing, pan_r, phi, solid_Yradius, solid_coG;
};

struct legacy_bufList {
    cfloat3* mpos;
    cfloat3* mveleval;
    float* mpress;
    float* mdensity;
    float* mf_restmass;
    float* mf_restdensity;
    float* mf_visc;
    float* mf_alpha;
    float* mf_alpha_pre;
    cfloat3* mf_vel_phrel;
    cfloat3* mforce;
    int* misbound;
    int* MFtype;
    uint* mgrid;
    uint* mgcell;
    int* mgridcnt;
    int* mgridoff;
    float* mf_pressure_modify;
    uint* mclr;
    /* project-U output (XSPH correction) */
    cfloat3* mf_velxcor;
    /* granular arrays (never touched by the oracle) */
    cfloat3* mf_alphagrad;
    float* last_mpress;
    float* MFpepsilon;
    float* MFtensor;
    float* MFtemptensor;
    float* MFRtensor;
    float* MFvelgrad;
};

inline cfloat3 make_cfloat3(float x, float y, float z) { return cfloat3(x, y, z); }
inline cfloat3 operator*(float s, const cfloat3& v) { return cfloat3(s * v.x, s * v.y, s * v.z); }
inline cfloat3 operator-(const cfloat3& v) { return cfloat3(-v.x, -v.y, -v.z); }

/* referenced only by the out-of-scope tensor code (multiphase.cu:855,992); the
   toolkit header it expects does not declare it */
void svdecomp3(float* w, float* u, float* v, float eps);
