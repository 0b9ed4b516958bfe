/* ref_driver_mp.cpp — runs the reference's drift-flux kernels (SPH_Solver/fluids/
 * multiphase.cu:18-349) and its project-U force (:488-616), compiled unmodified as host C++ against the legacy layout in
 * shim_legacy/) on the CPU, as the pin for the oracle restatement. TEST
 * INFRASTRUCTURE ONLY; built into oracle/_ref/ by oracle/ref/build_ref.sh.
 *
 * The legacy buffers are pointed straight at the arrays of an orc_state_f32
 * (float[3n] is laid out exactly like cfloat3[n]). `mgrid` is the identity after
 * the sort; `misbound` is type == TYPE_BOUNDARY and `MFtype` is the particle type.
 * gridAdj[] enumerates the 3x3x3 block from its low corner in y, z, x order,
 * which is how the legacy kernels address it (gc - nadj + gridAdj[c]). */
#include "fluid_system_host.cuh"
#include "fluid_system_kern.cuh"

#include <float.h>
#include <stdlib.h>
#include <vector>

#include "sph_oracle.h"

legacy_FluidParams simData;

__global__ void mfComputeDriftVel(bufList buf, int pnum);
__global__ void mfComputeAlphaAdvance(bufList buf, int pnum);
__global__ void mfComputeCorrection(bufList buf, int pnum);
__global__ void ComputeForce_projectu(bufList buf, int pnum);

void svdecomp3(float*, float*, float*, float) { abort(); }

static void set_sim(const sphmp_params* p) {
    memset(&simData, 0, sizeof(simData));
    simData.psimscale = p->simscale;
    simData.r2 = p->smoothradius * p->smoothradius;
    simData.psmoothradius = p->smoothradius;
    simData.spikykern = p->kspikydiff;
    simData.poly6kern = p->kpoly6;
    simData.mf_catnum = p->nphase;
    for (int k = 0; k < MAX_FLUIDNUM; k++) {
        simData.mf_dens[k] = p->densArr[k];
        simData.mf_visc[k] = p->viscArr[k];
    }
    simData.relax = p->mf_relax;
    simData.mf_diffusion = p->mf_diffusion;
    simData.cont = p->mf_cont;
    simData.cont1 = p->mf_cont1;
    simData.cont2 = p->mf_cont2;
    simData.gridRes = cint3(p->gridres[0], p->gridres[1], p->gridres[2]);
    simData.gridAdjCnt = 27;
    int cnt = 0;
    for (int y = 0; y < 3; y++)
        for (int z = 0; z < 3; z++)
            for (int x = 0; x < 3; x++)
                simData.gridAdj[cnt++] = (y * p->gridres[2] + z) * p->gridres[0] + x;
    simData.mf_dt = p->dt;
    simData.tohydro = FLT_MAX; /* the granular "becomes water" flip never fires */
    simData.pintstiff = p->mf_pintstiff;
    simData.omega = p->mf_omega;
    simData.visc_factor = p->mf_visc_factor;
}

/* `force_out`: mforce is the force output (the project-U force) rather than the
   previous step's g - a that the drift velocity reads. */
template <class K>
static void run(K kernel, const sphmp_params* p, orc_state_f32* s, bool force_out = false) {
    set_sim(p);
    const int n = s->n;
    std::vector<int> isbound(n), mftype(n);
    std::vector<uint> mgrid(n), mclr(n);
    for (int i = 0; i < n; i++) {
        isbound[i] = s->type[i] == 1 ? 1 : 0;
        mftype[i] = s->type[i];
        mgrid[i] = (uint)i;
    }
    legacy_bufList b;
    memset(&b, 0, sizeof(b));
    b.mpos = (cfloat3*)s->pos;
    b.mveleval = (cfloat3*)s->veleval;
    b.mpress = s->pressure;
    b.mdensity = s->dens;
    b.mf_restmass = s->mass;
    b.mf_restdensity = s->restdens;
    b.mf_visc = s->visc;
    b.mf_alpha = s->alpha;
    b.mf_alpha_pre = s->alpha_pre;
    b.mf_vel_phrel = (cfloat3*)s->drift;
    b.mforce = (cfloat3*)(force_out ? s->accel : s->aprev);
    b.mf_velxcor = (cfloat3*)s->velxcor;
    b.misbound = isbound.data();
    b.MFtype = mftype.data();
    b.mgrid = mgrid.data();
    b.mgcell = s->mgcell;
    b.mgridcnt = s->mgridcnt;
    b.mgridoff = s->mgridoff;
    b.mf_pressure_modify = s->pmod;
    b.mclr = mclr.data();
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; i++) {
        blockIdx.x = (unsigned)i;
        blockDim.x = 1;
        threadIdx.x = 0;
        kernel(b, n);
    }
}

extern "C" {

/* MfComputeDriftVelCUDA (its body is commented out at fluid_system_host.cu:353-362) */
void ref_compute_drift_vel(const sphmp_params* p, orc_state_f32* s) { run(mfComputeDriftVel, p, s); }
/* MfComputeAlphaAdvanceCUDA (fluid_system_host.cu:364-373) */
void ref_compute_alpha_advance(const sphmp_params* p, orc_state_f32* s) { run(mfComputeAlphaAdvance, p, s); }
/* MfComputeCorrectionCUDA (fluid_system_host.cu:374-383) */
void ref_compute_correction(const sphmp_params* p, orc_state_f32* s) { run(mfComputeCorrection, p, s); }
/* ComputeForceCUDA_ProjectU (its launch is commented out at fluid_system_host.cu:399) */
void ref_compute_force_projectu(const sphmp_params* p, orc_state_f32* s) {
    run(ComputeForce_projectu, p, s, true);
}

} /* extern "C" */
