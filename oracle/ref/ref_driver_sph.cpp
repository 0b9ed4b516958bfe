/* ref_driver_sph.cpp — runs the reference's own SPH kernels (SPH_Solver/fluids/
 * fluid_system_kern.cu, compiled unmodified as host C++) on the CPU, as the pin for
 * the oracle restatement. TEST INFRASTRUCTURE ONLY; built into oracle/_ref/ by
 * oracle/ref/build_ref.sh and never shipped.
 *
 * Each ref_* entry point restates one launch wrapper of SPH_Solver/fluids/
 * fluid_system_host.cu: it loads an orc_state_f32 into the reference's AoS buffers
 * (`bufList fbuf`), runs the kernel body once per particle (blockIdx.x = i,
 * blockDim.x = 1, threadIdx.x = 0) on OpenMP threads, and stores the buffers back.
 * thrust::sort_by_key (fluid_system_host.cu:164-166) is std::stable_sort on the
 * same (key, value) pairs, which yields the same permutation. */
#include "fluid_system_host.cuh"
#include "fluid_system_kern.cuh"

#include <algorithm>
#include <numeric>
#include <stdlib.h>
#include <vector>
#include <omp.h>

#include "sph_oracle.h"

thread_local orc_dim3 blockIdx, threadIdx, blockDim, gridDim;

extern ParamCarrier paramCarrier;

static_assert(sizeof(ParamCarrier) == 464, "ParamCarrier layout");
static_assert(sizeof(displayPack) == 32, "displayPack layout");
static_assert(sizeof(calculationPack) == 224, "calculationPack layout");
static_assert(sizeof(displayPack) == sizeof(sphmp_display_pack), "display pack mirror");
static_assert(sizeof(calculationPack) == sizeof(sphmp_calc_pack), "calc pack mirror");

static bufList fbuf;
static int cap_n = 0, cap_g = 0;

static void ensure(int n, int g) {
    if (n > cap_n) {
        free(fbuf.displayBuffer); free(fbuf.calcBuffer); free(fbuf.msortbuf);
        free(fbuf.mgcell); free(fbuf.mgndx); free(fbuf.midsort); free(fbuf.MFidTable);
        free(fbuf.dii); free(fbuf.aii); free(fbuf.rho_adv); free(fbuf.press_l); free(fbuf.press_l1);
        free(fbuf.dijpj); free(fbuf.densityResidue);
        fbuf.displayBuffer = (displayPack*)calloc(n, sizeof(displayPack));
        fbuf.calcBuffer = (calculationPack*)calloc(n, sizeof(calculationPack));
        fbuf.msortbuf = (char*)calloc(n, sizeof(displayPack) + sizeof(calculationPack));
        fbuf.mgcell = (uint*)calloc(n, sizeof(uint));
        fbuf.mgndx = (uint*)calloc(n, sizeof(uint));
        fbuf.midsort = (uint*)calloc(n, sizeof(uint));
        fbuf.MFidTable = (int*)calloc(n, sizeof(int));
        fbuf.dii = (cfloat3*)calloc(n, sizeof(cfloat3));
        fbuf.aii = (float*)calloc(n, sizeof(float));
        fbuf.rho_adv = (float*)calloc(n, sizeof(float));
        fbuf.press_l = (float*)calloc(n, sizeof(float));
        fbuf.press_l1 = (float*)calloc(n, sizeof(float));
        fbuf.dijpj = (cfloat3*)calloc(n, sizeof(cfloat3));
        fbuf.densityResidue = (float*)calloc(n, sizeof(float));
        cap_n = n;
    }
    if (g > cap_g) {
        free(fbuf.mgridcnt); free(fbuf.mgridoff);
        fbuf.mgridcnt = (int*)calloc(g, sizeof(int));
        fbuf.mgridoff = (int*)calloc(g, sizeof(int));
        cap_g = g;
    }
}

static void load(const sphmp_params* p, const orc_state_f32* s) {
    ensure(s->n > 0 ? s->n : 1, p->gridtotal);
    memcpy(&paramCarrier, p, sizeof(ParamCarrier)); /* CarryParam */
    for (int i = 0; i < s->n; i++) {
        displayPack& d = fbuf.displayBuffer[i];
        calculationPack& c = fbuf.calcBuffer[i];
        memset(&c, 0, sizeof(c));
        d.pos.Set(s->pos[3 * i], s->pos[3 * i + 1], s->pos[3 * i + 2]);
        d.color.Set(s->color[4 * i], s->color[4 * i + 1], s->color[4 * i + 2], s->color[4 * i + 3]);
        d.type = s->type[i];
        c.vel.Set(s->vel[3 * i], s->vel[3 * i + 1], s->vel[3 * i + 2]);
        c.veleval.Set(s->veleval[3 * i], s->veleval[3 * i + 1], s->veleval[3 * i + 2]);
        c.pressure = s->pressure[i];
        c.dens = s->dens[i];
        c.restdens = s->restdens[i];
        c.mass = s->mass[i];
        c.visc = s->visc[i];
        c.bornid = s->bornid[i];
        c.accel.Set(s->accel[3 * i], s->accel[3 * i + 1], s->accel[3 * i + 2]);
        fbuf.dii[i].Set(s->dii[3 * i], s->dii[3 * i + 1], s->dii[3 * i + 2]);
        fbuf.dijpj[i].Set(s->dijpj[3 * i], s->dijpj[3 * i + 1], s->dijpj[3 * i + 2]);
        fbuf.aii[i] = s->aii[i];
        fbuf.rho_adv[i] = s->rho_adv[i];
        fbuf.press_l[i] = s->press_l[i];
        fbuf.press_l1[i] = s->press_l1[i];
        fbuf.densityResidue[i] = s->residue[i];
    }
    memcpy(fbuf.mgcell, s->mgcell, sizeof(uint) * s->n);
    memcpy(fbuf.midsort, s->midsort, sizeof(uint) * s->n);
    memcpy(fbuf.mgndx, s->mgndx, sizeof(uint) * s->n);
    memcpy(fbuf.mgridcnt, s->mgridcnt, sizeof(int) * p->gridtotal);
    memcpy(fbuf.mgridoff, s->mgridoff, sizeof(int) * p->gridtotal);
}

static void store(const sphmp_params* p, orc_state_f32* s) {
    for (int i = 0; i < s->n; i++) {
        const displayPack& d = fbuf.displayBuffer[i];
        const calculationPack& c = fbuf.calcBuffer[i];
        s->pos[3 * i] = d.pos.x; s->pos[3 * i + 1] = d.pos.y; s->pos[3 * i + 2] = d.pos.z;
        s->color[4 * i] = d.color.x; s->color[4 * i + 1] = d.color.y;
        s->color[4 * i + 2] = d.color.z; s->color[4 * i + 3] = d.color.w;
        s->type[i] = d.type;
        s->vel[3 * i] = c.vel.x; s->vel[3 * i + 1] = c.vel.y; s->vel[3 * i + 2] = c.vel.z;
        s->veleval[3 * i] = c.veleval.x; s->veleval[3 * i + 1] = c.veleval.y; s->veleval[3 * i + 2] = c.veleval.z;
        s->pressure[i] = c.pressure;
        s->dens[i] = c.dens;
        s->restdens[i] = c.restdens;
        s->mass[i] = c.mass;
        s->visc[i] = c.visc;
        s->bornid[i] = c.bornid;
        s->accel[3 * i] = c.accel.x; s->accel[3 * i + 1] = c.accel.y; s->accel[3 * i + 2] = c.accel.z;
        s->dii[3 * i] = fbuf.dii[i].x; s->dii[3 * i + 1] = fbuf.dii[i].y; s->dii[3 * i + 2] = fbuf.dii[i].z;
        s->dijpj[3 * i] = fbuf.dijpj[i].x; s->dijpj[3 * i + 1] = fbuf.dijpj[i].y;
        s->dijpj[3 * i + 2] = fbuf.dijpj[i].z;
        s->aii[i] = fbuf.aii[i];
        s->rho_adv[i] = fbuf.rho_adv[i];
        s->press_l[i] = fbuf.press_l[i];
        s->press_l1[i] = fbuf.press_l1[i];
        s->residue[i] = fbuf.densityResidue[i];
    }
    memcpy(s->mgcell, fbuf.mgcell, sizeof(uint) * s->n);
    memcpy(s->midsort, fbuf.midsort, sizeof(uint) * s->n);
    memcpy(s->mgndx, fbuf.mgndx, sizeof(uint) * s->n);
    memcpy(s->mgridcnt, fbuf.mgridcnt, sizeof(int) * p->gridtotal);
    memcpy(s->mgridoff, fbuf.mgridoff, sizeof(int) * p->gridtotal);
}

template <class K>
static void launch(K kernel, int n) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; i++) {
        blockIdx.x = (unsigned)i;
        blockDim.x = 1;
        threadIdx.x = 0;
        kernel(fbuf, n);
    }
}

extern "C" {

/* GetParticleIndexCUDA, fluid_system_host.cu:147-159 */
void ref_get_particle_index(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    memset(fbuf.mgridcnt, 0, p->gridtotal * sizeof(int));
    memset(fbuf.mgridoff, 0, p->gridtotal * sizeof(int));
    memset(fbuf.mgcell, 0, s->n * sizeof(uint));
    launch(InitialSort, s->n);
    store(p, s);
}

/* GetGridListCUDA, fluid_system_host.cu:161-185 */
void ref_get_grid_list(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    const int n = s->n;
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [](int a, int b) { return fbuf.mgcell[a] < fbuf.mgcell[b]; });
    std::vector<uint> k(n), v(n);
    for (int i = 0; i < n; i++) { k[i] = fbuf.mgcell[order[i]]; v[i] = fbuf.midsort[order[i]]; }
    memcpy(fbuf.mgcell, k.data(), n * sizeof(uint));
    memcpy(fbuf.midsort, v.data(), n * sizeof(uint));
    launch(CalcFirstCnt, n);
    launch(GetCnt, n);
    store(p, s);
}

/* RearrageDataCUDA, fluid_system_host.cu:187-210 */
void ref_rearrange_data(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    const int n = s->n;
    memcpy(fbuf.msortbuf + n * BUF_DISPLAYBUF, fbuf.displayBuffer, n * sizeof(displayPack));
    memcpy(fbuf.msortbuf + n * BUF_CALCBUF, fbuf.calcBuffer, n * sizeof(calculationPack));
    launch(RearrangeData, n);
    store(p, s);
}

/* ComputeBoundaryDensity, fluid_system_host.cu:510-513 */
void ref_compute_boundary_volume(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    launch(ComputeBoundaryVolume, s->n);
    store(p, s);
}

/* MfComputePressureCUDA, fluid_system_host.cu:337-348 */
void ref_compute_pressure(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    launch(ComputeDensityPressure, s->n);
    store(p, s);
}

/* MfComputeForceCUDA, fluid_system_host.cu:421-438 */
void ref_compute_force(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    launch(ComputeForce, s->n);
    store(p, s);
}

/* SurfaceTension launch (commented in the reference at fluid_system_host.cu:433-437) */
void ref_surface_tension(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    launch(SurfaceTension, s->n);
    store(p, s);
}

/* MfAdvanceCUDA, fluid_system_host.cu:385-394 */
void ref_advance(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    launch(AdvanceParticles, s->n);
    store(p, s);
}

/* ComputeDensityIISPH_CUDA, fluid_system_host.cu:505-508 */
void ref_iisph_density(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    launch(ComputeDensityIISPH, s->n);
    store(p, s);
}

/* PredictAdvection, fluid_system_host.cu:515-524 */
void ref_iisph_predict(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    launch(ComputeDii, s->n);
    launch(ComputeAii, s->n);
    store(p, s);
}

/* One pass of PressureSolve's loop, fluid_system_host.cu:529-540: Pressure_DP,
   Pressure_Iter, press_l = press_l1, and the mean of densityResidue (thrust::reduce
   over pnum, divided by pnum). */
double ref_iisph_iteration(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    launch(Pressure_DP, s->n);
    launch(Pressure_Iter, s->n);
    memcpy(fbuf.press_l, fbuf.press_l1, sizeof(float) * s->n);
    double sum = 0;
    for (int i = 0; i < s->n; i++) sum += fbuf.densityResidue[i];
    store(p, s);
    return s->n > 0 ? sum / s->n : 0.0;
}

/* Integration (IntegrateIISPH), fluid_system_host.cu:553-556 */
void ref_iisph_integrate(const sphmp_params* p, orc_state_f32* s) {
    load(p, s);
    launch(IntegrateIISPH, s->n);
    store(p, s);
}

void ref_set_num_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}

} /* extern "C" */
