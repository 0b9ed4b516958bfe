/*
 * sph_oracle.c — CPU oracle for the multiphase SPH step. TEST INFRASTRUCTURE ONLY.
 *
 * Restates, function by function, the reference kernels of ZP-Z/sph-multiphase.
 * Every function names the reference lines it follows. Arithmetic is written
 * so that the FP32 build performs the same IEEE operations, in the same order,
 * as the reference compiled as host C++ without FMA contraction: float
 * operands stay float, double literals (2.5, 0.5, 0.01, 1.0, 0.0001, -0.99)
 * promote the expression to double exactly where C++ does, and C++ overload
 * resolution of pow/sqrt on float arguments (powf/sqrtf) is spelled out.
 * Compile with -ffp-contract=off.
 *
 * With ORC_F64 defined the same code runs entirely in double (the FP64 oracle);
 * the hash still quantises positions in float so both builds bin identical
 * inputs into identical cells.
 *
 * Loaded only by tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "sph_oracle.h"

#ifndef ORC_F64
typedef float R;
typedef orc_state_f32 ST;
#define FN(name) name##_f32
#define RSQRT(x) sqrtf(x)
#define RPOW(a, b) powf((a), (b))
#else
typedef double R;
typedef orc_state_f64 ST;
#define FN(name) name##_f64
#define RSQRT(x) sqrt(x)
#define RPOW(a, b) pow((a), (b))
#endif

#define UNDEF SPHMP_GRID_UNDEF

#ifndef ORC_F64
/* ---- helpers shared by both builds (defined once, in the FP32 object) ---- */

/* Reference SetupSimpleSphCase kernel constants, SPH_Solver/fluids/fluid_system.cpp:308-313.
   pow(float, float) resolves to the float overload (powf) in the reference's C++;
   the float*double products then run in double and narrow to float. */
int orc_setup_constants(sphmp_params* p) {
    float h = p->smoothradius;
    if (!(h > 0.0f)) return -1;
    p->cellsize = h * 2;
    p->kpoly6 = (float)(315.0f / ((double)64.0f * 3.141592 * (double)powf(h, 9.0f)));
    p->kspiky = (float)(15 / (3.141592 * (double)powf(h, 6.0f)));
    p->kspikydiff = (float)(-45.0f / (3.141592 * (double)powf(h, 6.0f)));
    p->klaplacian = (float)(45.0f / (3.141592 * (double)powf(h, 6.0f)));
    p->kspline = 1.0f / 3.141593f / powf(h, 3.0f);
    return 0;
}

/* Reference FluidSystem::SetupGrid, SPH_Solver/fluids/fluid_system.cpp:119-145. */
int orc_setup_grid(sphmp_params* p) {
    float worldcellsize = p->cellsize / p->simscale;
    for (int a = 0; a < 3; a++) {
        p->gridmin[a] = p->volmin[a];
        p->gridmax[a] = p->volmax[a];
        p->gridsize[a] = p->gridmax[a] - p->gridmin[a];
        p->gridres[a] = (int32_t)ceilf(p->gridsize[a] / worldcellsize);
        p->gridsize[a] = p->gridres[a] * worldcellsize;
        p->gridIdfac[a] = (float)(1.0 / (double)p->gridsize[a] * (double)p->gridres[a]);
    }
    p->gridtotal = p->gridres[0] * p->gridres[1] * p->gridres[2];
    p->searchnum = 3;
    p->neighbornum = 27;
    /* neighborid[i*9+j*3+k] = (i-1)*rx*rz + (j-1)*rx + (k-1): i walks y, j walks z, k walks x */
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                p->neighborid[i * 9 + j * 3 + k] =
                    (i - 1) * p->gridres[0] * p->gridres[2] + (j - 1) * p->gridres[0] + (k - 1);
    return 0;
}

/* ---- scene generation, so that a CPU-only run builds its inputs without the
   CUDA library (the benchmark's reference arm); tests check the records equal
   the library's generators byte for byte ---- */

/* Parameter defaults: the reference's ParamCarrier values where it has them,
   and the drift-flux constants the library chose where the reference reads
   them from a scene file that no longer exists (relax 1e-5, diffusion 1e-3,
   cont = cont1 = cont2 = 1, pintstiff 0.03, project-U factors 1). */
void orc_params_default(sphmp_params* p) {
    memset(p, 0, sizeof(*p));
    p->gravity[1] = -9.8f;
    p->simscale = 1.0f;
    p->dt = 1e-4f;
    p->smoothradius = 0.01f;
    p->viscosity = 0.2f;
    p->restdensity = 1000.0f;
    p->mass = 1.25e-4f;
    for (int k = 0; k < SPHMP_MAX_PHASES; k++) {
        p->massArr[k] = p->mass;
        p->densArr[k] = p->restdensity;
        p->viscArr[k] = p->viscosity;
    }
    p->bmass = 1.25e-4f;
    p->bRestdensity = 1000.0f;
    p->bvisc = 100.0f;
    p->nphase = 1;
    p->eos = SPHMP_EOS_TAIT;
    p->eos_stiffness = 3.0f;
    p->mf_relax = 1.0e-5f;
    p->mf_diffusion = 1.0e-3f;
    p->mf_cont = 1.0f;
    p->mf_cont1 = 1.0f;
    p->mf_cont2 = 1.0f;
    p->mf_pintstiff = 0.03f;
    p->mf_omega = 1.0f;
    p->mf_visc_factor = 1.0f;
}

/* The seeded lattice jitter: splitmix64 (Steele, Lea and Flood, "Fast splittable
   pseudorandom number generators", OOPSLA 2014) over the counter, stream seed
   * 0x100000001B3 + i, top 24 bits as a float in [0, 1). */
static uint64_t orc_splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

static float orc_uniform01(uint64_t seed, uint64_t i) {
    return (float)(orc_splitmix64(seed * 0x100000001B3ull + i) >> 40) * (1.0f / 16777216.0f);
}

/* AddParticle (SPH_Solver/fluids/fluid_system.cpp:702-717): a fresh record. */
static void orc_init_record(sphmp_display_pack* d, sphmp_calc_pack* c, int32_t n) {
    memset(d, 0, sizeof(*d));
    memset(c, 0, sizeof(*c));
    c->bornid = n;
    c->deformGrad[0] = c->deformGrad[4] = c->deformGrad[8] = 1.0f;
}

/* FluidSystem::AddFluidVolume (SPH_Solver/fluids/fluid_system.cpp:719-762): the
   lattice walked y, z, x (loop bounds compared against the float counts), each
   component jittered by U(-jitter/2, jitter/2) from the seeded stream in place of
   rand(). Returns 0, or -1 when `cap` records are not enough. */
int orc_add_fluid_volume(const sphmp_params* p, const float vmin[3], const float vmax[3], float spacing,
                         const float offs[3], int32_t phase, float jitter, uint64_t seed,
                         sphmp_display_pack* disp, sphmp_calc_pack* calc, int32_t cap, int32_t* count) {
    const float cnts[3] = {(vmax[0] - vmin[0]) / spacing, (vmax[1] - vmin[1]) / spacing,
                           (vmax[2] - vmin[2]) / spacing};
    uint64_t ctr = 0;
    for (int y = 0; y < cnts[1]; y++)
        for (int z = 0; z < cnts[2]; z++)
            for (int x = 0; x < cnts[0]; x++) {
                const int32_t n = *count;
                if (n >= cap) return -1;
                float r3[3];
                for (int a = 0; a < 3; a++) r3[a] = orc_uniform01(seed, ctr++) * jitter - jitter * 0.5f;
                sphmp_display_pack* d = disp + n;
                sphmp_calc_pack* c = calc + n;
                orc_init_record(d, c, n);
                const float xyz[3] = {(float)x, (float)y, (float)z};
                for (int a = 0; a < 3; a++) d->pos[a] = xyz[a] * spacing + vmin[a] + r3[a] + offs[a];
                d->color[0] = 0.2f; d->color[1] = 0.5f; d->color[2] = 0.8f; d->color[3] = 0.5f;
                d->type = SPHMP_TYPE_FLUID;
                c->restdens = p->densArr[phase];
                c->mass = p->massArr[phase];
                c->visc = p->viscArr[phase];
                *count = n + 1;
            }
    return 0;
}

/* SetupAddWall (SPH_Solver/fluids/AddShape.cpp:306-353) at the boundary spacing
   of CalcBoundarySpacing (:265-271): layers at y = min.y, min.y + s, ... (float
   accumulation, inclusive of max.y), each an x-z lattice of ceil(dx/s) * ceil(dz/s). */
int orc_add_wall(const sphmp_params* p, const float vmin[3], const float vmax[3], sphmp_display_pack* disp,
                 sphmp_calc_pack* calc, int32_t cap, int32_t* count) {
    const float spacing = powf((p->bmass / p->bRestdensity), 1 / 3.0f) / p->simscale;
    const int cntx = (int)ceilf((vmax[0] - vmin[0]) / spacing);
    const int cntz = (int)ceilf((vmax[2] - vmin[2]) / spacing);
    const int cnt = cntx * cntz;
    for (float y = vmin[1]; y <= vmax[1]; y += spacing)
        for (int xz = 0; xz < cnt; xz++) {
            const int32_t n = *count;
            if (n >= cap) return -1;
            sphmp_display_pack* d = disp + n;
            sphmp_calc_pack* c = calc + n;
            orc_init_record(d, c, n);
            d->pos[0] = vmin[0] + (xz % cntx) * spacing;
            d->pos[1] = y;
            d->pos[2] = vmin[2] + (xz / cntx) * spacing;
            d->color[0] = 1.0f; d->color[1] = 1.0f; d->color[2] = 1.0f; d->color[3] = d->pos[2] > 0 ? 0.0f : 0.2f;
            d->type = SPHMP_TYPE_BOUNDARY;
            c->mass = p->bmass;
            c->restdens = p->bRestdensity;
            c->visc = p->bvisc;
            *count = n + 1;
        }
    return 0;
}

/* SetupAddOpenBox (SPH_Solver/fluids/AddShape.cpp:355-366): the ground and four walls. */
int orc_add_open_box(const sphmp_params* p, const float mn[3], const float mx[3], float t, sphmp_display_pack* disp,
                     sphmp_calc_pack* calc, int32_t cap, int32_t* count) {
    const float walls[5][2][3] = {
        {{mn[0], mn[1] - t, mn[2]}, {mx[0], mn[1], mx[2]}},
        {{mn[0] - t, mn[1], mn[2] - t}, {mx[0] + t, mx[1], mn[2]}},
        {{mn[0] - t, mn[1], mx[2]}, {mx[0] + t, mx[1], mx[2] + t}},
        {{mn[0] - t, mn[1], mn[2]}, {mn[0], mx[1], mx[2]}},
        {{mx[0], mn[1], mn[2]}, {mx[0] + t, mx[1], mx[2]}},
    };
    for (int w = 0; w < 5; w++)
        if (orc_add_wall(p, walls[w][0], walls[w][1], disp, calc, cap, count)) return -1;
    return 0;
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_get_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
#endif /* !ORC_F64 */

/* ------------------------------------------------------------------------- */
/* Sort                                                                       */
/* ------------------------------------------------------------------------- */

/* GetParticleIndexCUDA (SPH_Solver/fluids/fluid_system_host.cu:147-159): clears
   mgridcnt/mgridoff/mgcell, then InitialSort (fluid_system_kern.cu:36-64): the cell
   of slot i is gs = (gy*res.z + gz)*res.x + gx with g = int((pos - gridmin)*gridIdfac);
   slots outside the interior cells [1, res-2] get GRID_UNDEF. midsort[i] = i. */
void FN(orc_get_particle_index)(const sphmp_params* p, ST* s) {
    memset(s->mgridcnt, 0, sizeof(int32_t) * (size_t)p->gridtotal);
    memset(s->mgridoff, 0, sizeof(int32_t) * (size_t)p->gridtotal);
    const int rx = p->gridres[0], ry = p->gridres[1], rz = p->gridres[2];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->n; i++) {
        float gcf[3];
        int gc[3];
        int inside = 1;
        for (int a = 0; a < 3; a++) {
            gcf[a] = ((float)s->pos[3 * i + a] - p->gridmin[a]) * p->gridIdfac[a];
            /* int(x) of a value outside int range (or NaN) is undefined in C++; the
               reference lands such particles in GRID_UNDEF on both host and GPU. */
            if (!(gcf[a] > -2147483520.0f && gcf[a] < 2147483520.0f)) { inside = 0; gc[a] = -1; }
            else gc[a] = (int)gcf[a];
        }
        if (inside && gc[0] >= 1 && gc[0] < rx - 1 && gc[1] >= 1 && gc[1] < ry - 1 && gc[2] >= 1 &&
            gc[2] < rz - 1)
            s->mgcell[i] = (uint32_t)((gc[1] * rz + gc[2]) * rx + gc[0]);
        else
            s->mgcell[i] = UNDEF;
        s->midsort[i] = (uint32_t)i;
    }
}

/* GetGridListCUDA (fluid_system_host.cu:161-185): thrust::sort_by_key(mgcell, midsort)
   is a stable sort on the cell key (ties keep slot order), restated as a sequential
   stable counting sort; then CalcFirstCnt (fluid_system_kern.cu:67-82) marks the head
   (mgridoff) and tail+1 (mgridcnt) of every run, and GetCnt (:84-95) turns the tail into
   a count and writes the rank-in-cell mgndx. */
void FN(orc_get_grid_list)(const sphmp_params* p, ST* s) {
    const int n = s->n;
    const int G = p->gridtotal;
    uint32_t* start = (uint32_t*)calloc((size_t)G + 2, sizeof(uint32_t));
    uint32_t* key = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) {
        uint32_t b = s->mgcell[i] == UNDEF ? (uint32_t)G : s->mgcell[i];
        start[b + 1]++;
    }
    for (int b = 0; b <= G; b++) start[b + 1] += start[b];
    for (int i = 0; i < n; i++) {
        uint32_t b = s->mgcell[i] == UNDEF ? (uint32_t)G : s->mgcell[i];
        uint32_t d = start[b]++;
        key[d] = s->mgcell[i];
        idx[d] = s->midsort[i];
    }
    memcpy(s->mgcell, key, sizeof(uint32_t) * (size_t)n);
    memcpy(s->midsort, idx, sizeof(uint32_t) * (size_t)n);
    free(start);
    free(key);
    free(idx);

    /* CalcFirstCnt */
    for (int i = 0; i < n; i++) {
        uint32_t c = s->mgcell[i];
        if (i == 0 || c != s->mgcell[i - 1]) {
            if (c != UNDEF) s->mgridoff[c] = i;
        }
        if (i != 0 && c != s->mgcell[i - 1] && s->mgcell[i - 1] != UNDEF) s->mgridcnt[s->mgcell[i - 1]] = i;
        if (i == n - 1 && c != UNDEF) s->mgridcnt[c] = i + 1;
    }
    /* GetCnt */
    for (int i = 0; i < n; i++) {
        uint32_t c = s->mgcell[i];
        if (c != UNDEF) {
            s->mgndx[i] = (uint32_t)(i - s->mgridoff[c]);
            if (s->mgndx[i] == 0) s->mgridcnt[c] -= s->mgridoff[c];
        }
    }
}

/* RearrageDataCUDA (fluid_system_host.cu:187-210): both record buffers are copied to
   msortbuf, then RearrangeData (fluid_system_kern.cu:98-121) gathers the record of
   pre-sort slot midsort[i] into sorted slot i. The kernel keeps the cell in an
   `int` and tests `cell != GRID_UNDEF` against the literal 4294967295, which is a
   64-bit `long` on LP64 hosts (every Linux / GB300 build), so the test is always
   true and out-of-grid slots are gathered like the others; their parking at
   (-1000,-1000,-1000) happens in AdvanceParticles. The legacy multiphase arrays
   travel with the record; mf_alpha_pre receives the sorted fractions (the
   start-of-step values the multiphase kernels read). MFidTable (written at :112,
   never read) is not restated. Returns 0 on success. */
int FN(orc_rearrange_data)(const sphmp_params* p, ST* s) {
    (void)p;
    const int n = s->n;
    if (n <= 0) return 0;
    size_t nn = (size_t)n;
#define DUP(field, T, k)                                                    \
    T* old_##field = (T*)malloc(sizeof(T) * nn * (k));                      \
    if (!old_##field) return -1;                                            \
    memcpy(old_##field, s->field, sizeof(T) * nn * (k));
    DUP(pos, R, 3) DUP(type, int32_t, 1) DUP(color, float, 4) DUP(vel, R, 3) DUP(veleval, R, 3)
    DUP(pressure, R, 1) DUP(dens, R, 1) DUP(restdens, R, 1) DUP(mass, R, 1) DUP(visc, R, 1)
    DUP(bornid, int32_t, 1) DUP(accel, R, 3) DUP(alpha, R, 3) DUP(aprev, R, 3)
#undef DUP
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        int e = (int)s->midsort[i];
#define MV(field, k) for (int c = 0; c < (k); c++) s->field[(size_t)i * (k) + c] = old_##field[(size_t)e * (k) + c];
        MV(pos, 3) MV(type, 1) MV(color, 4) MV(vel, 3) MV(veleval, 3) MV(pressure, 1) MV(dens, 1)
        MV(restdens, 1) MV(mass, 1) MV(visc, 1) MV(bornid, 1) MV(accel, 3) MV(alpha, 3) MV(aprev, 3)
#undef MV
        for (int k = 0; k < 3; k++) s->alpha_pre[3 * i + k] = s->alpha[3 * i + k];
    }
    free(old_pos); free(old_type); free(old_color); free(old_vel); free(old_veleval);
    free(old_pressure); free(old_dens); free(old_restdens); free(old_mass); free(old_visc);
    free(old_bornid); free(old_accel); free(old_alpha); free(old_aprev);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Density / boundary volume                                                  */
/* ------------------------------------------------------------------------- */

/* squared distance exactly as the reference: dist = (p_i - p_j)*simscale, then
   dist.x*dist.x + dist.y*dist.y + dist.z*dist.z evaluated left to right */
static inline R dist_sq(const ST* s, int i, int j, R ss, R d[3]) {
    d[0] = (s->pos[3 * i + 0] - s->pos[3 * j + 0]) * ss;
    d[1] = (s->pos[3 * i + 1] - s->pos[3 * j + 1]) * ss;
    d[2] = (s->pos[3 * i + 2] - s->pos[3 * j + 2]) * ss;
    return d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
}

/* ComputeBoundaryVolume + contributeDensity_boundary (fluid_system_kern.cu:183-212,
   249-277): V_b = 1 / (kpoly6 * sum over boundary j with r^2 < h^2 of (h^2 - r^2)^3). */
void FN(orc_compute_boundary_volume)(const sphmp_params* p, ST* s) {
    const R ss = (R)p->simscale;
    R r2 = (R)p->smoothradius;
    r2 = r2 * r2;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] != SPHMP_TYPE_BOUNDARY) continue;
        uint32_t gc = s->mgcell[i];
        if (gc == UNDEF) continue;
        R sum = (R)0.0;
        for (int c = 0; c < p->neighbornum; c++) {
            uint32_t cell = gc + (uint32_t)p->neighborid[c];
            if (s->mgridcnt[cell] == 0) continue;
            int cfirst = s->mgridoff[cell];
            int clast = cfirst + s->mgridcnt[cell];
            for (int j = cfirst; j < clast; j++) {
                if (s->type[j] != SPHMP_TYPE_BOUNDARY) continue;
                R d[3];
                R dsq = dist_sq(s, i, j, ss, d);
                if (dsq < r2) {
                    R cc = r2 - dsq;
                    sum += cc * cc * cc;
                }
            }
        }
        sum = sum * (R)p->kpoly6;
        if (sum == 0.0) sum = (R)1.0; /* the reference also prints "boundary density zero error." */
        s->dens[i] = 1 / sum;
    }
}

/* ComputeDensityPressure + contributeDensity (fluid_system_kern.cu:214-247, 279-318).
   rho_i = kpoly6 * sum_j (h^2-r^2)^3 m_j over r^2 < h^2 (self included), with
   m_j = mass_j for fluid j and restdens_i * V_j for boundary j. Stores 1/rho in dens
   and the Tait pressure 2.5*rho0*((rho/rho0)^7 - 1) (2.5 is a double literal),
   clamped at 0. The linear EOS extension evaluates k*(rho - rho0) in float. */
void FN(orc_compute_pressure)(const sphmp_params* p, ST* s) {
    const R ss = (R)p->simscale;
    R r2 = (R)p->smoothradius;
    r2 = r2 * r2;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == SPHMP_TYPE_BOUNDARY) continue;
        uint32_t gc = s->mgcell[i];
        if (gc == UNDEF) continue;
        R sum = (R)0.0;
        R dens = s->restdens[i];
        for (int c = 0; c < p->neighbornum; c++) {
            uint32_t cell = gc + (uint32_t)p->neighborid[c];
            if (s->mgridcnt[cell] == 0) continue;
            int cfirst = s->mgridoff[cell];
            int clast = cfirst + s->mgridcnt[cell];
            R massj = (R)0;
            for (int j = cfirst; j < clast; j++) {
                if (s->type[j] == 0) massj = s->mass[j];
                else if (s->type[j] == 1) massj = s->restdens[i] * s->dens[j];
                R d[3];
                R dsq = dist_sq(s, i, j, ss, d);
                if (dsq < r2) {
                    R cc = r2 - dsq;
                    sum += cc * cc * cc * massj;
                }
            }
        }
        sum = sum * (R)p->kpoly6;
        if (sum == 0.0) sum = (R)1.0;
        s->dens[i] = 1 / sum;
        R pr;
        if (p->eos == SPHMP_EOS_LINEAR)
            pr = (R)p->eos_stiffness * (sum - dens);
        else
            pr = (R)(2.5 * (double)dens * (double)(RPOW(sum / dens, (R)7.0f) - 1));
        if (pr < 0) pr = 0;
        s->pressure[i] = pr;
    }
}

/* ------------------------------------------------------------------------- */
/* Force, surface tension, advance                                            */
/* ------------------------------------------------------------------------- */

/* ComputeForce + contributeForce_new (fluid_system_kern.cu:325-424). Pairs with
   0 < r^2 < h^2; g1 = kspikydiff*(h-r)^2/r, g = g1*m_j*dens_j. Fluid j: pressure
   x_ij*(-0.5*g*p_j*(1/rho_i)) [in double] and viscosity (v_i - v_j)*g*(nu_i+nu_j)/rho_i.
   Boundary j: x_ij*(-g1*rho0_i*V_j*p_i/rho_i^2) plus the artificial viscosity when
   (v_i - v_j).x_ij < 0. The velocity used for i and j is `vel` (:410, :372). Each
   cell's contributions are summed separately and then added to the total (:420). */
void FN(orc_compute_force)(const sphmp_params* p, ST* s) {
    const R ss = (R)p->simscale;
    const R h = (R)p->smoothradius;
    R r2 = h;
    r2 = r2 * r2;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == 1) continue;
        uint32_t gc = s->mgcell[i];
        if (gc == UNDEF) continue;
        const R iv[3] = {s->vel[3 * i + 0], s->vel[3 * i + 1], s->vel[3 * i + 2]};
        const R ipress = s->pressure[i];
        const R idens = s->dens[i];
        const R ivisc = s->visc[i];
        R force[3] = {0, 0, 0};
        for (int c = 0; c < p->neighbornum; c++) {
            uint32_t cell = gc + (uint32_t)p->neighborid[c];
            if (s->mgridcnt[cell] == 0) continue;
            int cfirst = s->mgridoff[cell];
            int clast = cfirst + s->mgridcnt[cell];
            R cf[3] = {0, 0, 0};
            for (int j = cfirst; j < clast; j++) {
                R d[3];
                R dsq = dist_sq(s, i, j, ss, d);
                if (!(dsq < r2 && dsq > 0)) continue;
                dsq = RSQRT(dsq);
                R cc = (h - dsq);
                R cmterm1 = (R)p->kspikydiff * cc * cc / dsq;
                R cmterm = cmterm1 * s->mass[j] * s->dens[j];
                if (s->type[j] == 0) {
                    R pmterm = (R)(-0.5 * (double)cmterm * (double)s->pressure[j] * (double)idens);
                    cf[0] += d[0] * pmterm;
                    cf[1] += d[1] * pmterm;
                    cf[2] += d[2] * pmterm;
                    R vmr[3] = {iv[0] - s->vel[3 * j + 0], iv[1] - s->vel[3 * j + 1], iv[2] - s->vel[3 * j + 2]};
                    R vmterm = cmterm * (ivisc + s->visc[j]) * idens;
                    cf[0] += vmr[0] * vmterm;
                    cf[1] += vmr[1] * vmterm;
                    cf[2] += vmr[2] * vmterm;
                } else if (s->type[j] == 1) {
                    R pmterm = -cmterm1 * s->restdens[i] * s->dens[j] * (ipress)*idens * idens;
                    cf[0] += d[0] * pmterm;
                    cf[1] += d[1] * pmterm;
                    cf[2] += d[2] * pmterm;
                    R vmr[3] = {iv[0] - s->vel[3 * j + 0], iv[1] - s->vel[3 * j + 1], iv[2] - s->vel[3 * j + 2]};
                    R pi_ij = vmr[0] * d[0] + vmr[1] * d[1] + vmr[2] * d[2];
                    if (pi_ij < 0) {
                        pi_ij = (R)((double)pi_ij / ((double)(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) + (double)r2 * 0.01));
                        pi_ij = pi_ij * (R)p->bvisc * h / 2 / s->restdens[i];
                        pi_ij = cmterm1 * s->restdens[i] * s->dens[j] * pi_ij;
                        cf[0] += d[0] * pi_ij;
                        cf[1] += d[1] * pi_ij;
                        cf[2] += d[2] * pi_ij;
                    }
                }
            }
            force[0] += cf[0];
            force[1] += cf[1];
            force[2] += cf[2];
        }
        s->accel[3 * i + 0] = force[0];
        s->accel[3 * i + 1] = force[1];
        s->accel[3 * i + 2] = force[2];
    }
}

/* SurfaceTension + contributeSurfaceTensionYT (fluid_system_kern.cu:569-625; launch
   commented at fluid_system_host.cu:433-437). For every in-grid slot (boundary
   included), a += sum_j C*cos(1.5*3.14159*r/R)/r * x_ij over 0 != r^2 <= R, R = K*h
   (the squared distance is compared with R itself, as in the reference). */
void FN(orc_surface_tension)(const sphmp_params* p, ST* s) {
    const R ss = (R)p->simscale;
    R sr2 = (R)p->smoothradius;
    sr2 *= sr2;
    const R tensionRadius2 = (R)p->surfaceTensionK * (R)p->surfaceTensionK * sr2;
    const R tR = RSQRT(tensionRadius2);
    const R C = (R)p->surfaceTensionFluidC;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        uint32_t gc = s->mgcell[i];
        if (gc == UNDEF) continue;
        R res[3] = {0, 0, 0};
        for (int c = 0; c < p->neighbornum; c++) {
            uint32_t cell = gc + (uint32_t)p->neighborid[c];
            if (s->mgridcnt[cell] == 0) continue;
            int cfirst = s->mgridoff[cell];
            int clast = cfirst + s->mgridcnt[cell];
            for (int j = cfirst; j < clast; j++) {
                R d[3];
                R dsq = dist_sq(s, i, j, ss, d);
                if (dsq != 0.0 && dsq <= tR) {
                    dsq = RSQRT(dsq);
                    R forceMod = (R)((double)C * cos(1.5 * 3.14159 * (double)dsq / (double)tR) / (double)dsq);
                    res[0] += d[0] * forceMod;
                    res[1] += d[1] * forceMod;
                    res[2] += d[2] * forceMod;
                }
            }
        }
        s->accel[3 * i + 0] += res[0];
        s->accel[3 * i + 1] += res[1];
        s->accel[3 * i + 2] += res[2];
    }
}

/* AdvanceParticles (fluid_system_kern.cu:426-534): boundary slots are skipped; an
   out-of-grid slot is parked at (-1000)^3 with zero velocity; otherwise
   a = accel + gravity, v' = a*dt + v, pos += v'*dt/simscale, veleval = (v+v')*0.5,
   vel = v'. The drift velocity of the next step reads mforce = gravity - a, the
   convention of the legacy advance (SPH_Solver/fluids/MpmSolver.cu:1687) whose
   counterpart in the SPH advance is commented out (fluid_system_kern.cu:524). */
void FN(orc_advance)(const sphmp_params* p, ST* s) {
    const R dt = (R)p->dt;
    const R ss = (R)p->simscale;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == 1) continue;
        if (s->mgcell[i] == UNDEF) {
            s->pos[3 * i + 0] = -1000;
            s->pos[3 * i + 1] = -1000;
            s->pos[3 * i + 2] = -1000;
            s->vel[3 * i + 0] = 0;
            s->vel[3 * i + 1] = 0;
            s->vel[3 * i + 2] = 0;
            continue;
        }
        for (int a = 0; a < 3; a++) {
            R acc = (R)0;
            acc += s->accel[3 * i + a];
            acc += (R)p->gravity[a];
            R v = s->vel[3 * i + a];
            R vnext = acc * dt + v;
            s->pos[3 * i + a] += vnext * dt / ss;
            s->veleval[3 * i + a] = (v + vnext) * (R)0.5f;
            s->vel[3 * i + a] = vnext;
            s->aprev[3 * i + a] = (R)p->gravity[a] - acc;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Multiphase (drift-flux mixture model), SPH_Solver/fluids/multiphase.cu     */
/* ------------------------------------------------------------------------- */
/* Legacy field mapping: mpos=pos, mveleval=veleval, mpress=pressure, mdensity=dens
   (1/rho), mf_restmass=mass, mf_restdensity=restdens, mf_visc=visc, misbound[j]==1
   and MFtype[j]==1 both mean type==TYPE_BOUNDARY, mgrid[] is the identity after the
   sort, and gc - nadj + gridAdj[c] == gc + neighborid[c] (same y,z,x order).
   simData: psimscale=simscale, r2=h*h, psmoothradius=h, spikykern=kspikydiff,
   mf_catnum=nphase, mf_dens=densArr, mf_visc=viscArr, mf_dt=dt. */

/* mfComputeDriftVel + contributeDriftVel (multiphase.cu:19-166). */
void FN(orc_compute_drift_vel)(const sphmp_params* p, ST* s) {
    const int np = p->nphase;
    const R ss = (R)p->simscale;
    const R h = (R)p->smoothradius;
    const R d2 = ss * ss;
    const R r2 = (h * h) / d2;
    const R spikykern = (R)p->kspikydiff;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == 1) continue;
        uint32_t gc = s->mgcell[i];
        if (gc == UNDEF) continue;
        R relax_coef = (R)p->mf_relax;
        const R sigma = (R)p->mf_diffusion;
        const R cont = (R)p->mf_cont, conts = (R)p->mf_cont1, contr = (R)p->mf_cont2;
        const R accel[3] = {s->aprev[3 * i + 0], s->aprev[3 * i + 1], s->aprev[3 * i + 2]};
        const R invdens = (R)(1.0 / (double)s->restdens[i]);
        const R ipress = s->pressure[i];
        const R ipos[3] = {s->pos[3 * i + 0], s->pos[3 * i + 1], s->pos[3 * i + 2]};
        R alpha_pre[3], mass_concen[3], drift[3][3], agrad[3][3], sterm[3][3];
        relax_coef /= s->visc[i];
        for (int k = 0; k < np; k++) {
            alpha_pre[k] = s->alpha_pre[3 * i + k];
            mass_concen[k] = alpha_pre[k] * (R)p->densArr[k] * invdens;
            for (int a = 0; a < 3; a++) drift[k][a] = agrad[k][a] = 0;
        }
        for (int c = 0; c < p->neighbornum; c++) {
            uint32_t cell = gc + (uint32_t)p->neighborid[c];
            if (s->mgridcnt[cell] == 0) continue;
            int cfirst = s->mgridoff[cell];
            int clast = cfirst + s->mgridcnt[cell];
            for (int j = cfirst; j < clast; j++) {
                if (s->type[j] == 1) continue;
                R d[3] = {ipos[0] - s->pos[3 * j + 0], ipos[1] - s->pos[3 * j + 1], ipos[2] - s->pos[3 * j + 2]};
                R dsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                d[0] *= ss; d[1] *= ss; d[2] *= ss;
                if (dsq < r2 && dsq > 0) {
                    dsq = RSQRT(dsq * d2);
                    R cc = (h - dsq);
                    R cmterm = spikykern * cc * cc / dsq * s->mass[j] * s->dens[j];
                    R pgrad[3][3];
                    R pgradsum[3] = {0, 0, 0};
                    for (int k = 0; k < np; k++) {
                        R ja = s->alpha_pre[3 * j + k];
                        R pmterm = cmterm * (-alpha_pre[k] * ipress + ja * s->pressure[j]);
                        for (int a = 0; a < 3; a++) {
                            pgrad[k][a] = pmterm * d[a];
                            pgradsum[a] += pgrad[k][a] * mass_concen[k];
                            agrad[k][a] += (ja - alpha_pre[k]) * cmterm * d[a];
                        }
                    }
                    for (int k = 0; k < np; k++)
                        for (int a = 0; a < 3; a++) drift[k][a] -= relax_coef * (pgrad[k][a] - pgradsum[a]);
                }
            }
        }
        for (int k = 0; k < np; k++)
            for (int a = 0; a < 3; a++) s->drift[9 * i + 3 * k + a] = cont * contr * drift[k][a];
        R dsum = 0;
        R ssum[3] = {0, 0, 0};
        for (int k = 0; k < np; k++) {
            R temp = s->alpha_pre[3 * i + k];
            dsum += temp * (R)p->densArr[k] * (R)p->densArr[k] * invdens;
            for (int a = 0; a < 3; a++) {
                if ((double)temp > 0.0001) sterm[k][a] = agrad[k][a] / temp;
                else sterm[k][a] = 0;
                ssum[a] += sterm[k][a] * temp * (R)p->densArr[k] * invdens;
            }
        }
        for (int k = 0; k < np; k++) {
            R tdiff = (R)p->densArr[k] - dsum;
            tdiff *= relax_coef;
            for (int a = 0; a < 3; a++) {
                s->drift[9 * i + 3 * k + a] += accel[a] * tdiff;
                s->drift[9 * i + 3 * k + a] -= cont * conts * sigma * (sterm[k][a] - ssum[a]);
            }
        }
    }
}

/* mfComputeAlphaAdvance + contributeAlphaChange (multiphase.cu:169-272).
   dalpha_k = -sum_j g'[0.5(a_jk + a_ik)((ve_j - ve_i).x_ij) + (a_jk u_jk + a_ik u_ik).x_ij],
   times dt, clamped at -0.99, added to alpha_pre. The phase-2 "becomes water" type
   flip (:268-271) belongs to the granular model and is not restated. */
void FN(orc_compute_alpha_advance)(const sphmp_params* p, ST* s) {
    const int np = p->nphase;
    const R ss = (R)p->simscale;
    const R h = (R)p->smoothradius;
    const R d2 = ss * ss;
    const R r2 = (h * h) / d2;
    const R spikykern = (R)p->kspikydiff;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == 1) continue;
        uint32_t gc = s->mgcell[i];
        if (gc == UNDEF) continue;
        const R ipos[3] = {s->pos[3 * i + 0], s->pos[3 * i + 1], s->pos[3 * i + 2]};
        const R ive[3] = {s->veleval[3 * i + 0], s->veleval[3 * i + 1], s->veleval[3 * i + 2]};
        R alpha_pre[3], change[3], ivmk[3][3];
        for (int k = 0; k < np; k++) {
            alpha_pre[k] = s->alpha_pre[3 * i + k];
            change[k] = (R)0.0f;
            for (int a = 0; a < 3; a++) ivmk[k][a] = s->drift[9 * i + 3 * k + a];
        }
        for (int c = 0; c < p->neighbornum; c++) {
            uint32_t cell = gc + (uint32_t)p->neighborid[c];
            if (s->mgridcnt[cell] == 0) continue;
            int cfirst = s->mgridoff[cell];
            int clast = cfirst + s->mgridcnt[cell];
            for (int j = cfirst; j < clast; j++) {
                if (s->type[j] == 1) continue;
                R d[3] = {ipos[0] - s->pos[3 * j + 0], ipos[1] - s->pos[3 * j + 1], ipos[2] - s->pos[3 * j + 2]};
                R dsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                d[0] *= ss; d[1] *= ss; d[2] *= ss;
                if (dsq < r2 && dsq > 0) {
                    dsq = RSQRT(dsq * d2);
                    R cc = (h - dsq);
                    R cmterm = spikykern * cc * cc / dsq * s->mass[j] * s->dens[j];
                    R vmr[3] = {s->veleval[3 * j + 0] - ive[0], s->veleval[3 * j + 1] - ive[1], s->veleval[3 * j + 2] - ive[2]};
                    for (int k = 0; k < np; k++) {
                        R ja = s->alpha_pre[3 * j + k];
                        change[k] = (R)((double)change[k] -
                                        0.5 * (double)cmterm * (double)(ja + alpha_pre[k]) *
                                            (double)(vmr[0] * d[0] + vmr[1] * d[1] + vmr[2] * d[2]));
                        R vkr[3];
                        for (int a = 0; a < 3; a++) vkr[a] = ja * s->drift[9 * j + 3 * k + a] + alpha_pre[k] * ivmk[k][a];
                        change[k] -= cmterm * (vkr[0] * d[0] + vkr[1] * d[1] + vkr[2] * d[2]);
                    }
                }
            }
        }
        for (int k = 0; k < np; k++) {
            change[k] *= (R)p->dt;
            if ((double)change[k] < -0.99) change[k] = (R)-0.99;
            s->alpha[3 * i + k] = change[k] + alpha_pre[k];
        }
    }
}

/* mfComputeCorrection (multiphase.cu:275-349): clamp alpha at 0 and renormalise,
   or one-hot at the largest alpha_pre when every fraction vanished; accumulate the
   pressure correction -(6*(rho/rho0)^7 + 1)*pintstiff*rho_k*dalpha_k (pow(float, int)
   promotes to double in C++); rest density and viscosity become the
   alpha-weighted phase values (rest density kept for MFtype 1 and 2). */
void FN(orc_compute_correction)(const sphmp_params* p, ST* s) {
    const int np = p->nphase;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == 1) continue;
        if (s->mgcell[i] == UNDEF) continue;
        R sum = (R)0.0f;
        R apre[3];
        for (int k = 0; k < np; k++) {
            R* t = &s->alpha[3 * i + k];
            apre[k] = *t;
            if (*t < 0.0000) *t = (R)0.0f;
            sum += *t;
        }
        s->pmod[i] = (R)0.0f;
        int flag = (sum > 0.0f);
        sum = flag * sum + (1 - flag) * (R)1.0f;
        int maxcat = 0;
        for (int k = 1; k < np; k++)
            if (s->alpha_pre[3 * i + k] > s->alpha_pre[3 * i + maxcat]) maxcat = k;
        sum = (R)1.0f / sum;
        for (int k = 0; k < np; k++) {
            R* t = &s->alpha[3 * i + k];
            *t = (flag) * (*t) * sum + (1 - flag) * (k == maxcat ? 1 : 0);
            R alpha_modify = *t - apre[k];
            R x = 1 / (s->dens[i] * s->restdens[i]);
            s->pmod[i] = (R)((double)s->pmod[i] + -(6 * pow((double)x, 7) + 1.0) * (double)p->mf_pintstiff *
                                                       (double)p->densArr[k] * (double)alpha_modify);
        }
        R newdens = (R)0.0, newvisc = (R)0.0;
        for (int k = 0; k < np; k++) {
            newdens += s->alpha[3 * i + k] * (R)p->densArr[k];
            newvisc += s->alpha[3 * i + k] * (R)p->viscArr[k];
        }
        if (s->type[i] != 2 && s->type[i] != 1) s->restdens[i] = newdens;
        s->visc[i] = newvisc;
    }
}

/* ComputeForce_projectu + contributeForce_projectu (multiphase.cu:488-616; the
   launch in ComputeForceCUDA_ProjectU, fluid_system_host.cu:396-419, is commented
   out). For every in-grid non-boundary slot, per neighbour cell, over 0 < r^2 < h^2:
   fluid j: pressure -0.5 g (p_i + p_j) D_i x_ij, viscosity g (nu_i + nu_j) D_i
   (ve_i - ve_j), drift tensor sum_k (g (u_jk.x_ij) a_jk u_jk + g (u_ik.x_ij) a_ik u_ik)
   rho_k D_i, with g = kspikydiff (h - r)^2 / r m_j D_j and D the stored inverse
   density; boundary j: pressure -g1 rho0_i m_j / rho0_j p_i D_i^2 x_ij omega and,
   when (ve_i - ve_j).x_ij < 0, the artificial viscosity times visc_factor; every
   j adds the XSPH term -(ve_i - ve_j) cx^3 m_j 2/(1/D_j + 1/D_i) kpoly6 0.5 to
   velxcor (cx = (r2 - r^2) d2, a double literal 0.5). Per-cell force sums are
   added to the total, velxcor accumulates directly; mforce is accel here.
   Boundary and out-of-grid slots are left untouched, as in the reference. */
void FN(orc_compute_force_projectu)(const sphmp_params* p, ST* s) {
    const int np = p->nphase;
    const R ss = (R)p->simscale;
    const R h = (R)p->smoothradius;
    const R d2 = ss * ss;
    R r2h = h;
    r2h = r2h * r2h;
    const R r2 = r2h / d2;
    const R spikykern = (R)p->kspikydiff;
    const R poly6 = (R)p->kpoly6;
    const R omega = (R)p->mf_omega, vfac = (R)p->mf_visc_factor;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == 1) continue;
        uint32_t gc = s->mgcell[i];
        if (gc == UNDEF) continue;
        const R ipos[3] = {s->pos[3 * i + 0], s->pos[3 * i + 1], s->pos[3 * i + 2]};
        const R ive[3] = {s->veleval[3 * i + 0], s->veleval[3 * i + 1], s->veleval[3 * i + 2]};
        const R ipress = s->pressure[i];
        const R idens = s->dens[i];
        const R ivisc = s->visc[i];
        R alpha_pre[3], ivmk[3][3];
        for (int k = 0; k < np; k++) {
            alpha_pre[k] = s->alpha_pre[3 * i + k];
            for (int a = 0; a < 3; a++) ivmk[k][a] = s->drift[9 * i + 3 * k + a];
        }
        R force[3] = {0, 0, 0};
        R* xc = &s->velxcor[3 * i];
        xc[0] = xc[1] = xc[2] = 0;
        for (int c = 0; c < p->neighbornum; c++) {
            uint32_t cell = gc + (uint32_t)p->neighborid[c];
            if (s->mgridcnt[cell] == 0) continue;
            int cfirst = s->mgridoff[cell];
            int clast = cfirst + s->mgridcnt[cell];
            R cf[3] = {0, 0, 0};
            for (int j = cfirst; j < clast; j++) {
                R d[3] = {ipos[0] - s->pos[3 * j + 0], ipos[1] - s->pos[3 * j + 1], ipos[2] - s->pos[3 * j + 2]};
                R dsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                d[0] *= ss; d[1] *= ss; d[2] *= ss;
                if (!(dsq < r2 && dsq > 0)) continue;
                const R cx = (r2 - dsq) * d2;
                dsq = RSQRT(dsq * d2);
                const R cc = (h - dsq);
                const R cmterm1 = spikykern * cc * cc / dsq;
                const R cmterm = spikykern * cc * cc / dsq * s->mass[j] * s->dens[j];
                R vmr[3];
                if (s->type[j] != 1) {
                    const R pmterm = (R)-0.5f * cmterm * (ipress + s->pressure[j]) * idens;
                    for (int a = 0; a < 3; a++) cf[a] += pmterm * d[a];
                    for (int a = 0; a < 3; a++) vmr[a] = ive[a] - s->veleval[3 * j + a];
                    const R vmterm = cmterm * (ivisc + s->visc[j]) * idens;
                    for (int a = 0; a < 3; a++) cf[a] += vmterm * vmr[a];
                } else {
                    const R pmterm =
                        -cmterm1 * s->restdens[i] * s->mass[j] / s->restdens[j] * (ipress)*s->dens[i] * s->dens[i];
                    for (int a = 0; a < 3; a++) cf[a] += pmterm * d[a] * omega;
                    for (int a = 0; a < 3; a++) vmr[a] = ive[a] - s->veleval[3 * j + a];
                    R pi_ij = vmr[0] * d[0] + vmr[1] * d[1] + vmr[2] * d[2];
                    if (pi_ij < 0) {
                        pi_ij = (R)((double)pi_ij / ((double)(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) + (double)r2 * 0.01));
                        pi_ij = pi_ij * (R)2 * h * (ivisc + s->visc[j]) * idens / (R)2;
                        pi_ij = -cmterm1 * s->restdens[i] * s->mass[j] / s->restdens[j] * pi_ij;
                        for (int a = 0; a < 3; a++) cf[a] += pi_ij * d[a] * vfac;
                    }
                }
                if (s->type[j] != 1) {
                    for (int k = 0; k < np; k++) {
                        const R* uj = &s->drift[9 * j + 3 * k];
                        const R tj = cmterm * (uj[0] * d[0] + uj[1] * d[1] + uj[2] * d[2]) * s->alpha_pre[3 * j + k];
                        const R ti = cmterm * (ivmk[k][0] * d[0] + ivmk[k][1] * d[1] + ivmk[k][2] * d[2]) * alpha_pre[k];
                        for (int a = 0; a < 3; a++)
                            cf[a] += (tj * uj[a] + ti * ivmk[k][a]) * (R)p->densArr[k] * idens;
                    }
                }
                const R ave = (R)2 / ((R)1 / s->dens[j] + (R)1 / idens);
                const R xterm = (R)((double)(cx * cx * cx * s->mass[j] * ave * poly6) * 0.5);
                for (int a = 0; a < 3; a++) xc[a] += -vmr[a] * xterm;
            }
            force[0] += cf[0];
            force[1] += cf[1];
            force[2] += cf[2];
        }
        s->accel[3 * i + 0] = force[0];
        s->accel[3 * i + 1] = force[1];
        s->accel[3 * i + 2] = force[2];
    }
}

/* ------------------------------------------------------------------------- */
/* Step composition                                                            */
/* ------------------------------------------------------------------------- */

/* FluidSystem::BeforeFirstStep (fluid_system.cpp:62-70): sort, then boundary volumes. */
/* ------------------------------------------------------------------------- */
/* IISPH (fluid_system_kern.cu:637-1115, the launches of fluid_system_host.cu:504-557) */
/* ------------------------------------------------------------------------- */

/* kern (:637-645): the cubic spline of support 2h, kspline = 1/(pi h^3). */
static inline R FN(iikern)(const sphmp_params* p, const R d[3]) {
    R q = RSQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) / (R)p->smoothradius;
    if (q > 2) return (R)0;
    else if (q > 1) return (R)0.25f * RPOW(2 - q, (R)3.0f) * (R)p->kspline;
    else return (1 - (R)1.5f * q * q + (R)0.75f * RPOW(q, (R)3.0f)) * (R)p->kspline;
}

/* nablakern (:647-671): its gradient, r * fac. */
static inline void FN(iinabla)(const sphmp_params* p, const R d[3], R out[3]) {
    R rmod = RSQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    R q = rmod / (R)p->smoothradius;
    R fac = 0;
    if (q > 2) {
        out[0] = out[1] = out[2] = 0;
        return;
    } else if (q > 1) {
        fac = (R)0.75f * (2 - q) * (2 - q) * (-1) / (R)p->smoothradius / rmod * (R)p->kspline;
    } else {
        fac = (-3 * q + (R)2.25f * q * q) / (R)p->smoothradius / rmod * (R)p->kspline;
    }
    out[0] = d[0] * fac;
    out[1] = d[1] * fac;
    out[2] = d[2] * fac;
}

/* the reference's 27-cell loop around particle i's cell (gc + neighborid[c]),
   skipping empty cells, with the cell's slot range [cfirst, clast) */
#define II_CELLS(i, ...)                                                    \
    for (int c = 0; c < p->neighbornum; c++) {                              \
        uint32_t cell = s->mgcell[i] + (uint32_t)p->neighborid[c];          \
        if (s->mgridcnt[cell] == 0) continue;                               \
        int cfirst = s->mgridoff[cell];                                     \
        int clast = cfirst + s->mgridcnt[cell];                             \
        __VA_ARGS__                                                         \
    }

/* ComputeDensityIISPH + contributeIIDensity (:1067-1115): the density itself
   (not its inverse) over every candidate of the 27 cells, with m_j = mass_j for
   fluid and restdens_i * V_j for boundary neighbours. */
void FN(orc_iisph_density)(const sphmp_params* p, ST* s) {
    const R ss = (R)p->simscale;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == SPHMP_TYPE_BOUNDARY) continue;
        if (s->mgcell[i] == UNDEF) continue;
        R sum = (R)0.0;
        R massj = 0;
        II_CELLS(i, {
            for (int j = cfirst; j < clast; j++) {
                if (s->type[j] == 0) massj = s->mass[j];
                else if (s->type[j] == 1) massj = s->restdens[i] * s->dens[j];
                R d[3];
                dist_sq(s, i, j, ss, d);
                sum += FN(iikern)(p, d) * massj;
            }
        })
        s->dens[i] = sum;
    }
}

/* PredictAdvection (:516-524): ComputeDii (:673-799) then ComputeAii (:801-908).
   ComputeDii: the advection acceleration (boundary artificial viscosity within
   2h, per cell, plus gravity) gives veleval = vel + a_adv dt; dii = -sum over
   fluid j within h of nabla W_ij m_j, / rho_i / rho_i * dt * dt.
   ComputeAii: rho_adv = rho_i + dt sum_j m_j (veleval_i - veleval_j).nabla W_ij,
   press_l = 0.5 p_i (0.5 a double literal), aii = sum_j m_j (dii - dji).nabla W_ij
   with dji = nabla W_ij m_i / rho_i / rho_i dt dt. */
void FN(orc_iisph_predict)(const sphmp_params* p, ST* s) {
    const R ss = (R)p->simscale;
    const R h = (R)p->smoothradius;
    const R h2 = h * h;
    const R dt = (R)p->dt;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == SPHMP_TYPE_BOUNDARY) continue;
        if (s->mgcell[i] == UNDEF) continue;
        R acc[3] = {0, 0, 0};
        II_CELLS(i, {
            R accel[3] = {0, 0, 0};
            for (int j = cfirst; j < clast; j++) {
                R d[3];
                dist_sq(s, i, j, ss, d);
                R dist = RSQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (!(dist < 2 * h && dist > 0)) continue;
                R nw[3];
                FN(iinabla)(p, d, nw);
                if (s->type[j] == 1) {
                    R vij[3];
                    for (int a = 0; a < 3; a++) vij[a] = s->vel[3 * i + a] - s->vel[3 * j + a];
                    R pi_ij = d[0] * vij[0] + d[1] * vij[1] + d[2] * vij[2];
                    if (pi_ij < 0) {
                        pi_ij = (R)(pi_ij / (dist * dist + h2 * 0.01));
                        pi_ij = pi_ij * (R)p->bvisc * (R)p->smoothradius / 2 / s->restdens[i];
                        pi_ij = s->restdens[i] * s->dens[j] * pi_ij;
                        for (int a = 0; a < 3; a++) accel[a] += nw[a] * pi_ij;
                    }
                }
            }
            for (int a = 0; a < 3; a++) acc[a] = acc[a] + accel[a];
        })
        for (int a = 0; a < 3; a++) acc[a] += (R)p->gravity[a];
        for (int a = 0; a < 3; a++) s->veleval[3 * i + a] = s->vel[3 * i + a] + acc[a] * dt;
        R dii[3] = {0, 0, 0};
        II_CELLS(i, {
            for (int j = cfirst; j < clast; j++) {
                R d[3];
                dist_sq(s, i, j, ss, d);
                R dist = RSQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (!(dist < h && dist > 0)) continue;
                R nw[3];
                FN(iinabla)(p, d, nw);
                if (s->type[j] != SPHMP_TYPE_BOUNDARY)
                    for (int a = 0; a < 3; a++) dii[a] = dii[a] - nw[a] * s->mass[j];
            }
        })
        for (int a = 0; a < 3; a++) s->dii[3 * i + a] = dii[a] / s->dens[i] / s->dens[i] * dt * dt;
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == SPHMP_TYPE_BOUNDARY) continue;
        if (s->mgcell[i] == UNDEF) continue;
        R denschange = 0;
        II_CELLS(i, {
            R sum = 0;
            for (int j = cfirst; j < clast; j++) {
                R d[3];
                dist_sq(s, i, j, ss, d);
                R dist = RSQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (!(dist < h && dist > 0)) continue;
                R vij[3];
                for (int a = 0; a < 3; a++) vij[a] = s->veleval[3 * i + a] - s->veleval[3 * j + a];
                R nw[3];
                FN(iinabla)(p, d, nw);
                if (s->type[j] != SPHMP_TYPE_BOUNDARY)
                    sum += (vij[0] * nw[0] + vij[1] * nw[1] + vij[2] * nw[2]) * s->mass[j] * dt;
            }
            denschange += sum;
        })
        s->rho_adv[i] = s->dens[i] + denschange;
        s->press_l[i] = (R)(0.5 * (double)s->pressure[i]);
        R aii = 0;
        II_CELLS(i, {
            R sum = 0;
            for (int j = cfirst; j < clast; j++) {
                if (s->type[j] == SPHMP_TYPE_BOUNDARY) continue;
                R d[3];
                dist_sq(s, i, j, ss, d);
                R dist = RSQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (!(dist < h && dist > 0)) continue;
                R nw[3];
                FN(iinabla)(p, d, nw);
                R dtmp[3];
                for (int a = 0; a < 3; a++) {
                    R dji = nw[a] * s->mass[i] / s->dens[i] / s->dens[i] * dt * dt;
                    dtmp[a] = s->dii[3 * i + a] - dji;
                }
                sum += (dtmp[0] * nw[0] + dtmp[1] * nw[1] + dtmp[2] * nw[2]) * s->mass[j];
            }
            aii += sum;
        })
        s->aii[i] = aii;
    }
}

/* One relaxed-Jacobi iteration of PressureSolve (:526-549): Pressure_DP (:910-958)
   dijpj = -dt dt sum over fluid j within h of nabla W_ij p_j m_j / rho_j / rho_j;
   Pressure_Iter (:960-1050) with omega 0.1: p_l1 = (1 - omega) p_l + omega / aii
   (rho0 - rho_adv - sum_j m_j (dijpj_i - djj p_j - (dijpj_j - dji p_i)).nabla W_ij)
   (p_l1 = p_l where |aii| < 1e-5), the density residue, accel = (dii p_l +
   dijpj) / dt / dt and pressure = p_l1; then p_l = p_l1 (the device copy).
   Returns the reference's criterion quantity: the residues summed over all slots
   (boundary particles 0) divided by the slot count. */
double FN(orc_iisph_iteration)(const sphmp_params* p, ST* s) {
    const R ss = (R)p->simscale;
    const R h = (R)p->smoothradius;
    const R dt = (R)p->dt;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == SPHMP_TYPE_BOUNDARY) continue;
        if (s->mgcell[i] == UNDEF) continue;
        R dp[3] = {0, 0, 0};
        II_CELLS(i, {
            for (int j = cfirst; j < clast; j++) {
                if (s->type[j] == SPHMP_TYPE_BOUNDARY) continue;
                R d[3];
                dist_sq(s, i, j, ss, d);
                R dist = RSQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (!(dist < h && dist > 0)) continue;
                R nw[3];
                FN(iinabla)(p, d, nw);
                for (int a = 0; a < 3; a++)
                    dp[a] = dp[a] + nw[a] * s->press_l[j] * s->mass[j] / s->dens[j] / s->dens[j] * (-1);
            }
        })
        for (int a = 0; a < 3; a++) s->dijpj[3 * i + a] = dp[a] * dt * dt;
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == SPHMP_TYPE_BOUNDARY) {
            s->residue[i] = 0;
            continue;
        }
        if (s->mgcell[i] == UNDEF) continue;
        R updateterm = 0;
        II_CELLS(i, {
            for (int j = cfirst; j < clast; j++) {
                R d[3];
                dist_sq(s, i, j, ss, d);
                R dist = RSQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (!(dist < h && dist > 0)) continue;
                R nw[3];
                FN(iinabla)(p, d, nw);
                if (s->type[j] != SPHMP_TYPE_BOUNDARY) {
                    R tmp[3];
                    for (int a = 0; a < 3; a++) {
                        R dji = nw[a] * s->mass[i] / s->dens[i] / s->dens[i] * dt * dt;
                        R djkpk = s->dijpj[3 * j + a] - dji * s->press_l[i];
                        tmp[a] = s->dijpj[3 * i + a] - s->dii[3 * j + a] * s->press_l[j] - djkpk;
                    }
                    updateterm += s->mass[j] * (tmp[0] * nw[0] + tmp[1] * nw[1] + tmp[2] * nw[2]);
                }
            }
        })
        const R omega = (R)0.1f;
        R aii = s->aii[i];
        if ((aii < 0 ? -aii : aii) < (R)0.00001f)
            s->press_l1[i] = s->press_l[i];
        else
            s->press_l1[i] = (1 - omega) * s->press_l[i] + omega / aii * (s->restdens[i] - s->rho_adv[i] - updateterm);
        s->residue[i] = -s->restdens[i] + (s->rho_adv[i] + updateterm + aii * s->press_l[i]);
        for (int a = 0; a < 3; a++) {
            R force = s->dii[3 * i + a] * s->press_l[i] + s->dijpj[3 * i + a];
            s->accel[3 * i + a] = force / dt / dt;
        }
        s->pressure[i] = s->press_l1[i];
    }
    double sum = 0;
    for (int i = 0; i < s->n; i++) {
        s->press_l[i] = s->press_l1[i];
        sum += (double)s->residue[i];
    }
    return s->n > 0 ? sum / s->n : 0.0;
}

/* IntegrateIISPH (:1052-1065): vel = veleval + accel dt; pos += vel dt / simscale. */
void FN(orc_iisph_integrate)(const sphmp_params* p, ST* s) {
    const R dt = (R)p->dt;
    const R ss = (R)p->simscale;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->n; i++) {
        if (s->type[i] == SPHMP_TYPE_BOUNDARY) continue;
        if (s->mgcell[i] == UNDEF) continue;
        for (int a = 0; a < 3; a++) {
            s->vel[3 * i + a] = s->veleval[3 * i + a] + s->accel[3 * i + a] * dt;
            s->pos[3 * i + a] += s->vel[3 * i + a] * dt / ss;
        }
    }
}

int FN(orc_before_first_step)(const sphmp_params* p, ST* s) {
    FN(orc_get_particle_index)(p, s);
    FN(orc_get_grid_list)(p, s);
    if (FN(orc_rearrange_data)(p, s)) return -1;
    FN(orc_compute_boundary_volume)(p, s);
    return 0;
}

/* One step: RunSimpleSPH (fluid_system.cpp:514-539) with the legacy multiphase calls
   inserted where RunSimulateMultiCUDAFull (:375-420) places them. The fused schedule
   evaluates the force before the alpha advance and correction; the project-U
   schedule is RunSimulateMultiCUDAFull itself (ComputeForceCUDA_ProjectU in place
   of MfComputeForceCUDA). */
int FN(orc_step)(const sphmp_params* p, ST* s, int schedule, int nsteps) {
    for (int t = 0; t < nsteps; t++) {
        FN(orc_get_particle_index)(p, s);
        FN(orc_get_grid_list)(p, s);
        if (FN(orc_rearrange_data)(p, s)) return -1;
        FN(orc_compute_pressure)(p, s);
        if (schedule == SPHMP_SCHEDULE_FUSED) {
            if (p->multiphase) FN(orc_compute_drift_vel)(p, s);
            FN(orc_compute_force)(p, s);
            if (p->surface_tension) FN(orc_surface_tension)(p, s);
            if (p->multiphase) {
                FN(orc_compute_alpha_advance)(p, s);
                FN(orc_compute_correction)(p, s);
            }
        } else {
            if (p->multiphase) {
                FN(orc_compute_drift_vel)(p, s);
                FN(orc_compute_alpha_advance)(p, s);
                FN(orc_compute_correction)(p, s);
            }
            if (schedule == SPHMP_SCHEDULE_PROJECTU) FN(orc_compute_force_projectu)(p, s);
            else FN(orc_compute_force)(p, s);
            if (p->surface_tension) FN(orc_surface_tension)(p, s);
        }
        FN(orc_advance)(p, s);
    }
    return 0;
}
