// sphmp_host.cpp — host-side scene setup of the multiphase SPH step (no CUDA):
// parameter defaults, the SPH kernel constants and uniform grid exactly as the
// reference FluidSystem derives them, and the particle generators for fluid
// blocks and boundary walls. Compiled with -ffp-contract=off so the float and
// double arithmetic is identical on every host architecture.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "sphmp.h"
#include "sphmp_emit.h"

namespace {

using sphmp::uniform01;

// AddParticle (SPH_Solver/fluids/fluid_system.cpp:702-717): a fresh record.
void init_record(sphmp_display_pack* d, sphmp_calc_pack* c, int32_t n) {
    memset(d, 0, sizeof(*d));
    memset(c, 0, sizeof(*c));
    c->bornid = n;
    c->deformGrad[0] = c->deformGrad[4] = c->deformGrad[8] = 1.0f;
}

}  // namespace

extern "C" {

sphmp_status sphmp_params_default(sphmp_params* p) {
    if (!p) return SPHMP_ERR_INVALID_ARG;
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
    p->bvisc = 100.0f;  // <BoundInfo><Viscosity> of SPH_Solver/scene.xml
    p->nphase = 1;
    p->multiphase = 0;
    p->surface_tension = 0;
    p->eos = SPHMP_EOS_TAIT;
    p->eos_stiffness = 3.0f;
    // Drift-flux constants. The reference reads them from a scene file that no
    // longer exists; these values are this implementation's choice (sigma follows
    // the hint next to simData.mf_diffusion in multiphase.cu:85, pintstiff the
    // <IntStiff> of scene.xml's MultiScene 2).
    p->mf_relax = 1.0e-5f;
    p->mf_diffusion = 1.0e-3f;
    p->mf_cont = 1.0f;
    p->mf_cont1 = 1.0f;
    p->mf_cont2 = 1.0f;
    p->mf_pintstiff = 0.03f;
    // simData.omega and simData.visc_factor of the project-U force are set by no
    // remaining reference code; 1 leaves the boundary terms unscaled.
    p->mf_omega = 1.0f;
    p->mf_visc_factor = 1.0f;
    return SPHMP_OK;
}

// SetupSimpleSphCase kernel constants (SPH_Solver/fluids/fluid_system.cpp:308-313).
// pow(float, float) is the float overload; the float*double products are double.
sphmp_status sphmp_setup_constants(sphmp_params* p) {
    if (!p) return SPHMP_ERR_INVALID_ARG;
    const float h = p->smoothradius;
    if (!(h > 0.0f)) return SPHMP_ERR_INVALID_ARG;
    p->cellsize = h * 2;
    p->kpoly6 = (float)(315.0f / ((double)64.0f * 3.141592 * (double)powf(h, 9.0f)));
    p->kspiky = (float)(15 / (3.141592 * (double)powf(h, 6.0f)));
    p->kspikydiff = (float)(-45.0f / (3.141592 * (double)powf(h, 6.0f)));
    p->klaplacian = (float)(45.0f / (3.141592 * (double)powf(h, 6.0f)));
    p->kspline = 1.0f / 3.141593f / powf(h, 3.0f);
    return SPHMP_OK;
}

// FluidSystem::SetupGrid (SPH_Solver/fluids/fluid_system.cpp:119-145).
sphmp_status sphmp_setup_grid(sphmp_params* p) {
    if (!p) return SPHMP_ERR_INVALID_ARG;
    if (!(p->cellsize > 0.0f) || !(p->simscale > 0.0f)) return SPHMP_ERR_INVALID_ARG;
    const float worldcellsize = p->cellsize / p->simscale;
    long long total = 1;
    for (int a = 0; a < 3; a++) {
        p->gridmin[a] = p->volmin[a];
        p->gridmax[a] = p->volmax[a];
        p->gridsize[a] = p->gridmax[a] - p->gridmin[a];
        const float r = ceilf(p->gridsize[a] / worldcellsize);
        if (!(r >= 1.0f && r < 1.0e7f)) return SPHMP_ERR_GRID;
        p->gridres[a] = (int32_t)r;
        p->gridsize[a] = p->gridres[a] * worldcellsize;
        p->gridIdfac[a] = (float)(1.0 / (double)p->gridsize[a] * (double)p->gridres[a]);
        total *= p->gridres[a];
    }
    if (total > (1ll << 31) - 16) return SPHMP_ERR_GRID;
    p->gridtotal = (int32_t)total;
    p->searchnum = 3;
    p->neighbornum = 27;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                p->neighborid[i * 9 + j * 3 + k] =
                    (i - 1) * p->gridres[0] * p->gridres[2] + (j - 1) * p->gridres[0] + (k - 1);
    return SPHMP_OK;
}

// FluidSystem::AddFluidVolume (SPH_Solver/fluids/fluid_system.cpp:719-762): a lattice
// walked y, z, x with per-component jitter U(-jitter/2, jitter/2) (the reference
// draws rand()/RAND_MAX * 0.4 - 0.2). Records get the phase's rest density, mass
// and viscosity and zero velocity.
sphmp_status sphmp_add_fluid_volume(const sphmp_params* p, const float vmin[3], const float vmax[3], float spacing,
                                    const float offs[3], int32_t phase, float jitter, uint64_t seed,
                                    sphmp_display_pack* disp, sphmp_calc_pack* calc, int32_t cap, int32_t* count) {
    if (!p || !vmin || !vmax || !disp || !calc || !count) return SPHMP_ERR_INVALID_ARG;
    if (!(spacing > 0.0f) || phase < 0 || phase >= SPHMP_MAX_PHASES) return SPHMP_ERR_INVALID_ARG;
    const float cnts[3] = {(vmax[0] - vmin[0]) / spacing, (vmax[1] - vmin[1]) / spacing,
                           (vmax[2] - vmin[2]) / spacing};
    const float o[3] = {offs ? offs[0] : 0.0f, offs ? offs[1] : 0.0f, offs ? offs[2] : 0.0f};
    uint64_t ctr = 0;
    for (int y = 0; y < cnts[1]; y++) {
        for (int z = 0; z < cnts[2]; z++) {
            for (int x = 0; x < cnts[0]; x++) {
                const int32_t n = *count;
                if (n >= cap) return SPHMP_ERR_CAPACITY;
                float r3[3];
                for (int a = 0; a < 3; a++) r3[a] = uniform01(seed, ctr++) * jitter - jitter * 0.5f;
                sphmp_display_pack* d = disp + n;
                sphmp_calc_pack* c = calc + n;
                init_record(d, c, n);
                const float xyz[3] = {(float)x, (float)y, (float)z};
                for (int a = 0; a < 3; a++) d->pos[a] = xyz[a] * spacing + vmin[a] + r3[a] + o[a];
                d->color[0] = 0.2f; d->color[1] = 0.5f; d->color[2] = 0.8f; d->color[3] = 0.5f;
                d->type = SPHMP_TYPE_FLUID;
                c->restdens = p->densArr[phase];
                c->mass = p->massArr[phase];
                c->visc = p->viscArr[phase];
                *count = n + 1;
            }
        }
    }
    return SPHMP_OK;
}

// CalcBoundarySpacing (SPH_Solver/fluids/AddShape.cpp:265-271).
float sphmp_boundary_spacing(const sphmp_params* p) {
    if (!p) return 0.0f;
    return powf((p->bmass / p->bRestdensity), 1 / 3.0f) / p->simscale;
}

// SetupAddWall (SPH_Solver/fluids/AddShape.cpp:306-353): layers at y = min.y,
// min.y + s, ... (float accumulation, inclusive of max.y), each an x-z lattice of
// ceil(dx/s) * ceil(dz/s) boundary particles.
sphmp_status sphmp_add_wall(const sphmp_params* p, const float vmin[3], const float vmax[3],
                            sphmp_display_pack* disp, sphmp_calc_pack* calc, int32_t cap, int32_t* count) {
    if (!p || !vmin || !vmax || !disp || !calc || !count) return SPHMP_ERR_INVALID_ARG;
    const float spacing = sphmp_boundary_spacing(p);
    if (!(spacing > 0.0f)) return SPHMP_ERR_INVALID_ARG;
    const int cntx = (int)ceilf((vmax[0] - vmin[0]) / spacing);
    const int cntz = (int)ceilf((vmax[2] - vmin[2]) / spacing);
    const int cnt = cntx * cntz;
    for (float y = vmin[1]; y <= vmax[1]; y += spacing) {
        for (int xz = 0; xz < cnt; xz++) {
            const float x = vmin[0] + (xz % cntx) * spacing;
            const float z = vmin[2] + (xz / cntx) * spacing;
            const int32_t n = *count;
            if (n >= cap) return SPHMP_ERR_CAPACITY;
            sphmp_display_pack* d = disp + n;
            sphmp_calc_pack* c = calc + n;
            init_record(d, c, n);
            d->pos[0] = x; d->pos[1] = y; d->pos[2] = z;
            d->color[0] = 1.0f; d->color[1] = 1.0f; d->color[2] = 1.0f; d->color[3] = z > 0 ? 0.0f : 0.2f;
            d->type = SPHMP_TYPE_BOUNDARY;
            c->mass = p->bmass;
            c->restdens = p->bRestdensity;
            c->visc = p->bvisc;
            *count = n + 1;
        }
    }
    return SPHMP_OK;
}

// SetupAddOpenBox (SPH_Solver/fluids/AddShape.cpp:355-366): ground plus four walls.
sphmp_status sphmp_add_open_box(const sphmp_params* p, const float mn[3], const float mx[3], float t,
                                sphmp_display_pack* disp, sphmp_calc_pack* calc, int32_t cap, int32_t* count) {
    if (!mn || !mx) return SPHMP_ERR_INVALID_ARG;
    const float walls[5][2][3] = {
        {{mn[0], mn[1] - t, mn[2]}, {mx[0], mn[1], mx[2]}},                  // ground
        {{mn[0] - t, mn[1], mn[2] - t}, {mx[0] + t, mx[1], mn[2]}},          // front
        {{mn[0] - t, mn[1], mx[2]}, {mx[0] + t, mx[1], mx[2] + t}},          // back
        {{mn[0] - t, mn[1], mn[2]}, {mn[0], mx[1], mx[2]}},                  // left
        {{mx[0], mn[1], mn[2]}, {mx[0] + t, mx[1], mx[2]}},                  // right
    };
    for (int w = 0; w < 5; w++) {
        sphmp_status st = sphmp_add_wall(p, walls[w][0], walls[w][1], disp, calc, cap, count);
        if (st != SPHMP_OK) return st;
    }
    return SPHMP_OK;
}

// FluidSystem::EmitParticles / ParticleEmitter::EmitImmediate / InsertParticles
// (SPH_Solver/fluids/fluid_system.cpp:619-700): a disk of radius e->radius on a
// lattice of e->spacing in the plane normal to e->dir, each site moved by a
// uniform in-plane jitter of +-jitter/2 spacings (the reference draws +-1/2 from
// rand(); here a seeded stream), rotated so the lattice's y axis becomes dir,
// shifted to e->position; `layers` disks, layer k shifted by k spacings along
// +y as the reference's two calls are. Records as InsertParticles: velocity and
// veleval dir * vel, colour (frame/200, 0.5, 0.8, 0.5), the phase's rest
// density, mass and viscosity.
sphmp_status sphmp_emit_disk(const sphmp_params* p, const sphmp_emitter* e, int32_t layers, int32_t phase,
                             int32_t frame, float jitter, uint64_t seed, sphmp_display_pack* disp,
                             sphmp_calc_pack* calc, int32_t cap, int32_t* count) {
    if (!p || !e || !disp || !calc || !count || layers < 0) return SPHMP_ERR_INVALID_ARG;
    if (!(e->spacing > 0.0f) || !(e->radius >= 0.0f) || phase < 0 || phase >= SPHMP_MAX_PHASES)
        return SPHMP_ERR_INVALID_ARG;
    const float* dir = e->dir;
    float m[3][3];
    sphmp::emit_rotation(dir, m);
    const int res = (int)(e->radius / e->spacing);
    uint64_t ctr = 0;
    for (int layer = 0; layer < layers; layer++) {
        const float centre[3] = {e->position[0], e->position[1] + (float)layer * e->spacing, e->position[2]};
        for (int i = -res; i <= res; i++) {
            for (int j = -res; j <= res; j++) {
                const float jx = uniform01(seed, ctr++) * jitter * e->spacing - jitter * e->spacing * 0.5f;
                const float jz = uniform01(seed, ctr++) * jitter * e->spacing - jitter * e->spacing * 0.5f;
                const float t[3] = {(float)i * e->spacing + jx, 0.0f, (float)j * e->spacing + jz};
                if (t[0] * t[0] + t[1] * t[1] + t[2] * t[2] > e->radius * e->radius) continue;
                const int32_t n = *count;
                if (n >= cap) return SPHMP_ERR_CAPACITY;
                sphmp_display_pack* d = disp + n;
                sphmp_calc_pack* c = calc + n;
                init_record(d, c, n);
                for (int a = 0; a < 3; a++)
                    d->pos[a] = m[a][0] * t[0] + m[a][1] * t[1] + m[a][2] * t[2] + centre[a];
                d->color[0] = (float)frame / 200.0f;
                d->color[1] = 0.5f;
                d->color[2] = 0.8f;
                d->color[3] = 0.5f;
                d->type = SPHMP_TYPE_FLUID;
                for (int a = 0; a < 3; a++) c->vel[a] = c->veleval[a] = dir[a] * e->vel;
                c->restdens = p->densArr[phase];
                c->mass = p->massArr[phase];
                c->visc = p->viscArr[phase];
                *count = n + 1;
            }
        }
    }
    return SPHMP_OK;
}

}  // extern "C"
