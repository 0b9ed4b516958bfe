// sphmp_emit.h — the jitter stream and the disk-emitter geometry shared by the
// host particle generators (sphmp_host.cpp) and the device-side emitter
// (sphmp_kernels.cu), so that both produce the same records bit for bit.
// Host code that includes it is compiled with -ffp-contract=off.
#pragma once

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define SPHMP_HD __host__ __device__ __forceinline__
#else
#define SPHMP_HD inline
#endif

namespace sphmp {

// splitmix64: seeded, platform-independent stream for the lattice jitter.
SPHMP_HD uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// uniform float in [0, 1) from counter `i` of stream `seed` (24 random bits,
// so the conversion and the scaling are exact)
SPHMP_HD float uniform01(uint64_t seed, uint64_t i) {
    return (float)(splitmix64(seed * 0x100000001B3ull + i) >> 40) * (1.0f / 16777216.0f);
}

// ParticleEmitter::EmitImmediate's rotation (SPH_Solver/fluids/fluid_system.cpp:
// 644-656): columns (newx, dir, newz) with newx = dir x (0, 1, 0) normalised and
// newz = newx x dir; the identity when dir is (anti)parallel to y.
inline void emit_rotation(const float dir[3], float m[3][3]) {
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) m[a][b] = a == b ? 1.f : 0.f;
    float nx[3] = {dir[1] * 0.f - dir[2] * 1.f, dir[2] * 0.f - dir[0] * 0.f, dir[0] * 1.f - dir[1] * 0.f};
    const float nn = nx[0] * nx[0] + nx[1] * nx[1] + nx[2] * nx[2];
    if (nn > 0.001f) {
        const float inv = sqrtf(nn);
        for (int a = 0; a < 3; a++) nx[a] = nx[a] / inv;
        const float nz[3] = {nx[1] * dir[2] - nx[2] * dir[1], nx[2] * dir[0] - nx[0] * dir[2],
                             nx[0] * dir[1] - nx[1] * dir[0]};
        for (int a = 0; a < 3; a++) {
            m[a][0] = nx[a];
            m[a][1] = dir[a];
            m[a][2] = nz[a];
        }
    }
}

}  // namespace sphmp
