// legacy_host.cpp — test program: a host application in the shape of the
// reference's FluidSystem (SPH_Solver/fluids/fluid_system.cpp) that includes this
// library's headers, links libsphmp.so and drives it only through the reference's
// entry-point names: FluidSetupCUDA + CarryParam (:149-152), TransferToCUDA,
// BeforeFirstStep (:62-70), then RunSimpleSPH (:514-539) `steps` times, each
// ending with TransferFromCUDA. The extension fields of sphmp_params (phases,
// EOS), which a ParamCarrier does not hold, are set once on the legacy context.
//
// usage: legacy_host <params.bin> <display.bin> <calc.bin> <n> <steps> <out_display.bin>
// exit status: 0 ok, 2 usage / file error, 3 no legacy context (FluidSetupCUDA
// failed, e.g. no CUDA device), 4 an error reported after the steps.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sphmp_legacy.h"

struct ParamCarrier;  // the reference's parameter type, passed by reference (fluid_system_kern.cuh:71)
void CarryParam(ParamCarrier& hostCarrier);

static bool read_exact(const char* path, void* dst, size_t bytes) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    const bool ok = fread(dst, 1, bytes, f) == bytes;
    fclose(f);
    return ok;
}

int main(int argc, char** argv) {
    if (argc != 7) {
        fprintf(stderr, "usage: %s params.bin display.bin calc.bin n steps out_display.bin\n", argv[0]);
        return 2;
    }
    const int n = atoi(argv[4]), steps = atoi(argv[5]);
    if (n <= 0 || steps < 0) return 2;
    sphmp_params p;
    std::vector<sphmp_display_pack> disp(n);
    std::vector<sphmp_calc_pack> calc(n);
    if (!read_exact(argv[1], &p, sizeof(p)) || !read_exact(argv[2], disp.data(), sizeof(disp[0]) * n) ||
        !read_exact(argv[3], calc.data(), sizeof(calc[0]) * n))
        return 2;

    FluidSetupCUDA(&p);
    sphmp_ctx* ctx = sphmp_legacy_context();
    if (!ctx) {
        fprintf(stderr, "no legacy context: %s\n", sphmp_last_error());
        return 3;
    }
    CarryParam(*reinterpret_cast<ParamCarrier*>(&p));
    if (sphmp_set_params(ctx, &p) != SPHMP_OK) return 4;
    TransferToCUDA(disp.data(), calc.data(), n);

    GetParticleIndexCUDA();  // BeforeFirstStep
    GetGridListCUDA();
    RearrageDataCUDA();
    ComputeBoundaryDensity();
    for (int s = 0; s < steps; s++) {  // RunSimpleSPH
        GetParticleIndexCUDA();
        GetGridListCUDA();
        RearrageDataCUDA();
        MfComputePressureCUDA();
        MfComputeForceCUDA();
        MfAdvanceCUDA();
        TransferFromCUDA(disp.data(), n);
    }
    uint32_t bits = 0;
    const sphmp_status st = sphmp_sync(ctx);
    sphmp_device_errors(ctx, &bits);
    FluidClearCUDA();
    if (st != SPHMP_OK || bits != 0) {
        fprintf(stderr, "status %d, device error bits %#x: %s\n", (int)st, bits, sphmp_last_error());
        return 4;
    }
    FILE* f = fopen(argv[6], "wb");
    if (!f) return 2;
    const bool ok = fwrite(disp.data(), sizeof(disp[0]), n, f) == (size_t)n;
    fclose(f);
    return ok ? 0 : 2;
}
