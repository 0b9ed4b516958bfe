/*
 * sphmp_legacy.h — the reference's own entry-point names, exported by libsphmp.so.
 *
 * These are the `extern "C"` launch wrappers of ZP-Z/sph-multiphase
 * (SPH_Solver/fluids/fluid_system_host.cuh:44-106) plus the host transfers its
 * FluidSystem performs (SPH_Solver/fluids/fluid_system.cpp:979-999), re-implemented
 * over one process-wide default context. Like the reference they return void
 * and report failures on stderr ("CUDA ERROR: <call>: <reason>"); the status of
 * the last call is also available from sphmp_last_error(). Each wrapper
 * synchronises the device before returning, as the reference does after every
 * launch.
 *
 * `sphmp_params` starts with the reference's ParamCarrier layout (464 bytes), so
 * a ParamCarrier* can be passed wherever a `const sphmp_params*` is expected
 * below; the multiphase extension fields then take their defaults.
 */
#ifndef SPHMP_LEGACY_H
#define SPHMP_LEGACY_H

#include "sphmp.h"

#ifdef __cplusplus
extern "C" {
#endif

/* cudaInit (fluid_system_host.cu:30-48): prints the device properties. */
void cudaInit(int argc, char** argv);
/* cudaExit (fluid_system_host.cu:24-27): no-op, as in the reference. */
void cudaExit(int argc, char** argv);
/* FluidClearCUDA (fluid_system_host.cu:79-94): frees the default context. */
void FluidClearCUDA(void);
/* FluidSetupCUDA(ParamCarrier&) (fluid_system_host.cu:103-144): allocates the default
   context for params->maxNum particles; only the first 464 bytes (the ParamCarrier
   prefix) are read. */
void FluidSetupCUDA(const sphmp_params* params);
/* GetParticleIndexCUDA (fluid_system_host.cu:147-159) */
void GetParticleIndexCUDA(void);
/* GetGridListCUDA (fluid_system_host.cu:161-185) */
void GetGridListCUDA(void);
/* RearrageDataCUDA (fluid_system_host.cu:187-210; the reference's spelling) */
void RearrageDataCUDA(void);
/* The legacy names of the three sort steps, as the legacy multiphase step calls
   them (fluid_system.cpp:382-384 and 427-429, InitialSortCUDA(0x0, 0x0, 0x0),
   SortGridCUDA(0x0), CountingSortFullCUDA_(0x0)): the same as GetParticleIndexCUDA,
   GetGridListCUDA and RearrageDataCUDA. The pointer arguments (host mirrors of the
   older code) are ignored. */
void InitialSortCUDA(uint32_t* gcell, uint32_t* ccell, int* gcnt);
void SortGridCUDA(int* goff);
void CountingSortFullCUDA_(uint32_t* ggrid);
/* MfComputePressureCUDA (fluid_system_host.cu:337-348) */
void MfComputePressureCUDA(void);
/* MfComputeDriftVelCUDA (decl fluid_system_host.cuh:62) */
void MfComputeDriftVelCUDA(void);
/* MfComputeAlphaAdvanceCUDA (decl fluid_system_host.cuh:63) */
void MfComputeAlphaAdvanceCUDA(void);
/* MfComputeCorrectionCUDA (decl fluid_system_host.cuh:64) */
void MfComputeCorrectionCUDA(void);
/* MfComputeForceCUDA (fluid_system_host.cu:421-438) */
void MfComputeForceCUDA(void);
/* ComputeForceCUDA_ProjectU (fluid_system_host.cu:396-419; decl fluid_system_host.cuh:77).
   Runs the ComputeForce_projectu kernel, whose launch the reference comments out. */
void ComputeForceCUDA_ProjectU(void);
/* MfAdvanceCUDA (fluid_system_host.cu:385-394) */
void MfAdvanceCUDA(void);
/* ComputeBoundaryDensity (fluid_system_host.cu:510-513) */
void ComputeBoundaryDensity(void);
/* The IISPH step of RunIISPH (fluid_system.cpp:567-588):
   ComputeDensityIISPH_CUDA (fluid_system_host.cu:505-508), PredictAdvection
   (:515-524), PressureSolve (:526-550) and Integration (:552-556). The
   reference's PressureSolve loop never ends (its break is commented out); this
   one stops once the mean |density residue| over in-grid fluid particles is at
   most 0.1 kg/m^3 after at least 2 iterations, or after 100 iterations (the
   sphmp_iisph_pressure_solve entry point takes its own limits), and prints no
   per-iteration line. */
void ComputeDensityIISPH_CUDA(void);
void PredictAdvection(void);
void PressureSolve(void);
void Integration(void);
/* computeNumBlocks (fluid_system_host.cu:70-76): launch geometry helper. */
void computeNumBlocks(int numPnts, int maxThreads, int* numBlocks, int* numThreads);

/* FluidSystem::TransferToCUDA (fluid_system.cpp:979-982): upload n records. */
void TransferToCUDA(const sphmp_display_pack* disp, const sphmp_calc_pack* calc, int n);
/* FluidSystem::TransferFromCUDA (fluid_system.cpp:984-987): download n display records. */
void TransferFromCUDA(sphmp_display_pack* disp, int n);
/* FluidSystem::EmitUpdateCUDA (fluid_system.cpp:990-999): append records [startnum, endnum). */
void EmitUpdateCUDA(int startnum, int endnum, const sphmp_display_pack* disp, const sphmp_calc_pack* calc);

/* The default context behind these wrappers (NULL before FluidSetupCUDA). */
sphmp_ctx* sphmp_legacy_context(void);

#ifdef __cplusplus
}

/* CarryParam(ParamCarrier&) has C++ linkage in the reference
   (SPH_Solver/fluids/fluid_system_kern.cuh:71); the library exports the same
   mangled symbol. A caller without the ParamCarrier type may use
   sphmp_set_params(sphmp_legacy_context(), p) instead. */
struct ParamCarrier;
void CarryParam(ParamCarrier& hostCarrier);
#endif

#endif /* SPHMP_LEGACY_H */
