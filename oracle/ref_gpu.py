"""Device-ref: the reference's own GPU kernels, run on the GPU. TEST AND BASELINE
INFRASTRUCTURE ONLY.

oracle/ref/build_ref_dev.sh compiles the reference's SPH_Solver/fluids/
fluid_system_kern.cu, unmodified, into oracle/_ref/sph_ref_kern.cubin (sm_103a).
This module loads it with the CUDA driver API (ctypes on libcuda) into the
primary context that torch uses, and replays the reference's host launch
sequence (SPH_Solver/fluids/fluid_system_host.cu) on its AoS record buffers:

* GetParticleIndexCUDA (:147-159): clear mgridcnt, mgridoff, mgcell; InitialSort.
* GetGridListCUDA (:161-185): thrust::sort_by_key(mgcell, midsort) — here the
  same stable key sort done by torch.sort(stable=True) on the device —, then
  CalcFirstCnt and GetCnt.
* RearrageDataCUDA (:187-210): both record arrays into msortbuf, RearrangeData.
* ComputeBoundaryDensity, MfComputePressureCUDA, MfComputeForceCUDA,
  MfAdvanceCUDA: ComputeBoundaryVolume, ComputeDensityPressure, ComputeForce,
  AdvanceParticles.

Every launch uses the reference's geometry (computeNumBlocks(pnum, 384),
fluid_system_host.cu:70-76, FluidSetupCUDA :103-144). With `sync_each` the host
waits after every call, as the reference's wrappers do (cudaThreadSynchronize).

Only tests/ and bench.py use this module, to check the device-ref against the
oracle and to time it beside the library. The library never does.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "sph_ref_kern.cubin")
THREADS = 384  # the reference's numThreads (FluidSetupCUDA, computeNumBlocks(pnum, 384, ...))

# `__global__ void Name(bufList, int)` under the Itanium C++ ABI
KERNELS = {name: f"_Z{len(name)}{name}7bufListi" for name in (
    "InitialSort", "CalcFirstCnt", "GetCnt", "RearrangeData", "ComputeBoundaryVolume",
    "ComputeDensityPressure", "ComputeForce", "AdvanceParticles")}

# bufList (SPH_Solver/fluids/fluid_system_kern.cuh:33-67): every member is a pointer
_BUFLIST = ["displayBuffer", "calcBuffer", "densityResidue", "press_l", "press_l1", "rho_adv", "stress", "aii",
            "dii", "dijpj", "invDp", "msortbuf", "mgridcnt", "mgridoff", "mgcell", "mgndx", "MFidTable", "midsort",
            "mpmPos", "mpmMass", "mpmVel", "u", "v", "w", "mpmForce", "mpmGid"]


class BufList(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in _BUFLIST]


def available():
    return os.path.exists(CUBIN)


def build(verbose=False):
    import subprocess
    r = subprocess.run(["sh", os.path.join(HERE, "ref", "build_ref_dev.sh")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference device build failed:\n" + r.stderr[-4000:])
    if verbose:
        print(r.stdout.strip())
    return CUBIN


class _Driver:
    def __init__(self):
        cu = C.CDLL("libcuda.so.1")
        cu.cuCtxGetCurrent.argtypes = [C.POINTER(C.c_void_p)]
        cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        cu.cuModuleUnload.argtypes = [C.c_void_p]
        cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        cu.cuModuleGetGlobal_v2.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_size_t), C.c_void_p, C.c_char_p]
        cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        cu.cuGetErrorString.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        self.cu = cu

    def check(self, status, what):
        if status != 0:
            s = C.c_char_p()
            self.cu.cuGetErrorString(status, C.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {status} ({(s.value or b'?').decode()})")


class RefGPU:
    """The reference's kernels on one scene: `disp`, `calc` are numpy record arrays
    with the reference's displayPack / calculationPack layouts, `params` a sphmp
    Params whose first 464 bytes are the ParamCarrier."""

    def __init__(self, params, disp, calc, stream=None):
        import torch
        if not available():
            raise RuntimeError(f"{CUBIN} is missing: build it with oracle/ref/build_ref_dev.sh")
        self.torch = torch
        self.dev = torch.device("cuda", torch.cuda.current_device())
        torch.zeros(1, device=self.dev)  # the primary context is current from here on
        self.drv = _Driver()
        cu = self.drv.cu
        ctx = C.c_void_p()
        self.drv.check(cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        self.mod = C.c_void_p()
        self.drv.check(cu.cuModuleLoad(C.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        for name, sym in KERNELS.items():
            f = C.c_void_p()
            self.drv.check(cu.cuModuleGetFunction(C.byref(f), self.mod, sym.encode()), f"cuModuleGetFunction {name}")
            self.fn[name] = f
        dptr, size = C.c_uint64(), C.c_size_t()
        self.drv.check(cu.cuModuleGetGlobal_v2(C.byref(dptr), C.byref(size), self.mod, b"paramCarrier"),
                       "cuModuleGetGlobal paramCarrier")
        if size.value != 464:
            raise RuntimeError(f"paramCarrier is {size.value} bytes, not the ParamCarrier's 464")
        carrier = (C.c_char * 464).from_buffer_copy(bytes(params)[:464])
        self.drv.check(cu.cuMemcpyHtoD_v2(dptr.value, carrier, 464), "cuMemcpyHtoD paramCarrier")
        self.stream = stream if stream is not None else torch.cuda.Stream()
        n = len(disp)
        G = int(params.gridtotal)
        self.n = n
        u8 = dict(dtype=torch.uint8, device=self.dev)
        i32 = dict(dtype=torch.int32, device=self.dev)
        with torch.cuda.stream(self.stream):
            self.disp = torch.from_numpy(np.ascontiguousarray(disp).view(np.uint8).copy()).to(self.dev)
            self.calc = torch.from_numpy(np.ascontiguousarray(calc).view(np.uint8).copy()).to(self.dev)
            self.msort = torch.empty(n * (disp.dtype.itemsize + calc.dtype.itemsize), **u8)
            self.mgridcnt = torch.zeros(G, **i32)
            self.mgridoff = torch.zeros(G, **i32)
            self.mgcell = torch.zeros(n, **i32)
            self.mgndx = torch.zeros(n, **i32)
            self.midsort = torch.zeros(n, **i32)
            self.mfid = torch.zeros(n, **i32)
        self.stream.synchronize()
        self.buf = BufList(displayBuffer=self.disp.data_ptr(), calcBuffer=self.calc.data_ptr(),
                           msortbuf=self.msort.data_ptr(), mgridcnt=self.mgridcnt.data_ptr(),
                           mgridoff=self.mgridoff.data_ptr(), mgcell=self.mgcell.data_ptr(),
                           mgndx=self.mgndx.data_ptr(), MFidTable=self.mfid.data_ptr(),
                           midsort=self.midsort.data_ptr())
        self._pnum = C.c_int(n)
        self._args = (C.c_void_p * 2)(C.cast(C.pointer(self.buf), C.c_void_p), C.cast(C.pointer(self._pnum), C.c_void_p))
        self.sync_each = True

    def close(self):
        if self.mod:
            self.torch.cuda.synchronize()
            self.drv.cu.cuModuleUnload(self.mod)
            self.mod = None

    # ---- the reference's calls ----

    def _launch(self, name):
        blocks = (self.n + THREADS - 1) // THREADS  # computeNumBlocks(pnum, 384)
        self.drv.check(self.drv.cu.cuLaunchKernel(self.fn[name], max(blocks, 1), 1, 1, THREADS, 1, 1, 0,
                                                  C.c_void_p(self.stream.cuda_stream), self._args, None),
                       f"cuLaunchKernel {name}")

    def _done(self):
        if self.sync_each:
            self.stream.synchronize()

    def get_particle_index(self):
        with self.torch.cuda.stream(self.stream):
            self.mgridcnt.zero_()
            self.mgridoff.zero_()
            self.mgcell.zero_()
        self._launch("InitialSort")
        self._done()

    def get_grid_list(self):
        torch = self.torch
        with torch.cuda.stream(self.stream):
            keys = self.mgcell.to(torch.int64) & 0xFFFFFFFF
            sk, perm = torch.sort(keys, stable=True)
            vals = self.midsort[perm]
            self.mgcell.copy_(sk.to(torch.int32))
            self.midsort.copy_(vals)
        self._launch("CalcFirstCnt")
        self._launch("GetCnt")
        self._done()

    def rearrange_data(self):
        nd = self.disp.numel()
        with self.torch.cuda.stream(self.stream):
            self.msort[:nd].copy_(self.disp)
            self.msort[nd:].copy_(self.calc)
        self._launch("RearrangeData")
        self._done()

    def compute_boundary_density(self):
        self._launch("ComputeBoundaryVolume")
        self._done()

    def compute_pressure(self):
        self._launch("ComputeDensityPressure")
        self._done()

    def compute_force(self):
        self._launch("ComputeForce")
        self._done()

    def advance(self):
        self._launch("AdvanceParticles")
        self._done()

    def before_first_step(self):
        """FluidSystem::BeforeFirstStep (SPH_Solver/fluids/fluid_system.cpp:62-70)."""
        self.get_particle_index()
        self.get_grid_list()
        self.rearrange_data()
        self.compute_boundary_density()

    def step(self, nsteps=1):
        """FluidSystem::RunSimpleSPH (SPH_Solver/fluids/fluid_system.cpp:514-539) without the transfer."""
        for _ in range(nsteps):
            self.get_particle_index()
            self.get_grid_list()
            self.rearrange_data()
            self.compute_pressure()
            self.compute_force()
            self.advance()

    # ---- results ----

    def records(self, disp_dtype, calc_dtype):
        self.stream.synchronize()
        d = self.disp.cpu().numpy().view(disp_dtype)
        c = self.calc.cpu().numpy().view(calc_dtype)
        return d, c

    def sort_arrays(self):
        self.stream.synchronize()
        return {"mgcell": self.mgcell.cpu().numpy().view(np.uint32), "midsort": self.midsort.cpu().numpy().view(np.uint32),
                "mgndx": self.mgndx.cpu().numpy().view(np.uint32), "mgridoff": self.mgridoff.cpu().numpy(),
                "mgridcnt": self.mgridcnt.cpu().numpy()}
