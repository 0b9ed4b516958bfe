"""The drop-in boundary itself: the reference's own call sequences through its
extern "C" entry points, bound with ctypes the way a host application linking
libsphmp.so would call them, against the oracle running the same sequence.

* FluidSystem::BeforeFirstStep + RunSimpleSPH (SPH_Solver/fluids/fluid_system.cpp:
  62-70, 514-539): sort, pressure, force, advance, TransferFromCUDA, three times.
* The legacy multiphase step RunSimulateMultiCUDAFull (:375-420), with its sort
  names InitialSortCUDA / SortGridCUDA / CountingSortFullCUDA_, the drift /
  alpha / correction calls and ComputeForceCUDA_ProjectU.

Both scenes hold liquid phases only (Tait EOS next to a 1.2 kg/m^3 gas phase
scatters a small block within a step). Display records come back in slot
order, as the reference's; positions must agree with the oracle within
RTOL = 1e-5 (max |gpu - oracle| / max |oracle| over in-grid fluid slots), like
the other parity tests.
"""
import ctypes as C

import numpy as np
import pytest

import sphmp
import subprocess

from helpers import build_c_host, field_err, in_grid_fluid, oracle_state, write_c_host_inputs
from oracle import oracle as O
from sphmp import abi, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-5
VOID_CALLS = ("GetParticleIndexCUDA", "GetGridListCUDA", "RearrageDataCUDA", "MfComputePressureCUDA",
              "MfComputeDriftVelCUDA", "MfComputeAlphaAdvanceCUDA", "MfComputeCorrectionCUDA",
              "MfComputeForceCUDA", "ComputeForceCUDA_ProjectU", "MfAdvanceCUDA", "ComputeBoundaryDensity",
              "FluidClearCUDA")


@pytest.fixture
def legacy(built):
    L = C.CDLL(sphmp.load()._name)  # a separate handle: argtypes of its own, same library
    for name in VOID_CALLS:
        getattr(L, name).argtypes = []
        getattr(L, name).restype = None
    L.FluidSetupCUDA.argtypes = [C.c_void_p]
    L.TransferToCUDA.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.TransferFromCUDA.argtypes = [C.c_void_p, C.c_int]
    L.InitialSortCUDA.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.SortGridCUDA.argtypes = [C.c_void_p]
    L.CountingSortFullCUDA_.argtypes = [C.c_void_p]
    for f in (L.InitialSortCUDA, L.SortGridCUDA, L.CountingSortFullCUDA_, L.FluidSetupCUDA, L.TransferToCUDA,
              L.TransferFromCUDA):
        f.restype = None
    L.sphmp_legacy_context.restype = C.c_void_p
    L.sphmp_set_params.argtypes = [C.c_void_p, C.POINTER(abi.Params)]
    yield L
    L.FluidClearCUDA()


def _setup(L, sc):
    """FluidSetupCUDA with the ParamCarrier, the extension fields (not part of the
    ParamCarrier) through sphmp_set_params on the legacy context, then TransferToCUDA
    of the reference records."""
    p = sc.params
    L.FluidSetupCUDA(C.cast(C.pointer(p), C.c_void_p))
    assert L.sphmp_legacy_context()
    assert L.sphmp_set_params(L.sphmp_legacy_context(), C.byref(p)) == abi.OK
    calc = sc.calc[:sc.n].copy()
    bnd = sc.disp["type"][:sc.n] == abi.TYPE_BOUNDARY
    calc["accel"][bnd] = 0  # as the oracle state starts
    calc["pressure"][bnd] = 0
    disp = np.ascontiguousarray(sc.disp[:sc.n])
    L.TransferToCUDA(disp.ctypes.data, calc.ctypes.data, sc.n)
    return p


def _check(L, sc, s):
    out = sphmp.record_arrays(sc.n)[0]
    L.TransferFromCUDA(out.ctypes.data, sc.n)
    f = in_grid_fluid(s)
    assert f.sum() > 500
    assert field_err(out["pos"][f], s.pos[f]) < RTOL


def test_run_simple_sph_sequence(legacy):
    L = legacy
    sc = scenes.small_block(seed=71, n=(12, 10, 9), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.3, multiphase=0,
                            dens=(1000.0, 800.0, 900.0))
    p = _setup(L, sc)
    s = oracle_state(sc)
    L.GetParticleIndexCUDA()
    L.GetGridListCUDA()
    L.RearrageDataCUDA()
    L.ComputeBoundaryDensity()
    O.before_first_step(p, s)
    for _ in range(3):
        for name in ("GetParticleIndexCUDA", "GetGridListCUDA", "RearrageDataCUDA", "MfComputePressureCUDA",
                     "MfComputeForceCUDA", "MfAdvanceCUDA"):
            getattr(L, name)()
        O.step(p, s, abi.SCHEDULE_REFERENCE, 1)
        _check(L, sc, s)


def test_legacy_multiphase_sequence_with_projectu(legacy):
    L = legacy
    sc = scenes.small_block(seed=72, n=(12, 10, 9), nphase=3, eos=abi.EOS_TAIT, velocity_scale=0.3,
                            dens=(1000.0, 800.0, 900.0), phase_frac=0.5)
    p = _setup(L, sc)
    s = oracle_state(sc)
    L.GetParticleIndexCUDA()
    L.GetGridListCUDA()
    L.RearrageDataCUDA()
    L.ComputeBoundaryDensity()
    O.before_first_step(p, s)
    for _ in range(3):
        L.InitialSortCUDA(None, None, None)
        L.SortGridCUDA(None)
        L.CountingSortFullCUDA_(None)
        for name in ("MfComputePressureCUDA", "MfComputeDriftVelCUDA", "MfComputeAlphaAdvanceCUDA",
                     "MfComputeCorrectionCUDA", "ComputeForceCUDA_ProjectU", "MfAdvanceCUDA"):
            getattr(L, name)()
        O.step(p, s, abi.SCHEDULE_PROJECTU, 1)
        _check(L, sc, s)


def test_cpp_host_program(built, tmp_path):
    """The same BeforeFirstStep + RunSimpleSPH sequence from a compiled C++ host
    (tests/c_host/legacy_host.cpp, linked with -lsphmp), three steps."""
    exe = build_c_host(tmp_path)
    sc = scenes.small_block(seed=73, n=(12, 10, 9), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.3, multiphase=0,
                            dens=(1000.0, 800.0, 900.0))
    args = write_c_host_inputs(tmp_path, sc)
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, *args, str(sc.n), "3", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    disp = np.fromfile(out, dtype=abi.display_dtype())
    p = sc.params
    s = oracle_state(sc)
    O.before_first_step(p, s)
    O.step(p, s, abi.SCHEDULE_REFERENCE, 3)
    f = in_grid_fluid(s)
    assert f.sum() > 500
    assert field_err(disp["pos"][f], s.pos[f]) < RTOL
    assert np.array_equal(disp["type"], s.type)

