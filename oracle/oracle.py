"""Python access to the CPU oracle. TEST INFRASTRUCTURE ONLY.

Builds and loads:
  * liboracle.so  — the C restatement in sph_oracle.c, as FP32 (reference
    arithmetic, suffix _f32) and FP64 (suffix _f64) entry points;
  * libsphref.so  — the reference's own kernel sources compiled as host C++
    (oracle/ref/build_ref.sh), when they were built on this machine.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg and its
reference arm (--impl reference) import this module. The CUDA product never does.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "liboracle.so")
REF_SO = os.path.join(REF_DIR, "libsphref.so")

sys.path.insert(0, os.path.join(REPO, "sph-multiphase_gb300"))
from sphmp import abi  # noqa: E402  (ctypes struct definitions only)

UNDEF = abi.GRID_UNDEF
SOURCES = [os.path.join(HERE, "sph_oracle.c"), os.path.join(HERE, "sph_oracle.h"),
           os.path.join(REPO, "include", "sphmp.h")]


def build(force=False, verbose=False):
    """Compile sph_oracle.c twice (FP32 and FP64) into oracle/_build/liboracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(ORACLE_SO):
        so_t = os.path.getmtime(ORACLE_SO)
        if all(os.path.getmtime(s) <= so_t for s in SOURCES):
            return ORACLE_SO
    cc = os.environ.get("CC", "gcc")
    flags = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c11", "-Wall",
             "-Wno-unknown-pragmas"]
    src = os.path.join(HERE, "sph_oracle.c")
    o32 = os.path.join(BUILD_DIR, "sph_oracle_f32.o")
    o64 = os.path.join(BUILD_DIR, "sph_oracle_f64.o")
    procs = [subprocess.Popen([cc, *flags, "-c", src, "-o", o32]),
             subprocess.Popen([cc, *flags, "-DORC_F64", "-c", src, "-o", o64])]
    for pr in procs:
        if pr.wait() != 0:
            raise RuntimeError("oracle compile failed")
    tmp = ORACLE_SO + ".tmp"
    subprocess.check_call([cc, "-shared", "-fopenmp", "-o", tmp, o32, o64, "-lm"])
    os.replace(tmp, ORACLE_SO)
    if verbose:
        print("built", ORACLE_SO)
    return ORACLE_SO


def build_ref(verbose=False):
    """Build oracle/_ref/libsphref.so from the reference sources (needs the checkout)."""
    script = os.path.join(HERE, "ref", "build_ref.sh")
    r = subprocess.run(["sh", script], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference host build failed:\n" + r.stderr[-4000:])
    if verbose:
        print(r.stdout.strip())
    return REF_SO


def _state_struct(R):
    P = C.POINTER
    return type("orc_state_" + R.__name__, (C.Structure,), {"_fields_": [
        ("n", C.c_int32), ("pos", P(R)), ("type", P(C.c_int32)), ("color", P(C.c_float)),
        ("vel", P(R)), ("veleval", P(R)), ("pressure", P(R)), ("dens", P(R)), ("restdens", P(R)),
        ("mass", P(R)), ("visc", P(R)), ("bornid", P(C.c_int32)), ("accel", P(R)),
        ("alpha", P(R)), ("alpha_pre", P(R)), ("drift", P(R)), ("aprev", P(R)), ("pmod", P(R)),
        ("mgcell", P(C.c_uint32)), ("midsort", P(C.c_uint32)), ("mgndx", P(C.c_uint32)),
        ("mgridoff", P(C.c_int32)), ("mgridcnt", P(C.c_int32)), ("velxcor", P(R)),
        ("dii", P(R)), ("aii", P(R)), ("rho_adv", P(R)), ("press_l", P(R)), ("press_l1", P(R)),
        ("dijpj", P(R)), ("residue", P(R)),
    ]})


StateF32 = _state_struct(C.c_float)
StateF64 = _state_struct(C.c_double)

# per-particle real-valued fields and their trailing shapes
REAL_FIELDS = {"pos": (3,), "vel": (3,), "veleval": (3,), "pressure": (), "dens": (), "restdens": (),
               "mass": (), "visc": (), "accel": (3,), "alpha": (3,), "alpha_pre": (3,), "drift": (3, 3),
               "aprev": (3,), "pmod": (), "velxcor": (3,), "dii": (3,), "aii": (), "rho_adv": (),
               "press_l": (), "press_l1": (), "dijpj": (3,), "residue": ()}
INT_FIELDS = {"type": np.int32, "bornid": np.int32, "mgcell": np.uint32, "midsort": np.uint32,
              "mgndx": np.uint32}
GRID_FIELDS = ("mgridoff", "mgridcnt")


class State:
    """Numpy-backed particle state in the reference's per-slot layout."""

    def __init__(self, n, gridtotal, dtype=np.float32):
        self.n = int(n)
        self.gridtotal = int(gridtotal)
        self.dtype = np.dtype(dtype)
        for k, shp in REAL_FIELDS.items():
            setattr(self, k, np.zeros((self.n,) + shp, self.dtype))
        for k, t in INT_FIELDS.items():
            setattr(self, k, np.zeros(self.n, t))
        self.color = np.zeros((self.n, 4), np.float32)
        for k in GRID_FIELDS:
            setattr(self, k, np.zeros(self.gridtotal, np.int32))

    def fields(self):
        return list(REAL_FIELDS) + list(INT_FIELDS) + ["color"] + list(GRID_FIELDS)

    def copy(self, dtype=None):
        out = State(self.n, self.gridtotal, dtype or self.dtype)
        for k in self.fields():
            v = getattr(self, k)
            setattr(out, k, v.astype(out.dtype) if k in REAL_FIELDS else v.copy())
        return out

    def struct(self):
        S = StateF64 if self.dtype == np.float64 else StateF32
        for k in self.fields():
            v = getattr(self, k)
            if not v.flags.c_contiguous:
                setattr(self, k, np.ascontiguousarray(v))
        s = S()
        s.n = self.n
        for name, typ in S._fields_[1:]:
            arr = getattr(self, name)
            setattr(s, name, arr.ctypes.data_as(typ))
        self._keep = s
        return s


_ORACLE = None
_REF = None

_FUNCS = ["orc_get_particle_index", "orc_get_grid_list", "orc_rearrange_data",
          "orc_compute_boundary_volume", "orc_compute_pressure", "orc_compute_force",
          "orc_surface_tension", "orc_advance", "orc_compute_drift_vel", "orc_compute_alpha_advance",
          "orc_compute_correction", "orc_compute_force_projectu", "orc_before_first_step",
          "orc_iisph_density", "orc_iisph_predict", "orc_iisph_iteration", "orc_iisph_integrate"]


def lib():
    global _ORACLE
    if _ORACLE is None:
        build()
        L = C.CDLL(ORACLE_SO)
        for sfx, S in (("_f32", StateF32), ("_f64", StateF64)):
            for f in _FUNCS:
                fn = getattr(L, f + sfx)
                fn.argtypes = [C.POINTER(abi.Params), C.POINTER(S)]
            fn = getattr(L, "orc_step" + sfx)
            fn.argtypes = [C.POINTER(abi.Params), C.POINTER(S), C.c_int, C.c_int]
            getattr(L, "orc_iisph_iteration" + sfx).restype = C.c_double
        L.orc_params_default.argtypes = [C.POINTER(abi.Params)]
        L.orc_params_default.restype = None
        f3 = C.POINTER(C.c_float)
        L.orc_add_fluid_volume.argtypes = [C.POINTER(abi.Params), f3, f3, C.c_float, f3, C.c_int32, C.c_float,
                                           C.c_uint64, C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
        L.orc_add_open_box.argtypes = [C.POINTER(abi.Params), f3, f3, C.c_float, C.c_void_p, C.c_void_p, C.c_int32,
                                       C.POINTER(C.c_int32)]
        L.orc_setup_constants.argtypes = [C.POINTER(abi.Params)]
        L.orc_setup_grid.argtypes = [C.POINTER(abi.Params)]
        L.orc_set_num_threads.argtypes = [C.c_int]
        L.orc_get_num_threads.restype = C.c_int
        _ORACLE = L
    return _ORACLE


def ref_available():
    return os.path.exists(REF_SO)


def ref_lib():
    global _REF
    if _REF is None:
        L = C.CDLL(REF_SO)
        for f in ["ref_get_particle_index", "ref_get_grid_list", "ref_rearrange_data",
                  "ref_compute_boundary_volume", "ref_compute_pressure", "ref_compute_force",
                  "ref_surface_tension", "ref_advance", "ref_compute_drift_vel",
                  "ref_compute_alpha_advance", "ref_compute_correction", "ref_compute_force_projectu",
                  "ref_iisph_density", "ref_iisph_predict", "ref_iisph_iteration", "ref_iisph_integrate"]:
            getattr(L, f).argtypes = [C.POINTER(abi.Params), C.POINTER(StateF32)]
        L.ref_iisph_iteration.restype = C.c_double
        L.ref_set_num_threads.argtypes = [C.c_int]
        _REF = L
    return _REF


def call(name, params, state, *extra):
    """Run oracle function `name` (without suffix) on `state` in place."""
    L = lib()
    sfx = "_f64" if state.dtype == np.float64 else "_f32"
    return getattr(L, name + sfx)(C.byref(params), C.byref(state.struct()), *extra)


def call_ref(name, params, state):
    """Run the reference's own kernel `name` (ref_* entry point) on an FP32 state in place."""
    assert state.dtype == np.float32
    return getattr(ref_lib(), name)(C.byref(params), C.byref(state.struct()))


def setup_constants(params):
    lib().orc_setup_constants(C.byref(params))


def setup_grid(params):
    lib().orc_setup_grid(C.byref(params))


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


class Generators:
    """The scene-generation functions of sphmp.scenes (parameter defaults, kernel
    constants, grid, fluid lattice, open box) from the oracle's restatement, so that a
    CPU-only run (the benchmark's reference arm) builds its scene without loading the
    CUDA library. tests/test_host.py checks the records equal the library's."""

    @staticmethod
    def params_default():
        p = abi.Params()
        lib().orc_params_default(C.byref(p))
        return p

    @staticmethod
    def setup_constants(p):
        if lib().orc_setup_constants(C.byref(p)) != 0:
            raise ValueError("smoothing radius must be positive")
        return p

    @staticmethod
    def setup_grid(p):
        lib().orc_setup_grid(C.byref(p))
        return p

    @staticmethod
    def record_arrays(cap):
        return np.zeros(cap, abi.display_dtype()), np.zeros(cap, abi.calc_dtype())

    @staticmethod
    def add_fluid_volume(p, disp, calc, count, vmin, vmax, spacing, phase=0, jitter=0.0, seed=0, offs=(0, 0, 0)):
        n = C.c_int32(count)
        if lib().orc_add_fluid_volume(C.byref(p), _f3(vmin), _f3(vmax), float(spacing), _f3(offs), int(phase),
                                      float(jitter), int(seed), disp.ctypes.data, calc.ctypes.data, len(disp),
                                      C.byref(n)) != 0:
            raise ValueError("record arrays too small")
        return n.value

    @staticmethod
    def add_open_box(p, disp, calc, count, vmin, vmax, thickness):
        n = C.c_int32(count)
        if lib().orc_add_open_box(C.byref(p), _f3(vmin), _f3(vmax), float(thickness), disp.ctypes.data,
                                  calc.ctypes.data, len(disp), C.byref(n)) != 0:
            raise ValueError("record arrays too small")
        return n.value


def set_threads(n):
    lib().orc_set_num_threads(int(n))


def step(params, state, schedule=abi.SCHEDULE_FUSED, nsteps=1):
    return call("orc_step", params, state, int(schedule), int(nsteps))


def before_first_step(params, state):
    return call("orc_before_first_step", params, state)


def state_from_aos(disp, calc, gridtotal, dtype=np.float32):
    """State from reference records (numpy structured arrays of abi display/calc dtype)."""
    n = len(disp)
    s = State(n, gridtotal, dtype)
    s.pos[:] = disp["pos"]
    s.color[:] = disp["color"]
    s.type[:] = disp["type"]
    for k in ("vel", "veleval", "accel"):
        getattr(s, k)[:] = calc[k]
    for k in ("pressure", "dens", "restdens", "mass", "visc"):
        getattr(s, k)[:] = calc[k]
    s.bornid[:] = calc["bornid"]
    return s
