"""Python binding of libsphmp.so, the GB300-native multiphase SPH step.

Every call goes through the C ABI declared in include/sphmp.h. The library is
built in-tree by ``sphmp.build.build()``; importing this package never falls
back to anything else: if the shared library is missing or cannot be loaded,
``load()`` raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import CalcPack, DisplayPack, Params

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libsphmp.so")

_lib = None


class SphmpError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"sphmp error {status} ({abi.STATUS_NAMES.get(status, '?')}): {msg}")
        self.status = status


def load():
    """Load libsphmp.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with sphmp.build.build()")
    L = C.CDLL(LIB_PATH)
    P = C.POINTER
    vp = C.c_void_p
    ctx = C.c_void_p
    st = C.c_int
    sig = {
        "sphmp_params_default": (st, [P(Params)]),
        "sphmp_setup_constants": (st, [P(Params)]),
        "sphmp_setup_grid": (st, [P(Params)]),
        "sphmp_add_fluid_volume": (st, [P(Params), P(C.c_float), P(C.c_float), C.c_float, P(C.c_float), C.c_int32,
                                        C.c_float, C.c_uint64, vp, vp, C.c_int32, P(C.c_int32)]),
        "sphmp_add_wall": (st, [P(Params), P(C.c_float), P(C.c_float), vp, vp, C.c_int32, P(C.c_int32)]),
        "sphmp_add_open_box": (st, [P(Params), P(C.c_float), P(C.c_float), C.c_float, vp, vp, C.c_int32,
                                    P(C.c_int32)]),
        "sphmp_boundary_spacing": (C.c_float, [P(Params)]),
        "sphmp_create": (st, [P(Params), P(ctx)]),
        "sphmp_destroy": (st, [ctx]),
        "sphmp_set_params": (st, [ctx, P(Params)]),
        "sphmp_get_params": (st, [ctx, P(Params)]),
        "sphmp_set_stream": (st, [ctx, vp]),
        "sphmp_sync": (st, [ctx]),
        "sphmp_num_particles": (C.c_int32, [ctx]),
        "sphmp_upload_aos": (st, [ctx, vp, vp, C.c_int32]),
        "sphmp_download_aos": (st, [ctx, vp, vp, C.c_int32]),
        "sphmp_emit_aos": (st, [ctx, vp, vp, C.c_int32, C.c_int32]),
        "sphmp_upload_field": (st, [ctx, C.c_int32, vp, C.c_int32]),
        "sphmp_download_field": (st, [ctx, C.c_int32, vp, C.c_int32]),
        "sphmp_get_particle_index": (st, [ctx]),
        "sphmp_get_grid_list": (st, [ctx]),
        "sphmp_rearrange_data": (st, [ctx]),
        "sphmp_compute_boundary_density": (st, [ctx]),
        "sphmp_compute_pressure": (st, [ctx]),
        "sphmp_compute_drift_vel": (st, [ctx]),
        "sphmp_compute_alpha_advance": (st, [ctx]),
        "sphmp_compute_correction": (st, [ctx]),
        "sphmp_compute_force": (st, [ctx]),
        "sphmp_compute_force_projectu": (st, [ctx]),
        "sphmp_advance": (st, [ctx]),
        "sphmp_iisph_density": (st, [ctx]),
        "sphmp_iisph_predict_advection": (st, [ctx]),
        "sphmp_iisph_pressure_iteration": (st, [ctx, P(C.c_double)]),
        "sphmp_iisph_pressure_solve": (st, [ctx, C.c_float, C.c_int32, C.c_int32, P(C.c_int32), P(C.c_double)]),
        "sphmp_iisph_integrate": (st, [ctx]),
        "sphmp_step_iisph": (st, [ctx, C.c_int32, C.c_float, C.c_int32, P(C.c_int32), P(C.c_double)]),
        "sphmp_autotune": (st, [ctx, C.c_int32, C.c_int32, P(abi.Tuning)]),
        "sphmp_step": (st, [ctx, C.c_int32, C.c_int32, C.c_int32]),
        "sphmp_conservation": (st, [ctx, P(C.c_double), C.c_int32]),
        "sphmp_step_profile": (C.c_int32, [ctx, C.c_int32, P(C.c_float), C.c_char_p, C.c_int32]),
        "sphmp_device_errors": (st, [ctx, P(C.c_uint32)]),
        "sphmp_last_error": (C.c_char_p, []),
        "sphmp_version": (C.c_char_p, []),
        "sphmp_legacy_context": (ctx, []),
        "sphmp_write_frame_text": (st, [C.c_char_p, vp, vp, C.c_int32]),
        "sphmp_read_bi2": (st, [C.c_char_p, P(abi.Bi2Info), vp, vp, vp, C.c_int32]),
        "sphmp_add_bi2_shape": (st, [P(Params), vp, C.c_int32, C.c_float, P(C.c_float), P(C.c_float), C.c_int32,
                                     vp, vp, C.c_int32, P(C.c_int32)]),
        "sphmp_save_state": (st, [ctx, C.c_char_p]),
        "sphmp_download_display_async": (st, [ctx, vp, C.c_int32]),
        "sphmp_download_wait": (st, [ctx]),
        "sphmp_set_device_emitter": (st, [ctx, P(abi.Emitter), C.c_int32, C.c_int32, C.c_int32, C.c_float,
                                         C.c_uint64]),
        "sphmp_emit_disk": (st, [P(Params), P(abi.Emitter), C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_uint64,
                                 vp, vp, C.c_int32, P(C.c_int32)]),
        "sphmp_load_state": (st, [ctx, C.c_char_p]),
        # the learned large-step corrector (include/sphmp_learned.h)
        "sphmp_corrector_create": (st, [C.c_int32, vp, P(vp)]),
        "sphmp_corrector_destroy": (None, [vp]),
        "sphmp_corrector_set_params": (st, [vp, P(C.c_float)]),
        "sphmp_corrector_get_params": (st, [vp, P(C.c_float)]),
        "sphmp_corrector_set_normalisation": (st, [vp, P(C.c_float), P(C.c_float), P(C.c_float)]),
        "sphmp_corrector_forward": (st, [vp, vp, C.c_int32, vp]),
        "sphmp_corrector_gradients": (st, [vp, vp, vp, C.c_int32, P(C.c_float), P(C.c_float)]),
        "sphmp_corrector_train_step": (st, [vp, vp, vp, C.c_int32, C.c_float, P(C.c_float)]),
        "sphmp_corrector_sync": (st, [vp]),
        "sphmp_gemm_bf16_tn": (st, [vp, C.c_int32, vp, C.c_int32, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    vp]),
        "sphmp_step_large": (st, [ctx, vp, C.c_int32, C.c_int32]),
        "sphmp_learned_features": (st, [ctx, vp, vp, vp, P(C.c_int32)]),
        "sphmp_copy_state": (st, [ctx, ctx]),
        "sphmp_compare_states": (st, [ctx, ctx, P(C.c_double), C.c_int32]),
        "sphmp_rollout": (st, [ctx, ctx, vp, C.c_int32, C.c_int32, C.c_int32, C.c_double, P(abi.RolloutStats)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error():
    return load().sphmp_last_error().decode()


def check(status):
    if status != abi.OK:
        raise SphmpError(status, last_error())


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


# ---------------------------------------------------------------------------
# host-side setup (no GPU needed)
# ---------------------------------------------------------------------------

def params_default():
    p = Params()
    check(load().sphmp_params_default(C.byref(p)))
    return p


def setup_constants(p):
    check(load().sphmp_setup_constants(C.byref(p)))
    return p


def setup_grid(p):
    check(load().sphmp_setup_grid(C.byref(p)))
    return p


def boundary_spacing(p):
    return float(load().sphmp_boundary_spacing(C.byref(p)))


def record_arrays(cap):
    """Zeroed numpy record arrays (display, calc) with the reference layouts."""
    return np.zeros(cap, abi.display_dtype()), np.zeros(cap, abi.calc_dtype())


def add_fluid_volume(p, disp, calc, count, vmin, vmax, spacing, phase=0, jitter=0.0, seed=0, offs=(0, 0, 0)):
    n = C.c_int32(count)
    check(load().sphmp_add_fluid_volume(C.byref(p), _f3(vmin), _f3(vmax), float(spacing), _f3(offs), int(phase),
                                        float(jitter), int(seed), disp.ctypes.data, calc.ctypes.data, len(disp),
                                        C.byref(n)))
    return n.value


def add_wall(p, disp, calc, count, vmin, vmax):
    n = C.c_int32(count)
    check(load().sphmp_add_wall(C.byref(p), _f3(vmin), _f3(vmax), disp.ctypes.data, calc.ctypes.data, len(disp),
                                C.byref(n)))
    return n.value


def add_open_box(p, disp, calc, count, vmin, vmax, thickness):
    n = C.c_int32(count)
    check(load().sphmp_add_open_box(C.byref(p), _f3(vmin), _f3(vmax), float(thickness), disp.ctypes.data,
                                    calc.ctypes.data, len(disp), C.byref(n)))
    return n.value


# ---------------------------------------------------------------------------
# device context
# ---------------------------------------------------------------------------

FIELD_SHAPES = {
    abi.F_POS: (3,), abi.F_VEL: (3,), abi.F_VELEVAL: (3,), abi.F_ACCEL: (3,), abi.F_ALPHA: (3,),
    abi.F_ALPHA_PRE: (3,), abi.F_APREV: (3,), abi.F_DRIFT: (3, 3), abi.F_VELXCOR: (3,),
}
FIELD_DTYPES = {abi.F_TYPE: np.int32, abi.F_BORNID: np.int32, abi.F_MGCELL: np.uint32, abi.F_MIDSORT: np.uint32,
                abi.F_MGNDX: np.uint32, abi.F_MGRIDOFF: np.int32, abi.F_MGRIDCNT: np.int32}


class Context:
    """One simulation on the current CUDA device (owns its device buffers)."""

    def __init__(self, params):
        L = load()
        self._lib = L
        self._ptr = C.c_void_p()
        check(L.sphmp_create(C.byref(params), C.byref(self._ptr)))
        self.params = params.copy()

    def close(self):
        if self._ptr:
            self._lib.sphmp_destroy(self._ptr)
            self._ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def n(self):
        return int(self._lib.sphmp_num_particles(self._ptr))

    def set_params(self, p):
        check(self._lib.sphmp_set_params(self._ptr, C.byref(p)))
        self.params = p.copy()

    def get_params(self):
        p = Params()
        check(self._lib.sphmp_get_params(self._ptr, C.byref(p)))
        return p

    def set_stream(self, stream_ptr):
        check(self._lib.sphmp_set_stream(self._ptr, C.c_void_p(stream_ptr or 0)))

    def sync(self):
        check(self._lib.sphmp_sync(self._ptr))

    # transfers
    def upload_aos(self, disp, calc, n=None):
        n = len(disp) if n is None else n
        check(self._lib.sphmp_upload_aos(self._ptr, disp.ctypes.data, calc.ctypes.data, int(n)))

    def emit_aos(self, disp, calc, start, end):
        check(self._lib.sphmp_emit_aos(self._ptr, disp.ctypes.data, calc.ctypes.data, int(start), int(end)))

    def download_aos(self, n=None, calc=True, out=None):
        n = self.n if n is None else n
        if out is None:
            d, c = record_arrays(n)
        else:
            d, c = out
        check(self._lib.sphmp_download_aos(self._ptr, d.ctypes.data, c.ctypes.data if calc else None, int(n)))
        return (d, c) if calc else d

    def upload_field(self, field, arr):
        dt = FIELD_DTYPES.get(field, np.float32)
        a = np.ascontiguousarray(arr, dtype=dt)
        n = a.shape[0]
        check(self._lib.sphmp_upload_field(self._ptr, int(field), a.ctypes.data, int(n)))

    def download_field(self, field, n=None):
        if field in (abi.F_MGRIDOFF, abi.F_MGRIDCNT):
            n = self.params.gridtotal if n is None else n
        else:
            n = self.n if n is None else n
        dt = FIELD_DTYPES.get(field, np.float32)
        a = np.zeros((n,) + FIELD_SHAPES.get(field, ()), dt)
        check(self._lib.sphmp_download_field(self._ptr, int(field), a.ctypes.data, int(n)))
        return a

    # per-pass entry points (reference launch wrappers)
    def get_particle_index(self):
        check(self._lib.sphmp_get_particle_index(self._ptr))

    def get_grid_list(self):
        check(self._lib.sphmp_get_grid_list(self._ptr))

    def rearrange_data(self):
        check(self._lib.sphmp_rearrange_data(self._ptr))

    def sort(self):
        self.get_particle_index()
        self.get_grid_list()
        self.rearrange_data()

    def compute_boundary_density(self):
        check(self._lib.sphmp_compute_boundary_density(self._ptr))

    def compute_pressure(self):
        check(self._lib.sphmp_compute_pressure(self._ptr))

    def compute_drift_vel(self):
        check(self._lib.sphmp_compute_drift_vel(self._ptr))

    def compute_alpha_advance(self):
        check(self._lib.sphmp_compute_alpha_advance(self._ptr))

    def compute_correction(self):
        check(self._lib.sphmp_compute_correction(self._ptr))

    def compute_force(self):
        check(self._lib.sphmp_compute_force(self._ptr))

    def compute_force_projectu(self):
        check(self._lib.sphmp_compute_force_projectu(self._ptr))

    def advance(self):
        check(self._lib.sphmp_advance(self._ptr))

    def autotune(self, trial_steps=10, allow_reorder=False):
        """Pick the fastest launch configuration for the current state (sphmp_autotune)."""
        t = abi.Tuning()
        check(self._lib.sphmp_autotune(self._ptr, int(trial_steps), int(bool(allow_reorder)), C.byref(t)))
        return t.as_dict()

    # ---- IISPH step ----
    def iisph_density(self):
        check(self._lib.sphmp_iisph_density(self._ptr))

    def iisph_predict_advection(self):
        check(self._lib.sphmp_iisph_predict_advection(self._ptr))

    def iisph_pressure_iteration(self):
        """One pressure iteration; returns (the reference's mean residue over all slots,
        mean |residue| over in-grid fluid particles)."""
        r = (C.c_double * 2)()
        check(self._lib.sphmp_iisph_pressure_iteration(self._ptr, r))
        return r[0], r[1]

    def iisph_pressure_solve(self, tol=0.1, min_iter=2, max_iter=100):
        it = C.c_int32(0)
        r = (C.c_double * 2)()
        check(self._lib.sphmp_iisph_pressure_solve(self._ptr, float(tol), int(min_iter), int(max_iter),
                                                   C.byref(it), r))
        return it.value, (r[0], r[1])

    def iisph_integrate(self):
        check(self._lib.sphmp_iisph_integrate(self._ptr))

    def step_iisph(self, nsteps=1, tol=0.1, max_iter=100):
        its = (C.c_int32 * max(int(nsteps), 1))()
        r = (C.c_double * 2)()
        check(self._lib.sphmp_step_iisph(self._ptr, int(nsteps), float(tol), int(max_iter), its, r))
        return list(its)[:int(nsteps)], (r[0], r[1])

    def set_device_emitter(self, position, direction, speed, radius, spacing, layers=2, phase=0, interval=22,
                           jitter=1.0, seed=0):
        """Emit disks on the device inside every step whose frame is a multiple of
        `interval` (see sphmp_set_device_emitter); interval 0 turns it off."""
        e = abi.Emitter()
        for a in range(3):
            e.position[a] = position[a]
            e.dir[a] = direction[a]
        e.vel, e.radius, e.spacing = speed, radius, spacing
        check(self._lib.sphmp_set_device_emitter(self._ptr, C.byref(e), int(layers), int(phase), int(interval),
                                                 float(jitter), int(seed)))

    def before_first_step(self):
        """Sort, then boundary volumes (reference FluidSystem::BeforeFirstStep)."""
        self.sort()
        self.compute_boundary_density()

    def step(self, nsteps=1, schedule=abi.SCHEDULE_FUSED, use_graph=True):
        check(self._lib.sphmp_step(self._ptr, int(nsteps), int(schedule), int(bool(use_graph))))

    def step_profile(self, schedule=abi.SCHEDULE_FUSED):
        """One eager step; returns [(stage name, milliseconds)] timed with CUDA events."""
        ms = (C.c_float * 24)()
        names = C.create_string_buffer(32 * 24)
        n = self._lib.sphmp_step_profile(self._ptr, int(schedule), ms, names, 24)
        if n < 0:
            raise SphmpError(-n, last_error())
        raw = names.raw
        return [(raw[32 * i:32 * i + 32].split(b"\0")[0].decode(), float(ms[i])) for i in range(n)]

    def conservation(self):
        k = self.params.nphase
        out = (C.c_double * (3 + k))()
        check(self._lib.sphmp_conservation(self._ptr, out, 3 + k))
        return {"mass": out[0], "volume": out[1], "phase_volume": [out[2 + i] for i in range(k)],
                "alpha_sum_err": out[2 + k]}

    def device_errors(self):
        bits = C.c_uint32(0)
        check(self._lib.sphmp_device_errors(self._ptr, C.byref(bits)))
        return bits.value

    def download_display_async(self, disp, n=None):
        """Queue a download of the display records into `disp` (pinned numpy memory); see download_wait."""
        n = self.n if n is None else n
        check(self._lib.sphmp_download_display_async(self._ptr, disp.ctypes.data, int(n)))

    def download_wait(self):
        check(self._lib.sphmp_download_wait(self._ptr))

    def save_state(self, path):
        check(self._lib.sphmp_save_state(self._ptr, os.fsencode(path)))

    def load_state(self, path):
        check(self._lib.sphmp_load_state(self._ptr, os.fsencode(path)))

    # the learned large step (include/sphmp_learned.h)
    def step_large(self, factor=8, nsteps=1, corrector=None):
        """nsteps fused steps of factor x dt, each corrected by `corrector` (a Corrector) when given."""
        cor = corrector._ptr if corrector is not None else None
        check(self._lib.sphmp_step_large(self._ptr, cor, int(factor), int(nsteps)))

    def learned_features(self, feat=None, ids=None, corr=None):
        """Copy the last corrected step's per-row features / bornids / corrections into
        device buffers (torch tensors or None); returns the row count."""
        cnt = C.c_int32(0)
        ptr = lambda t: None if t is None else C.c_void_p(t.data_ptr())
        check(self._lib.sphmp_learned_features(self._ptr, ptr(feat), ptr(ids), ptr(corr), C.byref(cnt)))
        return cnt.value

    def copy_state_from(self, src):
        """Replace this context's particles by those of `src` (on the device)."""
        check(self._lib.sphmp_copy_state(self._ptr, src._ptr))

    def compare_to(self, ref):
        """Differences of this state against `ref`'s (sphmp_compare_states)."""
        out = (C.c_double * 6)()
        check(self._lib.sphmp_compare_states(ref._ptr, self._ptr, out, 6))
        return {"density_rms": out[0], "density_max": out[1], "alpha_rms": out[2], "velocity_rms_rel": out[3],
                "count": int(out[4]), "position_rms_m": out[5]}

    def rollout(self, audit, steps, factor=8, corrector=None, audit_every=16, tol=0.01):
        """Advance by `steps` plain steps' worth of time in audited large steps (sphmp_rollout)."""
        st = abi.RolloutStats()
        cor = corrector._ptr if corrector is not None else None
        check(self._lib.sphmp_rollout(self._ptr, audit._ptr, cor, int(factor), int(steps), int(audit_every),
                                      float(tol), C.byref(st)))
        return st.as_dict()


class Corrector:
    """The learned large-step corrector network (device parameters, Adam state,
    training buffers for batches of up to max_batch rows). Device arrays are
    passed as torch tensors (float32, contiguous, on the current device)."""

    def __init__(self, max_batch=0, stream_ptr=0):
        self._lib = load()
        self._ptr = C.c_void_p()
        check(self._lib.sphmp_corrector_create(int(max_batch), C.c_void_p(stream_ptr or 0), C.byref(self._ptr)))
        self.max_batch = max_batch

    def close(self):
        if self._ptr:
            self._lib.sphmp_corrector_destroy(self._ptr)
            self._ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        a = np.ascontiguousarray(params, np.float32)
        if a.size != abi.LC_PARAMS:
            raise ValueError(f"need {abi.LC_PARAMS} parameters, got {a.size}")
        check(self._lib.sphmp_corrector_set_params(self._ptr, a.ctypes.data_as(C.POINTER(C.c_float))))

    def get_params(self):
        a = np.zeros(abi.LC_PARAMS, np.float32)
        check(self._lib.sphmp_corrector_get_params(self._ptr, a.ctypes.data_as(C.POINTER(C.c_float))))
        return a

    def set_normalisation(self, feat_shift, feat_scale, out_scale):
        fp = lambda v, n: np.ascontiguousarray(v, np.float32).reshape(n)
        a, b, c = fp(feat_shift, abi.LC_FEATURES), fp(feat_scale, abi.LC_FEATURES), fp(out_scale, abi.LC_OUTPUTS)
        P = C.POINTER(C.c_float)
        check(self._lib.sphmp_corrector_set_normalisation(self._ptr, a.ctypes.data_as(P), b.ctypes.data_as(P),
                                                          c.ctypes.data_as(P)))

    def forward(self, x, y):
        check(self._lib.sphmp_corrector_forward(self._ptr, C.c_void_p(x.data_ptr()), int(x.shape[0]),
                                                C.c_void_p(y.data_ptr())))

    def gradients(self, x, t):
        """(flat gradient array, loss) of one batch, no update."""
        g = np.zeros(abi.LC_PARAMS, np.float32)
        loss = C.c_float(0.0)
        check(self._lib.sphmp_corrector_gradients(self._ptr, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()),
                                                  int(x.shape[0]), g.ctypes.data_as(C.POINTER(C.c_float)),
                                                  C.byref(loss)))
        return g, loss.value

    def train_step(self, x, t, lr, want_loss=False):
        loss = C.c_float(0.0)
        check(self._lib.sphmp_corrector_train_step(self._ptr, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()),
                                                   int(x.shape[0]), float(lr),
                                                   C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def sync(self):
        check(self._lib.sphmp_corrector_sync(self._ptr))


def gemm_bf16_tn(a, b, d, splits=1, stream_ptr=0):
    """d[s] = a @ b.T over split s's K range (torch bf16 a [m][k], b [n][k]; float32 d [splits][m][n])."""
    m, k = a.shape
    n = b.shape[0]
    check(load().sphmp_gemm_bf16_tn(C.c_void_p(a.data_ptr()), int(a.stride(0)), C.c_void_p(b.data_ptr()),
                                    int(b.stride(0)), C.c_void_p(d.data_ptr()), int(m), int(n), int(k), int(splits),
                                    C.c_void_p(stream_ptr or 0)))


# ---------------------------------------------------------------------------
# particle data formats (host only)
# ---------------------------------------------------------------------------

def write_frame_text(path, disp, calc, n=None):
    """The reference's text frame dump (FluidSystem::outputFile)."""
    n = len(disp) if n is None else n
    check(load().sphmp_write_frame_text(os.fsencode(path), disp.ctypes.data, calc.ctypes.data, int(n)))


def read_bi2(path, header_only=False):
    """(info dict, pos[np,3], vel[np,3], rhop[np]) of a BINX-020 file."""
    info = abi.Bi2Info()
    L = load()
    check(L.sphmp_read_bi2(os.fsencode(path), C.byref(info), None, None, None, 0))
    if header_only:
        return info.as_dict(), None, None, None
    n = info.np
    pos = np.zeros((n, 3), np.float32)
    vel = np.zeros((n, 3), np.float32)
    rhop = np.zeros(n, np.float32)
    check(L.sphmp_read_bi2(os.fsencode(path), C.byref(info), pos.ctypes.data, vel.ctypes.data, rhop.ctypes.data, n))
    return info.as_dict(), pos, vel, rhop


def emit_disk(p, disp, calc, count, position, direction, speed, radius, spacing, layers=2, phase=0, frame=0,
              jitter=1.0, seed=0):
    """Append emitted disks (the reference's EmitParticles); returns the new count."""
    e = abi.Emitter()
    for a in range(3):
        e.position[a] = position[a]
        e.dir[a] = direction[a]
    e.vel, e.radius, e.spacing = speed, radius, spacing
    n = C.c_int32(count)
    check(load().sphmp_emit_disk(C.byref(p), C.byref(e), int(layers), int(phase), int(frame), float(jitter),
                                 int(seed), disp.ctypes.data, calc.ctypes.data, len(disp), C.byref(n)))
    return n.value


def add_bi2_shape(p, disp, calc, count, pos, scale=0.005, offs=(0, 0, 0), vel=(0, -1.5, 0), phase=2):
    """Append .bi2 shape particles as fluid (the reference's FluidSystem::AddShape); returns the new count."""
    pos = np.ascontiguousarray(pos, np.float32)
    n = C.c_int32(count)
    check(load().sphmp_add_bi2_shape(C.byref(p), pos.ctypes.data, len(pos), float(scale), _f3(offs), _f3(vel),
                                     int(phase), disp.ctypes.data, calc.ctypes.data, len(disp), C.byref(n)))
    return n.value


__all__ = ["abi", "Params", "DisplayPack", "CalcPack", "Context", "Corrector", "gemm_bf16_tn", "SphmpError", "load",
           "check", "last_error",
           "params_default", "setup_constants", "setup_grid", "boundary_spacing", "record_arrays",
           "add_fluid_volume", "add_wall", "add_open_box", "write_frame_text", "read_bi2", "add_bi2_shape", "emit_disk"]
