"""Shared helpers for the parity tests: oracle states mirroring a device context,
field comparison, and scene construction."""
import numpy as np

import sphmp
from oracle import oracle as O
from sphmp import abi, scenes

UNDEF = abi.GRID_UNDEF


def onehot_alpha(params, restdens):
    """One-hot volume fractions at the first phase whose rest density matches (the
    rule sphmp_upload_aos applies)."""
    n = len(restdens)
    ph = np.zeros(n, np.int64)
    found = np.zeros(n, bool)
    for k in range(params.nphase):
        hit = (restdens == np.float32(params.densArr[k])) & ~found
        ph[hit] = k
        found |= hit
    a = np.zeros((n, 3), np.float32)
    a[np.arange(n), ph] = 1.0
    return a


def oracle_state(scene, dtype=np.float32):
    p = scene.params
    s = O.state_from_aos(scene.disp, scene.calc, p.gridtotal, dtype)
    a = onehot_alpha(p, scene.calc["restdens"])
    s.alpha[:] = a
    s.alpha_pre[:] = a
    # the device keeps no accel/pressure for boundary records; start them at zero on both sides
    bnd = s.type == 1
    s.accel[bnd] = 0
    s.pressure[bnd] = 0
    return s


def device_ctx(scene):
    ctx = sphmp.Context(scene.params)
    calc = scene.calc.copy()
    bnd = scene.disp["type"] == 1
    calc["accel"][bnd] = 0
    calc["pressure"][bnd] = 0
    ctx.upload_aos(scene.disp, calc)
    return ctx


def field_err(got, ref, floor=0.0):
    """max |got - ref| / max(max |ref|, floor) (0 when both are empty)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    if ref.size == 0:
        return 0.0
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    if not np.all(np.isfinite(ref) | same):
        return float("inf")  # a non-finite reference value the device does not reproduce
    got = np.where(same, 0.0, got)
    ref = np.where(same, 0.0, ref)
    if not np.all(np.isfinite(got)):
        return float("inf")
    scale = max(float(np.max(np.abs(ref))), floor)
    if scale == 0.0:
        return float(np.max(np.abs(got)))
    return float(np.max(np.abs(got - ref))) / scale


def rel_err_quantile(got, ref, q=99.9, floor_frac=1e-3):
    """The q-th percentile over elements of |got - ref| / max(|ref|, floor_frac * max|ref|):
    a per-element relative error beside the max-norm of field_err (the floor keeps
    elements near zero from reading as large relative errors)."""
    got = np.asarray(got, np.float64).ravel()
    ref = np.asarray(ref, np.float64).ravel()
    if ref.size == 0:
        return 0.0
    den = np.maximum(np.abs(ref), floor_frac * max(float(np.max(np.abs(ref))), 1e-300))
    return float(np.percentile(np.abs(got - ref) / den, q))


def rms_err(got, ref):
    """sqrt(mean (got - ref)^2) / sqrt(mean ref^2)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.sqrt(np.mean((got - ref) ** 2)) / max(np.sqrt(np.mean(ref ** 2)), 1e-300))


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.dtype == np.float32:
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    return np.array_equal(a, b)


def download_state(ctx, n=None):
    """Per-slot arrays of a device context in the oracle's layout."""
    out = {}
    F = abi
    for name, fid in [("pos", F.F_POS), ("vel", F.F_VEL), ("veleval", F.F_VELEVAL), ("pressure", F.F_PRESSURE),
                      ("dens", F.F_DENS), ("restdens", F.F_RESTDENS), ("visc", F.F_VISC), ("accel", F.F_ACCEL),
                      ("alpha", F.F_ALPHA), ("alpha_pre", F.F_ALPHA_PRE), ("drift", F.F_DRIFT),
                      ("aprev", F.F_APREV), ("pmod", F.F_PMOD), ("type", F.F_TYPE), ("mass", F.F_MASS),
                      ("bornid", F.F_BORNID), ("mgcell", F.F_MGCELL), ("midsort", F.F_MIDSORT),
                      ("mgndx", F.F_MGNDX), ("mgridoff", F.F_MGRIDOFF), ("mgridcnt", F.F_MGRIDCNT),
                      ("velxcor", F.F_VELXCOR)]:
        out[name] = ctx.download_field(fid, None if name in ("mgridoff", "mgridcnt") else n)
    return out


def upload_state_fields(ctx, s, names):
    """Copy oracle-state arrays into the device context (fields that can be uploaded)."""
    F = abi
    fid = {"pos": F.F_POS, "vel": F.F_VEL, "veleval": F.F_VELEVAL, "pressure": F.F_PRESSURE,
           "restdens": F.F_RESTDENS, "visc": F.F_VISC, "accel": F.F_ACCEL, "alpha": F.F_ALPHA,
           "alpha_pre": F.F_ALPHA_PRE, "drift": F.F_DRIFT, "aprev": F.F_APREV, "pmod": F.F_PMOD}
    for nm in names:
        ctx.upload_field(fid[nm], getattr(s, nm))


def in_grid_fluid(s_or_dict):
    get = (lambda k: s_or_dict[k]) if isinstance(s_or_dict, dict) else (lambda k: getattr(s_or_dict, k))
    return (get("mgcell") != UNDEF) & (get("type") == 0)


def build_c_host(out_dir):
    """Compile tests/c_host/legacy_host.cpp against include/ and link libsphmp.so, as
    a C++ host application of the reference would; returns the executable's path."""
    import os
    import subprocess
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.dirname(sphmp.load()._name)
    exe = os.path.join(str(out_dir), "legacy_host")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++14", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(repo, "include"), os.path.join(repo, "tests", "c_host", "legacy_host.cpp"),
           "-o", exe, "-L", libdir, "-lsphmp", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def write_c_host_inputs(out_dir, scene):
    """params.bin, display.bin, calc.bin for legacy_host (boundary accel/pressure zeroed, as the
    oracle state starts); returns the three paths."""
    import os
    calc = scene.calc[:scene.n].copy()
    bnd = scene.disp["type"][:scene.n] == abi.TYPE_BOUNDARY
    calc["accel"][bnd] = 0
    calc["pressure"][bnd] = 0
    paths = [os.path.join(str(out_dir), f) for f in ("params.bin", "display.bin", "calc.bin")]
    with open(paths[0], "wb") as f:
        f.write(bytes(scene.params))
    np.ascontiguousarray(scene.disp[:scene.n]).tofile(paths[1])
    calc.tofile(paths[2])
    return paths

