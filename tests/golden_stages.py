"""Stage list shared by the golden-fixture generator and the tests that replay it."""
import numpy as np

from oracle import oracle as O

# (stage, fields saved after it). "multiphase_inputs" seeds alpha / alpha_pre / aprev.
# Stages in SIDE_STAGES run on a copy of the state: the chain goes on from the
# state before them (the project-U force replaces MfComputeForce's accel only in
# its own schedule, so the advance keeps reading the MfComputeForce result).
STAGES = [
    ("get_particle_index", ["mgcell", "midsort"]),
    ("get_grid_list", ["mgcell", "midsort", "mgridoff", "mgridcnt", "mgndx"]),
    ("rearrange_data", ["pos", "type", "vel", "veleval", "restdens", "mass", "visc", "bornid", "dens"]),
    ("compute_boundary_volume", ["dens"]),
    ("compute_pressure", ["dens", "pressure"]),
    ("compute_force", ["accel"]),
    ("surface_tension", ["accel"]),
    ("multiphase_inputs", ["alpha", "alpha_pre", "aprev"]),
    ("compute_drift_vel", ["drift"]),
    ("compute_alpha_advance", ["alpha"]),
    ("compute_correction", ["alpha", "restdens", "visc", "pmod"]),
    ("compute_force_projectu", ["accel", "velxcor"]),
    ("advance", ["pos", "vel", "veleval"]),
]
SIDE_STAGES = {"compute_force_projectu"}


def state_arrays(s):
    return {k: getattr(s, k).copy() for k in s.fields()}


def prepare_multiphase(p, s, seed):
    """Seeded fractions (one-hot by rest density, blended with noise) and previous accelerations."""
    rng = np.random.default_rng(seed)
    k = p.nphase
    a = np.zeros((s.n, 3), s.dtype)
    for q in range(k):
        a[:, q] = s.restdens == np.float32(p.densArr[q])
    a[:, :k] = a[:, :k] * 0.8 + 0.2 * rng.random((s.n, k)).astype(s.dtype)
    a[:, :k] /= a[:, :k].sum(1, keepdims=True)
    s.alpha[:] = a
    s.alpha_pre[:] = a
    s.aprev[:] = rng.normal(0.0, 3.0, (s.n, 3)).astype(s.dtype)


def load_fixture(path):
    from sphmp import abi
    z = np.load(path)
    p = abi.Params.from_buffer_copy(z["params"].tobytes())
    s = O.State(int(z["n"]), p.gridtotal)
    for k in s.fields():
        if "init_" + k in z.files:  # state fields added after a fixture was written start at zero
            getattr(s, k)[...] = z["init_" + k]
    return p, s, z
