"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

Sort outputs (cell ids, offsets, counts, rank-in-cell, permutation) and the
reordered positions must be bit-identical. Per-pass floating-point fields must
agree within RTOL = 1e-5 measured as max|gpu - oracle| / max|oracle| over
in-grid slots, on identical inputs. The advance is bit-identical given the same
acceleration.
"""
import numpy as np
import pytest

import sphmp
from helpers import (UNDEF, bits_equal, device_ctx, download_state, field_err, in_grid_fluid, oracle_state,
                     upload_state_fields)
from oracle import oracle as O
from sphmp import abi, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _scene(kind):
    if kind == "tait2":
        return scenes.small_block(seed=11, n=(14, 12, 10), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.3)
    if kind == "tait3":
        return scenes.small_block(seed=12, n=(16, 10, 12), nphase=3, eos=abi.EOS_TAIT, velocity_scale=0.5)
    if kind == "linear1":
        return scenes.small_block(seed=13, n=(10, 14, 9), nphase=1, eos=abi.EOS_LINEAR, velocity_scale=0.2)
    if kind == "simscale":
        return scenes.small_block(seed=14, n=(12, 12, 12), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.2,
                                  simscale=0.5, h=0.01, d=0.01)
    if kind == "dam":
        return scenes.dam_break_2phase(seed=15, n_side=16, box=0.32)
    if kind == "liquids3":  # no gas next to liquid: the project-U force stays finite
        sc = scenes.small_block(seed=16, n=(14, 12, 13), nphase=3, eos=abi.EOS_TAIT, velocity_scale=0.4,
                                dens=(1000.0, 800.0, 900.0), phase_frac=0.5)
        sc.params.mf_omega = 0.7
        sc.params.mf_visc_factor = 1.3
        return sc
    raise KeyError(kind)


KINDS = ["tait2", "tait3", "linear1", "simscale", "dam"]


def _resort(p, s, ctx):
    for st in ("orc_get_particle_index", "orc_get_grid_list", "orc_rearrange_data"):
        O.call(st, p, s)
    ctx.sort()


def _sorted_pair(kind, resort=True):
    """Both sides sorted with boundary volumes computed. With `resort`, a second
    sort (idempotent on the slot order) rebuilds the device's octant order, so the
    density runs its octant-order kernel; without it, the slot-order kernel."""
    sc = _scene(kind)
    s = oracle_state(sc)
    O.before_first_step(sc.params, s)
    ctx = device_ctx(sc)
    ctx.before_first_step()
    if resort:
        _resort(sc.params, s, ctx)
    ctx.sync()
    return sc, s, ctx


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    sphmp.load()


@pytest.mark.parametrize("kind", KINDS)
def test_sort_bit_exact(kind):
    sc, s, ctx = _sorted_pair(kind)
    g = download_state(ctx)
    for k in ("mgcell", "midsort", "mgridoff", "mgridcnt"):
        assert bits_equal(g[k], getattr(s, k)), k
    m = s.mgcell != UNDEF
    assert np.array_equal(g["mgndx"][m], s.mgndx[m])
    assert bits_equal(g["pos"], s.pos)
    assert np.array_equal(g["type"], s.type)
    assert np.array_equal(g["bornid"], s.bornid)
    assert bits_equal(g["mass"], s.mass)
    # boundary volumes (V_b in dens for boundary slots)
    b = (s.type == 1) & m
    assert field_err(g["dens"][b], s.dens[b]) < RTOL
    ctx.close()


@pytest.mark.parametrize("resort", [True, False], ids=["octant", "slot_order"])
@pytest.mark.parametrize("kind", KINDS)
def test_density_force_advance(kind, resort):
    sc, s, ctx = _sorted_pair(kind, resort)
    p = sc.params
    O.call("orc_compute_pressure", p, s)
    ctx.compute_pressure()
    g = download_state(ctx)
    f = in_grid_fluid(s)
    assert field_err(g["dens"][f], s.dens[f]) < RTOL
    assert field_err(g["pressure"][f], s.pressure[f], floor=1e-3) < RTOL
    O.call("orc_compute_force", p, s)
    ctx.compute_force()
    g = download_state(ctx)
    assert field_err(g["accel"][f], s.accel[f]) < RTOL
    # advance from identical accelerations is bit-identical
    upload_state_fields(ctx, s, ["accel"])
    O.call("orc_advance", p, s)
    ctx.advance()
    g = download_state(ctx)
    for k in ("pos", "vel", "veleval", "aprev"):
        assert bits_equal(g[k][f], getattr(s, k)[f]), k
    ctx.close()


@pytest.mark.parametrize("kind", ["tait2", "tait3", "simscale", "dam"])
def test_multiphase_passes(kind):
    sc, s, ctx = _sorted_pair(kind)
    p = sc.params
    rng = np.random.default_rng(3)
    # perturb the fractions and give every particle a previous acceleration
    a = s.alpha.copy()
    npz = p.nphase
    a[:, :npz] = a[:, :npz] * 0.7 + 0.3 * rng.random((s.n, npz)).astype(np.float32)
    a[:, :npz] /= a[:, :npz].sum(1, keepdims=True)
    s.alpha[:] = a
    s.alpha_pre[:] = a
    s.aprev[:] = rng.normal(0, 3.0, (s.n, 3)).astype(np.float32)
    upload_state_fields(ctx, s, ["alpha_pre", "aprev"])
    O.call("orc_compute_pressure", p, s)
    ctx.compute_pressure()
    O.call("orc_compute_drift_vel", p, s)
    ctx.compute_drift_vel()
    g = download_state(ctx)
    f = in_grid_fluid(s)
    k = p.nphase
    assert field_err(g["drift"][f][:, :k], s.drift[f][:, :k]) < RTOL
    # alpha advance from the oracle's drift velocities
    upload_state_fields(ctx, s, ["drift"])
    O.call("orc_compute_alpha_advance", p, s)
    ctx.compute_alpha_advance()
    g = download_state(ctx)
    assert field_err(g["alpha"][f][:, :k], s.alpha[f][:, :k], floor=1.0) < RTOL
    # correction from the oracle's advanced fractions
    upload_state_fields(ctx, s, ["alpha"])
    O.call("orc_compute_correction", p, s)
    ctx.compute_correction()
    g = download_state(ctx)
    assert field_err(g["alpha"][f][:, :k], s.alpha[f][:, :k], floor=1.0) < RTOL
    assert field_err(g["restdens"][f], s.restdens[f]) < RTOL
    assert field_err(g["visc"][f], s.visc[f]) < RTOL
    assert field_err(g["pmod"][f], s.pmod[f], floor=1e-6) < 1e-4
    ctx.close()


@pytest.mark.parametrize("kind", ["liquids3", "dam"])
def test_projectu_pass(kind):
    """ComputeForce_projectu on identical inputs: drift velocities, start-of-step
    fractions and the corrected rest densities and viscosities of the oracle."""
    sc, s, ctx = _sorted_pair(kind)
    p = sc.params
    rng = np.random.default_rng(4)
    a = s.alpha.copy()
    k = p.nphase
    a[:, :k] = a[:, :k] * 0.7 + 0.3 * rng.random((s.n, k)).astype(np.float32)
    a[:, :k] /= a[:, :k].sum(1, keepdims=True)
    s.alpha[:] = a
    s.alpha_pre[:] = a
    s.aprev[:] = rng.normal(0, 3.0, (s.n, 3)).astype(np.float32)
    fl = s.type == 0  # moving fluid (the dam starts at rest), so the XSPH term is not zero
    s.veleval[fl] = rng.normal(0, 0.3, (int(fl.sum()), 3)).astype(np.float32)
    upload_state_fields(ctx, s, ["alpha_pre", "aprev", "veleval"])
    O.call("orc_compute_pressure", p, s)
    ctx.compute_pressure()
    for st in ("orc_compute_drift_vel", "orc_compute_alpha_advance", "orc_compute_correction"):
        O.call(st, p, s)
    ctx.compute_drift_vel()
    ctx.compute_alpha_advance()
    ctx.compute_correction()
    upload_state_fields(ctx, s, ["drift", "restdens", "visc"])
    O.call("orc_compute_force_projectu", p, s)
    ctx.compute_force_projectu()
    g = download_state(ctx)
    f = in_grid_fluid(s)
    assert np.isfinite(s.accel[f]).all() and np.abs(s.velxcor[f]).max() > 0
    assert field_err(g["accel"][f], s.accel[f]) < RTOL
    assert field_err(g["velxcor"][f], s.velxcor[f]) < RTOL
    # boundary and out-of-grid slots carry no correction
    assert not g["velxcor"][~f].any()
    ctx.close()


@pytest.mark.parametrize("kind", ["liquids3", "dam"])
def test_projectu_step(kind):
    """One step of the legacy multiphase schedule with the project-U force."""
    sc, s, ctx = _sorted_pair(kind)
    p = sc.params
    O.step(p, s, abi.SCHEDULE_PROJECTU, 1)
    ctx.step(1, abi.SCHEDULE_PROJECTU, use_graph=True)
    ctx.sync()
    g = download_state(ctx)
    for key in ("mgcell", "midsort", "mgridoff", "mgridcnt"):
        assert bits_equal(g[key], getattr(s, key)), key
    f = in_grid_fluid(s)
    assert field_err(g["accel"][f], s.accel[f]) < RTOL
    assert field_err(g["velxcor"][f], s.velxcor[f]) < RTOL
    for key in ("pos", "vel", "veleval"):
        assert field_err(g[key][f], getattr(s, key)[f]) < RTOL, key
    kk = p.nphase
    assert field_err(g["alpha"][f][:, :kk], s.alpha[f][:, :kk], floor=1.0) < RTOL
    ctx.close()


def test_projectu_schedule_needs_multiphase():
    sc = _scene("liquids3")
    sc.params.multiphase = 0
    ctx = device_ctx(sc)
    with pytest.raises(sphmp.SphmpError) as e:
        ctx.step(1, abi.SCHEDULE_PROJECTU)
    assert e.value.status == abi.ERR_INVALID_ARG
    ctx.close()


@pytest.mark.parametrize("schedule", [abi.SCHEDULE_FUSED, abi.SCHEDULE_REFERENCE])
@pytest.mark.parametrize("kind", ["tait3", "dam"])
def test_full_step(kind, schedule):
    sc, s, ctx = _sorted_pair(kind)
    p = sc.params
    O.step(p, s, schedule, 1)
    ctx.step(1, schedule, use_graph=False)
    ctx.sync()
    g = download_state(ctx)
    for k in ("mgcell", "midsort", "mgridoff", "mgridcnt"):
        assert bits_equal(g[k], getattr(s, k)), k
    f = in_grid_fluid(s)
    assert field_err(g["dens"][f], s.dens[f]) < RTOL
    assert field_err(g["accel"][f], s.accel[f]) < RTOL
    for k in ("pos", "vel", "veleval"):
        assert field_err(g[k][f], getattr(s, k)[f]) < RTOL, k
    kk = p.nphase
    assert field_err(g["alpha"][f][:, :kk], s.alpha[f][:, :kk], floor=1.0) < RTOL
    ctx.close()


def test_graph_matches_eager():
    sc = _scene("tait3")
    res = []
    for use_graph in (False, True):
        ctx = device_ctx(sc)
        ctx.before_first_step()
        ctx.step(5, abi.SCHEDULE_FUSED, use_graph=use_graph)
        ctx.sync()
        res.append(download_state(ctx))
        ctx.close()
    for k in ("pos", "vel", "alpha", "mgcell", "midsort"):
        assert bits_equal(res[0][k], res[1][k]), k


@pytest.mark.parametrize("schedule", [abi.SCHEDULE_REFERENCE, abi.SCHEDULE_PROJECTU], ids=["reference", "projectu"])
def test_two_step_graph_matches_eager(schedule):
    """The reference-order schedules replay a captured pair of steps (an odd
    remainder runs eagerly): five steps, bit-identical to five eager steps."""
    sc = _scene("liquids3")
    res = []
    for use_graph in (False, True):
        ctx = device_ctx(sc)
        ctx.before_first_step()
        ctx.step(2, schedule, use_graph=use_graph)
        ctx.step(3, schedule, use_graph=use_graph)
        ctx.sync()
        res.append(download_state(ctx))
        ctx.close()
    for k in ("pos", "vel", "veleval", "alpha", "alpha_pre", "accel", "velxcor", "mgcell", "midsort"):
        assert bits_equal(res[0][k], res[1][k]), k


def test_pass_after_graph_steps_uses_fresh_neighbours():
    """A per-pass call after graph-replayed steps sees the state a step leaves
    (no neighbour list from before the steps): same bits as after eager steps."""
    sc = _scene("tait3")
    res = []
    for use_graph in (False, True):
        ctx = device_ctx(sc)
        ctx.before_first_step()
        ctx.step(1, abi.SCHEDULE_FUSED, use_graph=use_graph)  # with a graph: captured here
        ctx.compute_pressure()  # neighbour lists for the current positions
        ctx.step(1, abi.SCHEDULE_FUSED, use_graph=use_graph)  # replayed: the positions move
        ctx.compute_force()
        ctx.sync()
        res.append(download_state(ctx))
        ctx.close()
    assert bits_equal(res[0]["accel"], res[1]["accel"])


def test_graph_after_buffer_flipping_calls_matches_eager():
    """A captured step reads and writes the double buffers selected when it was
    captured. Between replays, an eager step of the reference order flips every
    selector an odd number of times; the next replay must use a graph captured
    for the new selectors: same bits as the same sequence run eagerly."""
    sc = _scene("tait3")
    res = []
    for use_graph in (False, True):
        ctx = device_ctx(sc)
        ctx.before_first_step()
        ctx.step(1, abi.SCHEDULE_FUSED, use_graph=use_graph)  # with a graph: captured here
        ctx.step(1, abi.SCHEDULE_REFERENCE, use_graph=False)  # odd number of selector flips
        ctx.step(2, abi.SCHEDULE_FUSED, use_graph=use_graph)
        ctx.sync()
        res.append(download_state(ctx))
        ctx.close()
    for name in ("pos", "vel", "dens", "alpha", "accel"):
        assert bits_equal(res[0][name], res[1][name]), name


def test_graph_survives_a_reupload_and_first_sort():
    """The end-to-end pattern: steps from a captured graph, then the same records
    uploaded again and the first-step sort (which flips the selectors), then more
    graph steps: same bits as a fresh context running the second part eagerly."""
    sc = _scene("tait3")
    calc = sc.calc.copy()
    bnd = sc.disp["type"] == 1
    calc["accel"][bnd] = 0
    calc["pressure"][bnd] = 0
    ctx = device_ctx(sc)
    ctx.before_first_step()
    ctx.step(3, abi.SCHEDULE_FUSED, use_graph=True)
    ctx.upload_aos(sc.disp, calc)
    ctx.before_first_step()
    ctx.step(3, abi.SCHEDULE_FUSED, use_graph=True)
    ctx.sync()
    got = download_state(ctx)
    ctx.close()
    ref = device_ctx(sc)
    ref.before_first_step()
    ref.step(3, abi.SCHEDULE_FUSED, use_graph=False)
    ref.sync()
    want = download_state(ref)
    ref.close()
    for name in ("pos", "vel", "dens", "alpha", "accel"):
        assert bits_equal(got[name], want[name]), name


def test_passes_after_advance_without_resort_match_oracle():
    """MfComputePressure / MfComputeForce called after an advance with no new sort:
    the neighbour loops scan the 27 cells around each particle's cell from the
    last sort (gc + neighborid, as the reference does), with positions that have
    moved since. Several steps of this, against the oracle doing the same."""
    sc, s, ctx = _sorted_pair("tait3")
    p = sc.params
    for _ in range(3):
        O.step(p, s, abi.SCHEDULE_FUSED, 1)
        ctx.step(1, abi.SCHEDULE_FUSED, use_graph=False)
        for st in ("orc_compute_pressure", "orc_compute_force"):
            O.call(st, p, s)
        ctx.compute_pressure()
        ctx.compute_force()
        ctx.sync()
        g = download_state(ctx)
        f = in_grid_fluid(s)
        assert field_err(g["dens"][f], s.dens[f]) < RTOL
        assert field_err(g["accel"][f], s.accel[f]) < RTOL
        upload_state_fields(ctx, s, ["pos", "vel", "veleval", "accel"])
        ctx.upload_field(abi.F_ALPHA, s.alpha)
    ctx.close()


def test_multi_step_tracks_oracle():
    """Ten fused steps: bit-identical sorts while positions stay bit-identical is not
    guaranteed, so compare particles by bornid with a loose bound."""
    sc = _scene("tait2")
    p = sc.params
    s = oracle_state(sc)
    O.before_first_step(p, s)
    ctx = device_ctx(sc)
    ctx.before_first_step()
    O.step(p, s, abi.SCHEDULE_FUSED, 10)
    ctx.step(10, abi.SCHEDULE_FUSED)
    ctx.sync()
    g = download_state(ctx)
    og = np.argsort(s.bornid)
    gg = np.argsort(g["bornid"])
    assert np.array_equal(s.bornid[og], g["bornid"][gg])
    fl = (s.type[og] == 0) & (s.mgcell[og] != UNDEF)
    assert field_err(g["pos"][gg][fl], s.pos[og][fl]) < 1e-5
    assert field_err(g["vel"][gg][fl], s.vel[og][fl]) < 1e-3
    ctx.close()


def test_conservation_fp64():
    sc = _scene("tait3")
    ctx = device_ctx(sc)
    ctx.before_first_step()
    ctx.step(2, abi.SCHEDULE_FUSED)
    c = ctx.conservation()
    g = download_state(ctx)
    f = in_grid_fluid(g)
    m = g["mass"][f].astype(np.float64)
    assert abs(c["mass"] - m.sum()) <= 1e-12 * m.sum()
    vol = (m * g["dens"][f].astype(np.float64)).sum()
    assert abs(c["volume"] - vol) <= 1e-9 * vol
    assert c["alpha_sum_err"] < 1e-5
    assert abs(sum(c["phase_volume"]) - c["volume"]) < 1e-5 * c["volume"]
    ctx.close()


def test_fp64_oracle_error():
    """FP32 density/force of the GPU against the FP64 oracle: no worse than the
    reference's own FP32 arithmetic plus a small margin."""
    sc = _scene("tait3")
    p = sc.params
    s32 = oracle_state(sc)
    O.before_first_step(p, s32)
    s64 = s32.copy(np.float64)
    ctx = device_ctx(sc)
    ctx.before_first_step()
    O.call("orc_compute_pressure", p, s32)
    O.call("orc_compute_pressure", p, s64)
    ctx.compute_pressure()
    O.call("orc_compute_force", p, s32)
    O.call("orc_compute_force", p, s64)
    ctx.compute_force()
    g = download_state(ctx)
    f = in_grid_fluid(s32)
    for k in ("dens", "accel"):
        e_gpu = field_err(g[k][f], getattr(s64, k)[f])
        e_ref = field_err(getattr(s32, k)[f], getattr(s64, k)[f])
        assert e_gpu <= max(4 * e_ref, 2e-7), (k, e_gpu, e_ref)
    ctx.close()


# ---------------------------------------------------------------------------
# edge cases
# ---------------------------------------------------------------------------

def test_grid_list_needs_keys_for_the_current_count():
    """GetGridList scatters every slot by the cell key and rank of GetParticleIndex:
    without keys for the current particle count it is refused, not run."""
    sc = _scene("tait2")
    ctx = device_ctx(sc)
    with pytest.raises(sphmp.SphmpError) as e:
        ctx.get_grid_list()
    assert e.value.status == abi.ERR_STATE
    ctx.get_particle_index()
    ctx.get_grid_list()
    n0 = sc.n - 100
    ctx.upload_aos(sc.disp[:n0], sc.calc[:n0])  # the count changed since the keys
    with pytest.raises(sphmp.SphmpError) as e:
        ctx.get_grid_list()
    assert e.value.status == abi.ERR_STATE
    ctx.close()


def test_sort_array_uploads_are_checked():
    """Caller-supplied sort arrays are indexed with on the device: border or
    out-of-range cell ids and negative or excess counts are refused."""
    sc, s, ctx = _sorted_pair("tait2")
    p = sc.params
    mgcell = ctx.download_field(abi.F_MGCELL).astype(np.uint32)
    ctx.upload_field(abi.F_MGCELL, mgcell)  # its own cells: accepted
    for bad in (0, p.gridres[0] - 1, p.gridtotal, p.gridtotal + 5):  # border cells, beyond the grid
        m = mgcell.copy()
        m[7] = bad
        with pytest.raises(sphmp.SphmpError) as e:
            ctx.upload_field(abi.F_MGCELL, m)
        assert e.value.status == abi.ERR_INVALID_ARG
    cnt = ctx.download_field(abi.F_MGRIDCNT).astype(np.int32)
    for k, v in ((3, -1), (5, sc.n + 1)):
        c2 = cnt.copy()
        c2[k] = v
        with pytest.raises(sphmp.SphmpError) as e:
            ctx.upload_field(abi.F_MGRIDCNT, c2)
        assert e.value.status == abi.ERR_INVALID_ARG
    ctx.close()


def test_empty_context():
    sc = _scene("tait2")
    p = sc.params.copy()
    p.num = 0
    ctx = sphmp.Context(p)
    ctx.upload_aos(sc.disp[:0], sc.calc[:0], 0)
    ctx.before_first_step()
    ctx.step(3, abi.SCHEDULE_FUSED)
    ctx.step(1, abi.SCHEDULE_REFERENCE)
    ctx.sync()
    assert ctx.n == 0
    assert ctx.download_field(abi.F_MGRIDCNT).sum() == 0
    ctx.close()


def test_two_particles():
    p = scenes.make_params(h=0.02, d=0.01, dt=1e-4, box_min=(0, 0, 0), box_max=(0.2, 0.2, 0.2), nphase=1,
                           dens=(1000.0,), visc=(0.2,), eos=abi.EOS_TAIT)
    disp, calc = sphmp.record_arrays(2)
    disp["pos"][0] = (0.1, 0.1, 0.1)
    disp["pos"][1] = (0.11, 0.1, 0.1)
    calc["mass"] = p.massArr[0]
    calc["restdens"] = 1000.0
    calc["visc"] = 0.2
    calc["bornid"] = [0, 1]
    calc["vel"][0] = (1.0, 0.2, 0.0)
    calc["vel"][1] = (-1.0, -0.2, 0.0)
    p.num = p.maxNum = 2
    sc = scenes.Scene(params=p, disp=disp, calc=calc, n_fluid=2, n_boundary=0)
    s = oracle_state(sc)
    O.before_first_step(p, s)
    O.call("orc_compute_pressure", p, s)
    O.call("orc_compute_force", p, s)
    ctx = device_ctx(sc)
    ctx.before_first_step()
    ctx.compute_pressure()
    ctx.compute_force()
    g = download_state(ctx)
    assert field_err(g["dens"], s.dens) < RTOL
    assert field_err(g["accel"], s.accel) < RTOL
    # symmetric pair: equal and opposite (viscous) accelerations
    assert abs(g["accel"][0, 0]) > 0
    assert np.all(np.abs(g["accel"][0] + g["accel"][1]) <= 1e-6 * np.abs(g["accel"][0]).max())
    ctx.close()


def test_out_of_grid_particles():
    """Particles on the outermost cell layer or outside the grid sort after every
    in-grid slot in their previous order and are parked at -1000 by the advance."""
    sc = _scene("tait2")
    p = sc.params
    disp = sc.disp.copy()
    rng = np.random.default_rng(9)
    idx = rng.choice(sc.n_fluid, 40, replace=False)
    lo = np.array(p.gridmin, np.float32)
    cell = np.float32(p.cellsize / p.simscale)
    disp["pos"][idx[:10]] = lo + 0.5 * cell                           # cell layer 0
    disp["pos"][idx[10:20]] = lo - 1.0                                # outside
    disp["pos"][idx[20:30], 1] = np.float32(p.gridmin[1] + p.gridsize[1]) - 0.25 * cell  # top layer
    disp["pos"][idx[30:40], 0] = np.float32(1e9)
    sc2 = scenes.Scene(params=p, disp=disp, calc=sc.calc, n_fluid=sc.n_fluid, n_boundary=sc.n_boundary)
    s = oracle_state(sc2)
    O.before_first_step(p, s)
    O.step(p, s, abi.SCHEDULE_FUSED, 2)
    ctx = device_ctx(sc2)
    ctx.before_first_step()
    ctx.step(2, abi.SCHEDULE_FUSED, use_graph=False)
    g = download_state(ctx)
    assert (s.mgcell == UNDEF).sum() >= 40
    for k in ("mgcell", "midsort", "mgridoff", "mgridcnt"):
        assert bits_equal(g[k], getattr(s, k)), k
    und = (s.mgcell == UNDEF) & (s.type == 0)
    assert np.all(g["pos"][und] == -1000.0)
    assert bits_equal(g["pos"][s.mgcell == UNDEF], s.pos[s.mgcell == UNDEF])
    ctx.close()


def _cell_interior(p, k, m, rng):
    """m points strictly inside grid cell (k, k, k)."""
    lo = np.array(p.gridmin, np.float32)
    cell = np.float32(p.cellsize / p.simscale)
    return (lo + (k + rng.uniform(0.05, 0.95, (m, 3))) * cell).astype(np.float32)


def test_big_cells_sorted_stably():
    """Cells with more members than one warp sorts (> 256) go through the CTA sort."""
    p = scenes.make_params(h=0.02, d=0.01, dt=1e-4, box_min=(0, 0, 0), box_max=(0.4, 0.4, 0.4), nphase=1,
                           dens=(1000.0,), visc=(0.2,), eos=abi.EOS_TAIT)
    n = 5000
    disp, calc = sphmp.record_arrays(n)
    rng = np.random.default_rng(4)
    disp["pos"][:3000] = _cell_interior(p, 5, 3000, rng)
    disp["pos"][3000:4000] = _cell_interior(p, 6, 1000, rng)
    disp["pos"][4000:] = rng.uniform(0.05, 0.35, (1000, 3)).astype(np.float32)
    disp["pos"] = disp["pos"][rng.permutation(n)]
    calc["mass"] = p.massArr[0]
    calc["restdens"] = 1000.0
    calc["visc"] = 0.2
    calc["bornid"] = np.arange(n)
    p.num = p.maxNum = n
    sc = scenes.Scene(params=p, disp=disp, calc=calc, n_fluid=n, n_boundary=0)
    s = oracle_state(sc)
    O.before_first_step(p, s)
    ctx = device_ctx(sc)
    ctx.before_first_step()
    g = download_state(ctx)
    assert s.mgridcnt.max() >= 3000
    for k in ("mgcell", "midsort", "mgridoff", "mgridcnt"):
        assert bits_equal(g[k], getattr(s, k)), k
    ctx.close()


def test_overfull_cell_is_reported():
    p = scenes.make_params(h=0.02, d=0.01, dt=1e-4, box_min=(0, 0, 0), box_max=(0.4, 0.4, 0.4), nphase=1,
                           dens=(1000.0,), visc=(0.2,), eos=abi.EOS_TAIT)
    n = 9000
    disp, calc = sphmp.record_arrays(n)
    disp["pos"] = _cell_interior(p, 5, n, np.random.default_rng(1))
    calc["mass"] = p.massArr[0]
    calc["restdens"] = 1000.0
    calc["visc"] = 0.2
    p.num = p.maxNum = n
    ctx = sphmp.Context(p)
    ctx.upload_aos(disp, calc)
    ctx.get_particle_index()
    ctx.get_grid_list()
    with pytest.raises(sphmp.SphmpError) as e:
        ctx.sync()
    assert e.value.status == abi.ERR_CELL_OVERFLOW
    ctx.close()


def test_upload_rejects_bad_records():
    sc = _scene("tait2")
    for mutate, code in [
        (lambda d, c: d["type"].__setitem__(3, 2), abi.ERR_UNSUPPORTED_TYPE),
        (lambda d, c: c["mass"].__setitem__(5, 0.0), abi.ERR_BAD_MASS),
        (lambda d, c: d["pos"].__setitem__(7, (np.nan, 0, 0)), abi.ERR_NOT_FINITE),
    ]:
        d, c = sc.disp.copy(), sc.calc.copy()
        mutate(d, c)
        ctx = sphmp.Context(sc.params)
        with pytest.raises(sphmp.SphmpError) as e:
            ctx.upload_aos(d, c)
        assert e.value.status == code
        ctx.close()
    ctx = sphmp.Context(sc.params)
    big_d, big_c = sphmp.record_arrays(sc.n + 1)
    with pytest.raises(sphmp.SphmpError) as e:
        ctx.upload_aos(big_d, big_c)
    assert e.value.status == abi.ERR_CAPACITY
    with pytest.raises(sphmp.SphmpError) as e:
        ctx.compute_force()  # no sort yet
    assert e.value.status == abi.ERR_STATE
    ctx.close()


def test_nan_particle_is_deleted_like_the_reference():
    sc = _scene("tait2")
    d = sc.disp.copy()
    d["pos"][10] = (np.nan, np.nan, np.nan)
    sc2 = scenes.Scene(params=sc.params, disp=d, calc=sc.calc, n_fluid=sc.n_fluid, n_boundary=sc.n_boundary)
    s = oracle_state(sc2)
    O.before_first_step(sc.params, s)
    ctx = sphmp.Context(sc.params)
    with pytest.raises(sphmp.SphmpError):
        ctx.upload_aos(d, sc.calc)  # reported, but the records are stored
    ctx.before_first_step()
    g = download_state(ctx)
    for k in ("mgcell", "midsort", "mgridcnt"):
        assert bits_equal(g[k], getattr(s, k)), k
    ctx.close()


def test_emit_appends_particles():
    sc = _scene("tait2")
    n0 = sc.n - 200
    p = sc.params
    s_full = oracle_state(sc)
    ctx = sphmp.Context(p)
    ctx.upload_aos(sc.disp[:n0], sc.calc[:n0])
    ctx.emit_aos(sc.disp[n0:], sc.calc[n0:], n0, sc.n)
    assert ctx.n == sc.n
    ctx.before_first_step()
    O.before_first_step(p, s_full)
    g = download_state(ctx)
    for k in ("mgcell", "midsort", "mgridoff", "mgridcnt"):
        assert bits_equal(g[k], getattr(s_full, k)), k
    assert np.array_equal(g["bornid"], s_full.bornid)
    ctx.close()


def test_aos_round_trip():
    sc = _scene("tait3")
    ctx = device_ctx(sc)
    d, c = ctx.download_aos()
    assert bits_equal(d["pos"], sc.disp["pos"])
    assert bits_equal(d["color"], sc.disp["color"])
    assert np.array_equal(d["type"], sc.disp["type"])
    for k in ("vel", "veleval", "restdens", "mass", "visc"):
        assert bits_equal(c[k], sc.calc[k]), k
    assert np.array_equal(c["bornid"], sc.calc["bornid"])
    ctx.close()


def test_surface_tension_matches_reference():
    sc = _scene("tait2")
    p = sc.params
    p.surface_tension = 1
    p.surfaceTensionK = 1.0
    p.surfaceTensionFluidC = 0.05
    s = oracle_state(sc)
    O.before_first_step(p, s)
    ctx = device_ctx(sc)
    ctx.set_params(p)
    ctx.before_first_step()
    O.call("orc_compute_pressure", p, s)
    O.call("orc_compute_force", p, s)
    O.call("orc_surface_tension", p, s)
    ctx.compute_pressure()
    ctx.compute_force()
    g = download_state(ctx)
    m = s.mgcell != UNDEF
    assert field_err(g["accel"][m], s.accel[m]) < RTOL
    ctx.close()
