"""The IISPH step (RunIISPH, fluid_system.cpp:567-588; kernels
fluid_system_kern.cu:637-1115) on the GPU against the oracle's restatement,
which tests/test_oracle_pin.py pins bit for bit to the reference's own kernels.

Each pass runs on identical inputs on both sides after the same sort:
density (the density itself), PredictAdvection (veleval; d_ii and a_ii are
checked through the first iteration's acceleration and pressure), pressure
iterations (pressure, acceleration and both residues), and the integration.
Floating-point fields agree within RTOL = 1e-5 (max norm over in-grid fluid
slots; the GPU sums each cell in its own member order). The solver with its
stopping rule stops after the same number of iterations as the same rule on
the oracle.
"""
import numpy as np
import pytest

import sphmp
from helpers import device_ctx, download_state, field_err, in_grid_fluid, oracle_state, upload_state_fields
from oracle import oracle as O
from sphmp import abi, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _scene(kind):
    if kind == "liquids":
        return scenes.small_block(seed=51, n=(14, 12, 13), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.3,
                                  dens=(1000.0, 800.0), multiphase=0)
    return scenes.dam_break_2phase(seed=52, n_side=16, box=0.32, eos=abi.EOS_TAIT, multiphase=0)


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    sphmp.load()


def _pair(kind, start_pressure):
    sc = _scene(kind)
    p = sc.params
    s = oracle_state(sc)
    O.before_first_step(p, s)
    ctx = device_ctx(sc)
    ctx.before_first_step()
    if start_pressure:  # a pressure field to start the iterate from (p_l = p / 2)
        O.call("orc_compute_pressure", p, s)
        s.pressure *= 1e-3
        upload_state_fields(ctx, s, ["pressure"])
    ctx.sync()
    return sc, s, ctx


@pytest.mark.parametrize("start_pressure", [False, True], ids=["p0", "p_tait"])
@pytest.mark.parametrize("kind", ["liquids", "dam"])
def test_iisph_passes(kind, start_pressure):
    sc, s, ctx = _pair(kind, start_pressure)
    p = sc.params
    f = in_grid_fluid(s)
    O.call("orc_iisph_density", p, s)
    ctx.iisph_density()
    g = download_state(ctx)
    assert field_err(g["dens"][f], s.dens[f]) < RTOL
    O.call("orc_iisph_predict", p, s)
    ctx.iisph_predict_advection()
    g = download_state(ctx)
    assert field_err(g["veleval"][f], s.veleval[f]) < RTOL
    for it in range(3):
        ro = O.call("orc_iisph_iteration", p, s)
        rg = ctx.iisph_pressure_iteration()
        g = download_state(ctx)
        assert field_err(g["pressure"][f], s.pressure[f], floor=1e-3) < RTOL, it
        assert field_err(g["accel"][f], s.accel[f]) < RTOL, it
        assert abs(rg[0] - ro) <= RTOL * max(abs(ro), 1.0), (it, rg[0], ro)
        mabs = float(np.abs(s.residue[f].astype(np.float64)).mean())
        assert abs(rg[1] - mabs) <= RTOL * max(mabs, 1.0), (it, rg[1], mabs)
    O.call("orc_iisph_integrate", p, s)
    ctx.iisph_integrate()
    g = download_state(ctx)
    assert field_err(g["vel"][f], s.vel[f]) < RTOL
    assert field_err(g["pos"][f], s.pos[f]) < RTOL
    assert ctx.device_errors() == 0
    ctx.close()


def test_iisph_solve_stops_like_the_oracle():
    """The stopping rule (mean |residue| <= tol after at least min_iter, at most
    max_iter iterations) applied to the GPU iterates and to the oracle's: the same
    iteration counts, with a tolerance each side reaches and one neither does."""
    for tol, max_iter in ((1e9, 5), (1e-6, 4)):
        sc, s, ctx = _pair("liquids", False)
        p = sc.params
        f = in_grid_fluid(s)
        O.call("orc_iisph_density", p, s)
        O.call("orc_iisph_predict", p, s)
        it_o = 0
        while it_o < max_iter:
            O.call("orc_iisph_iteration", p, s)
            it_o += 1
            if it_o >= 2 and float(np.abs(s.residue[f].astype(np.float64)).mean()) <= tol:
                break
        ctx.iisph_density()
        ctx.iisph_predict_advection()
        it_g, r = ctx.iisph_pressure_solve(tol, 2, max_iter)
        assert it_g == it_o, (tol, it_g, it_o)
        ctx.close()


def test_iisph_whole_step_tracks_the_oracle():
    """One whole IISPH step (sort, density, PredictAdvection, four iterations,
    integration) on both sides from the same start. (The reference's iteration
    diverges on these scenes, so rounding differences grow by orders of magnitude
    within a second step; the passes above hold on identical inputs.)"""
    sc, s, ctx = _pair("liquids", False)
    p = sc.params
    for _ in range(1):
        for st in ("orc_get_particle_index", "orc_get_grid_list", "orc_rearrange_data"):
            O.call(st, p, s)
        O.call("orc_iisph_density", p, s)
        O.call("orc_iisph_predict", p, s)
        for _ in range(4):
            O.call("orc_iisph_iteration", p, s)
        O.call("orc_iisph_integrate", p, s)
    its, _ = ctx.step_iisph(1, tol=0.0, max_iter=4)
    assert its == [4]
    g = download_state(ctx)
    ctx.close()
    og = np.argsort(g["bornid"], kind="stable")
    oo = np.argsort(s.bornid, kind="stable")
    f = in_grid_fluid(s)[oo] & in_grid_fluid(g)[og]
    assert f.sum() > 0.9 * sc.n_fluid
    assert field_err(g["pos"][og][f], s.pos[oo][f]) < RTOL
    assert field_err(g["vel"][og][f], s.vel[oo][f]) < RTOL
