"""Batched scenes: independent scenes of uneven particle counts tiled into one
domain (sphmp.scenes.tile) run in one launch per pass. On the tiled input the
GPU matches the oracle within the parity tolerance (1e-5). Against each scene
run alone the inputs differ: tiled positions lie up to ~1 m from the origin,
where float32 resolves 6e-8 m, about 1e-5 of a 5 mm particle spacing, so that
comparison allows 20 float32 ulps of the largest coordinate per particle
spacing (1e-4 here) on top of the parity tolerance."""
import numpy as np
import pytest

import sphmp
from helpers import bits_equal, device_ctx, download_state, field_err, in_grid_fluid, oracle_state
from oracle import oracle as O
from sphmp import abi, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    sphmp.load()


def _state(ctx):
    d, c = ctx.download_aos()
    return {"pos": d["pos"].copy(), "vel": c["vel"].copy(), "dens": c["dens"].copy(), "accel": c["accel"].copy(),
            "alpha": ctx.download_field(abi.F_ALPHA).reshape(-1, 3), "bornid": c["bornid"].copy(),
            "type": d["type"].copy()}


def _solo_and_tiled():
    rng = np.random.default_rng(17)
    sizes = np.exp(rng.uniform(np.log(1500), np.log(9000), size=5)).astype(int)
    solo = [scenes.bubble_scene(seed=100 + i, n_particles=int(n)) for i, n in enumerate(sizes)]
    return solo, scenes.tile(solo)


def test_tiled_scenes_match_oracle():
    _, (big, _) = _solo_and_tiled()
    p = big.params
    s = oracle_state(big)
    O.before_first_step(p, s)
    ctx = device_ctx(big)
    ctx.before_first_step()
    O.step(p, s, abi.SCHEDULE_FUSED, 1)
    ctx.step(1, abi.SCHEDULE_FUSED, use_graph=False)
    ctx.sync()
    g = download_state(ctx)
    for k in ("mgcell", "midsort", "mgridoff", "mgridcnt"):
        assert bits_equal(g[k], getattr(s, k)), k
    f = in_grid_fluid(s)
    assert f.sum() == big.n_fluid
    for k in ("dens", "accel", "pos", "vel"):
        assert field_err(g[k][f], getattr(s, k)[f]) < RTOL, k
    assert field_err(g["alpha"][f][:, :2], s.alpha[f][:, :2], floor=1.0) < RTOL
    ctx.close()


def test_tiled_scenes_match_solo_runs():
    solo, (big, layout) = _solo_and_tiled()
    d = 0.01
    tol = RTOL + 20 * np.finfo(np.float32).eps * float(np.abs(big.disp["pos"]).max()) / d
    steps = 2
    ctx = sphmp.Context(big.params)
    ctx.upload_aos(big.disp, big.calc)
    ctx.before_first_step()
    ctx.step(steps, abi.SCHEDULE_FUSED, use_graph=True)
    ctx.sync()
    gb = _state(ctx)
    ctx.close()
    order = np.argsort(gb["bornid"])  # slot order changes with the sort; bornid is the upload index
    for i, sc in enumerate(solo):
        first, count, off = layout[i]
        c1 = sphmp.Context(sc.params)
        c1.upload_aos(sc.disp, sc.calc)
        c1.before_first_step()
        c1.step(steps, abi.SCHEDULE_FUSED, use_graph=True)
        c1.sync()
        g1 = _state(c1)
        c1.close()
        o1 = np.argsort(g1["bornid"])
        ob = order[first:first + count]
        assert np.array_equal(gb["bornid"][ob] - first, g1["bornid"][o1])
        f = g1["type"][o1] == 0
        assert field_err(gb["pos"][ob][f] - off, g1["pos"][o1][f]) < tol
        for k in ("vel", "dens", "accel"):
            assert field_err(gb[k][ob][f], g1[k][o1][f]) < tol, (i, k)
        assert field_err(gb["alpha"][ob][f][:, :2], g1["alpha"][o1][f][:, :2], floor=1.0) < tol


@pytest.mark.slow
def test_512_scenes_match_solo_runs():
    """The batched configuration at its size: 512 two-phase bubble scenes,
    particle counts log-uniform in [4096, 65536] (20.2 M particles, 11.2 M fluid),
    tiled into one domain and run three fused steps in one launch per pass; every
    scene against the same scene run alone (tolerance as above, from the largest
    tiled coordinate, about 9 m here)."""
    rng = np.random.default_rng(7)
    counts = np.floor(np.exp(rng.uniform(np.log(4096), np.log(65536), 512))).astype(int)
    solo = [scenes.bubble_scene(seed=7 * 100003 + i, n_particles=int(c)) for i, c in enumerate(counts)]
    big, layout = scenes.tile(solo)
    assert len(layout) == 512 and big.n_fluid > 10_000_000
    tol = RTOL + 20 * np.finfo(np.float32).eps * float(np.abs(big.disp["pos"]).max()) / 0.01
    steps = 3
    ctx = sphmp.Context(big.params)
    ctx.upload_aos(big.disp, big.calc)
    ctx.before_first_step()
    ctx.step(steps, abi.SCHEDULE_FUSED, use_graph=True)
    ctx.sync()
    assert ctx.device_errors() == 0
    gb = _state(ctx)
    ctx.close()
    order = np.argsort(gb["bornid"])
    worst = 0.0
    for i, sc in enumerate(solo):
        first, count, off = layout[i]
        c1 = sphmp.Context(sc.params)
        c1.upload_aos(sc.disp, sc.calc)
        c1.before_first_step()
        c1.step(steps, abi.SCHEDULE_FUSED, use_graph=False)
        c1.sync()
        g1 = _state(c1)
        c1.close()
        o1 = np.argsort(g1["bornid"])
        ob = order[first:first + count]
        assert np.array_equal(gb["bornid"][ob] - first, g1["bornid"][o1]), i
        f = g1["type"][o1] == 0
        errs = [field_err(gb["pos"][ob][f] - off, g1["pos"][o1][f])]
        errs += [field_err(gb[k][ob][f], g1[k][o1][f]) for k in ("vel", "dens", "accel")]
        errs.append(field_err(gb["alpha"][ob][f][:, :2], g1["alpha"][o1][f][:, :2], floor=1.0))
        worst = max(worst, max(errs))
        assert max(errs) < tol, (i, errs, tol)
    print(f"512 scenes: largest difference to the solo runs {worst:.2e} (tolerance {tol:.2e})")
