"""Device-ref: the reference's own GPU kernels (SPH_Solver/fluids/fluid_system_kern.cu,
built unmodified for sm_103a by oracle/ref/build_ref_dev.sh and driven by
oracle/ref_gpu.py with the reference's launch sequence) against the oracle on
the same scene: the sort arrays bit for bit, positions, velocities and
densities within RTOL = 1e-5 over in-grid fluid slots. This checks the
device-ref harness before bench.py times it; skipped where the module was not
built (it needs the reference checkout at build time)."""
import numpy as np
import pytest

from helpers import bits_equal, device_ctx, download_state, field_err, in_grid_fluid, oracle_state
from oracle import oracle as O
from oracle import ref_gpu
from sphmp import abi, scenes

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(), reason="oracle/_ref/sph_ref_kern.cubin not built")]

RTOL = 1e-5


def _compare(R, s):
    d, c = R.records(abi.display_dtype(), abi.calc_dtype())
    srt = R.sort_arrays()
    for k in ("mgcell", "midsort", "mgridoff", "mgridcnt"):
        assert bits_equal(srt[k], getattr(s, k)), k
    m = s.mgcell != abi.GRID_UNDEF
    assert np.array_equal(srt["mgndx"][m], s.mgndx[m])
    f = in_grid_fluid(s)
    assert f.sum() > 500
    assert field_err(d["pos"][f], s.pos[f]) < RTOL
    assert field_err(c["vel"][f], s.vel[f]) < RTOL
    assert field_err(c["dens"][f], s.dens[f]) < RTOL


def test_device_ref_matches_oracle(built):
    sc = scenes.small_block(seed=81, n=(12, 10, 9), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.3, multiphase=0,
                            dens=(1000.0, 800.0, 900.0))
    p = sc.params
    calc = sc.calc[:sc.n].copy()
    bnd = sc.disp["type"][:sc.n] == abi.TYPE_BOUNDARY
    calc["accel"][bnd] = 0
    calc["pressure"][bnd] = 0
    R = ref_gpu.RefGPU(p, sc.disp[:sc.n], calc)
    s = oracle_state(sc)
    R.before_first_step()
    O.before_first_step(p, s)
    for _ in range(3):
        R.step(1)
        O.step(p, s, abi.SCHEDULE_REFERENCE, 1)
        _compare(R, s)
    R.close()


@pytest.mark.slow
def test_library_matches_device_ref_at_full_size(built):
    """The library against the reference's own GPU kernels on the benchmark lattice
    (1,048,576 fluid + 267,030 boundary particles) with the reference's Tait EOS and
    liquid phases: the first sort (GetParticleIndex .. RearrageData) bit for bit on
    every slot, then one RunSimpleSPH step in the reference call order: sort arrays
    bit for bit, densities, positions and velocities within RTOL."""
    sc = scenes.blobs_3phase(seed=2, eos=abi.EOS_TAIT, multiphase=0)
    gas = sc.calc["restdens"][:sc.n] == np.float32(sc.params.densArr[2])
    sc.calc["restdens"][:sc.n][gas] = sc.params.densArr[0]
    sc.calc["mass"][:sc.n][gas] = sc.params.massArr[0]
    p = sc.params
    calc = sc.calc[:sc.n].copy()
    bnd = sc.disp["type"][:sc.n] == abi.TYPE_BOUNDARY
    calc["accel"][bnd] = 0
    calc["pressure"][bnd] = 0
    R = ref_gpu.RefGPU(p, sc.disp[:sc.n], calc)
    R.before_first_step()
    ctx = device_ctx(sc)
    ctx.before_first_step()
    for step in range(2):
        srt = R.sort_arrays()
        g = download_state(ctx)
        for k in ("mgcell", "midsort", "mgridoff", "mgridcnt"):
            assert bits_equal(srt[k], g[k]), (step, k)
        if step == 1:
            d, c = R.records(abi.display_dtype(), abi.calc_dtype())
            f = in_grid_fluid(g)
            assert f.sum() > 1_000_000
            assert field_err(g["dens"][f], c["dens"][f]) < RTOL
            for k, ref in (("pos", d["pos"]), ("vel", c["vel"])):
                assert field_err(g[k][f], ref[f]) < RTOL, k
            break
        R.step(1)
        ctx.step(1, abi.SCHEDULE_REFERENCE, use_graph=False)
        ctx.sync()
    R.close()
    ctx.close()

