"""The Morton (Z-order) cell order against the reference's linear order.

The cell key stays the reference's linear id (fluid_system_kern.cu:55); the
Morton order only changes the sequence of the cells in the sorted arrays. So,
after the same sort of the same upload: every cell holds the same particles in
the same order (its slice of midsort, its rank-in-cell entries and the sorted
positions are bit-identical, the counts equal), the cell offsets follow the
Z-order of the cells, and the physics of a step agrees with the linear order
(and with the oracle) within RTOL = 1e-5, particles matched by bornid.
"""
import numpy as np
import pytest

import sphmp
from helpers import bits_equal, device_ctx, download_state, field_err, in_grid_fluid, oracle_state
from oracle import oracle as O
from sphmp import abi, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _scene(kind):
    if kind == "tait3":
        return scenes.small_block(seed=12, n=(16, 10, 12), nphase=3, eos=abi.EOS_TAIT, velocity_scale=0.5)
    if kind == "dam":
        return scenes.dam_break_2phase(seed=15, n_side=16, box=0.32)
    return scenes.blobs_3phase(seed=3, lattice=(48, 24, 40))


def _ctx(sc, order):
    p = sc.params.copy()
    p.cell_order = order
    c = device_ctx(scenes.Scene(params=p, disp=sc.disp, calc=sc.calc, n_fluid=sc.n_fluid,
                                n_boundary=sc.n_boundary, name=sc.name))
    c.before_first_step()
    return c


def _morton(x, y, z):
    m = 0
    for b in range(21):
        m |= ((x >> b) & 1) << (3 * b) | ((z >> b) & 1) << (3 * b + 1) | ((y >> b) & 1) << (3 * b + 2)
    return m


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    sphmp.load()


@pytest.mark.parametrize("kind", ["tait3", "dam", "blobs"])
def test_same_cells_same_order(kind):
    sc = _scene(kind)
    lin, mor = _ctx(sc, abi.CELL_ORDER_LINEAR), _ctx(sc, abi.CELL_ORDER_MORTON)
    a, b = download_state(lin), download_state(mor)
    lin.close()
    mor.close()
    assert np.array_equal(a["mgridcnt"], b["mgridcnt"])
    cnt = a["mgridcnt"]
    occ = np.nonzero(cnt)[0]
    assert len(occ) > 10
    n_in = int(cnt.sum())
    for c in occ:
        la, lb = a["mgridoff"][c], b["mgridoff"][c]
        k = cnt[c]
        assert np.array_equal(a["midsort"][la:la + k], b["midsort"][lb:lb + k]), c
        assert np.array_equal(b["mgndx"][lb:lb + k], np.arange(k)), c
        assert np.all(b["mgcell"][lb:lb + k] == c), c
        assert bits_equal(a["pos"][la:la + k], b["pos"][lb:lb + k]), c
    # out-of-grid particles keep slot order after the cells in both orders
    assert np.array_equal(a["midsort"][n_in:], b["midsort"][n_in:])
    # the cells follow the Z-order of their grid coordinates in the Morton arrays
    rx, ry, rz = sc.params.gridres[0], sc.params.gridres[1], sc.params.gridres[2]
    gx, rest = occ % rx, occ // rx
    gz, gy = rest % rz, rest // rz
    codes = np.array([_morton(int(x), int(y), int(z)) for x, y, z in zip(gx, gy, gz)])
    assert np.array_equal(np.argsort(b["mgridoff"][occ], kind="stable"), np.argsort(codes, kind="stable"))
    assert not np.array_equal(a["midsort"], b["midsort"])  # the order does differ


def _by_bornid(g, k):
    return g[k][np.argsort(g["bornid"], kind="stable")]


@pytest.mark.parametrize("kind", ["tait3", "dam", "blobs"])
def test_step_matches_linear_order_and_oracle(kind):
    sc = _scene(kind)
    p = sc.params
    s = oracle_state(sc)
    O.before_first_step(p, s)
    O.step(p, s, abi.SCHEDULE_FUSED, 1)
    lin, mor = _ctx(sc, abi.CELL_ORDER_LINEAR), _ctx(sc, abi.CELL_ORDER_MORTON)
    for c in (lin, mor):
        c.step(1, abi.SCHEDULE_FUSED, use_graph=True)
        c.sync()
        assert c.device_errors() == 0
    a, b = download_state(lin), download_state(mor)
    lin.close()
    mor.close()
    o = {k: getattr(s, k) for k in ("bornid", "pos", "vel", "dens", "accel", "alpha", "mgcell", "type")}
    fa = _by_bornid(a, "mgcell") != abi.GRID_UNDEF
    fa &= _by_bornid(a, "type") == 0
    assert np.array_equal(_by_bornid(b, "mgcell") != abi.GRID_UNDEF, _by_bornid(a, "mgcell") != abi.GRID_UNDEF)
    for k in ("pos", "vel", "dens", "accel", "alpha"):
        fl = 1.0 if k == "alpha" else 0.0
        ref = _by_bornid(o, k)[fa]
        assert field_err(_by_bornid(b, k)[fa], _by_bornid(a, k)[fa], floor=fl) < RTOL, k
        assert field_err(_by_bornid(b, k)[fa], ref, floor=fl) < RTOL, k


def test_ten_steps_track_linear_order():
    sc = _scene("blobs")
    lin, mor = _ctx(sc, abi.CELL_ORDER_LINEAR), _ctx(sc, abi.CELL_ORDER_MORTON)
    for c in (lin, mor):
        c.step(10, abi.SCHEDULE_FUSED, use_graph=True)
        c.sync()
    a, b = download_state(lin), download_state(mor)
    lin.close()
    mor.close()
    f = (_by_bornid(a, "mgcell") != abi.GRID_UNDEF) & (_by_bornid(a, "type") == 0)
    for k in ("pos", "vel", "dens"):
        assert field_err(_by_bornid(b, k)[f], _by_bornid(a, k)[f]) < 1e-4, k


def test_sort_uploads_refused_in_morton_order():
    sc = _scene("tait3")
    mor = _ctx(sc, abi.CELL_ORDER_MORTON)
    with pytest.raises(sphmp.SphmpError) as e:
        mor.upload_field(abi.F_MIDSORT, np.arange(sc.n, dtype=np.uint32))
    assert e.value.status == abi.ERR_STATE
    mor.close()
