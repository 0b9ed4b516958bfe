"""sphmp_sort_cells_noalloc: the allocation-free cell sort against the context's
own sort (sphmp_get_particle_index + sphmp_get_grid_list) on the same keys.

The sort is integer work, so the tolerance is zero: every output must equal the
context path's bit for bit, on two calls in a row into buffers pre-filled with
garbage (the second call proves the static scratch is cleared per call). The
file is named to be collected last; it needs nothing from the other files.
"""
import ctypes as C

import numpy as np
import pytest

import sphmp
from sphmp import abi, scenes

UNDEF = 0xFFFFFFFF
MAX_N = 262144


def _lib():
    L = sphmp.load()
    fn = L.sphmp_sort_cells_noalloc
    fn.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def test_noalloc_rejects_sizes_beyond_its_scratch(built):
    fn = _lib()
    assert fn(None, MAX_N + 1, 100, None, None, None, None, None) == abi.ERR_CAPACITY
    assert "262144" in sphmp.last_error()
    assert fn(None, 10, MAX_N + 1, None, None, None, None, None) == abi.ERR_CAPACITY
    assert fn(None, -1, 100, None, None, None, None, None) == abi.ERR_CAPACITY


def _context_sort(sc, move_out):
    """Keys, then the context's sort outputs, for scene sc with some particles moved out of the grid."""
    ctx = sphmp.Context(sc.params)
    ctx.upload_aos(sc.disp, sc.calc)
    pos = ctx.download_field(abi.F_POS).reshape(-1, 3)
    pos[move_out] = (-7.0, 0.5, 0.5)          # far outside the grid: GRID_UNDEF
    ctx.upload_field(abi.F_POS, pos)
    ctx.get_particle_index()
    keys = ctx.download_field(abi.F_MGCELL).astype(np.uint32)
    ctx.get_grid_list()
    G = sc.params.gridtotal
    out = {
        "midsort": ctx.download_field(abi.F_MIDSORT).astype(np.uint32),
        "mgndx": ctx.download_field(abi.F_MGNDX).astype(np.uint32),
        "gridoff": ctx.download_field(abi.F_MGRIDOFF, G).astype(np.int32),
        "gridcnt": ctx.download_field(abi.F_MGRIDCNT, G).astype(np.int32),
    }
    ctx.close()
    return keys, out


@pytest.mark.gpu
@pytest.mark.parametrize("seed,shape,n_out", [(5, (12, 10, 8), 37), (9, (40, 30, 25), 1000)])
def test_noalloc_matches_context_sort_twice(built, seed, shape, n_out):
    import torch
    sc = scenes.small_block(seed=seed, n=shape, walls=True)
    n = sc.n
    rng = np.random.default_rng(seed)
    move_out = rng.choice(n, n_out, replace=False)
    keys, ref = _context_sort(sc, move_out)
    assert (keys == UNDEF).sum() >= n_out
    assert np.all((keys < sc.params.gridtotal) | (keys == UNDEF))
    G = sc.params.gridtotal
    dev = torch.device("cuda:0")
    d_keys = torch.from_numpy(keys.view(np.int32)).to(dev)
    fn = _lib()
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        outs = {
            "midsort": torch.full((n,), -0x54545455, dtype=torch.int32, device=dev),
            "mgndx": torch.full((n,), 12345, dtype=torch.int32, device=dev),
            "gridoff": torch.full((G,), -3, dtype=torch.int32, device=dev),
            "gridcnt": torch.full((G,), 77, dtype=torch.int32, device=dev),
        }
        torch.cuda.synchronize()
        st = fn(d_keys.data_ptr(), n, G, outs["midsort"].data_ptr(), outs["mgndx"].data_ptr(),
                outs["gridoff"].data_ptr(), outs["gridcnt"].data_ptr(), stream.cuda_stream)
        assert st == abi.OK, sphmp.last_error()
        for name, t in outs.items():
            got = t.cpu().numpy().view(np.uint32 if name in ("midsort", "mgndx") else np.int32)
            assert np.array_equal(got, ref[name]), (call, name)


def _noalloc_call(fn, keys, G, torch):
    """One call on device copies of `keys`; returns the status and the four outputs."""
    dev = torch.device("cuda:0")
    n = len(keys)
    d_keys = torch.from_numpy(keys.view(np.int32)).to(dev)
    outs = {
        "midsort": torch.full((max(n, 1),), -7, dtype=torch.int32, device=dev),
        "mgndx": torch.full((max(n, 1),), -7, dtype=torch.int32, device=dev),
        "gridoff": torch.full((G,), -3, dtype=torch.int32, device=dev),
        "gridcnt": torch.full((G,), 77, dtype=torch.int32, device=dev),
    }
    torch.cuda.synchronize()
    st = fn(d_keys.data_ptr(), n, G, outs["midsort"].data_ptr(), outs["mgndx"].data_ptr(),
            outs["gridoff"].data_ptr(), outs["gridcnt"].data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    got = {k: v.cpu().numpy()[:n if k in ("midsort", "mgndx") else G].view(
        np.uint32 if k in ("midsort", "mgndx") else np.int32) for k, v in outs.items()}
    return st, got


def _stable_sort_reference(keys, G):
    """GetGridListCUDA's outputs for `keys` from a stable sort (in-grid keys by cell,
    then GRID_UNDEF keys, each group in index order)."""
    order = np.argsort(keys.astype(np.uint64), kind="stable").astype(np.uint32)
    sk = keys[order]
    cnt = np.bincount(keys[keys != UNDEF].astype(np.int64), minlength=G).astype(np.int32)
    off = np.zeros(G, np.int32)
    off[1:] = np.cumsum(cnt)[:-1]
    off[cnt == 0] = 0
    ndx = np.full(len(keys), UNDEF, np.uint32)
    ing = sk != UNDEF
    starts = np.zeros(G + 1, np.int64)
    starts[1:] = np.cumsum(cnt)
    ndx[ing] = (np.arange(len(keys))[ing] - starts[sk[ing].astype(np.int64)]).astype(np.uint32)
    return {"midsort": order, "mgndx": ndx, "gridoff": off, "gridcnt": cnt}


@pytest.mark.gpu
def test_noalloc_at_its_limits_matches_a_stable_sort(built):
    """n = gridtotal = 262144 (the single-block scan runs 256 rounds, the serial
    chunk prefix 1024 entries), random keys with a tenth GRID_UNDEF, twice."""
    import torch
    fn = _lib()
    G = MAX_N
    rng = np.random.default_rng(11)
    keys = rng.integers(0, G, MAX_N).astype(np.uint32)
    keys[rng.random(MAX_N) < 0.1] = UNDEF
    ref = _stable_sort_reference(keys, G)
    for call in range(2):
        st, got = _noalloc_call(fn, keys, G, torch)
        assert st == abi.OK, sphmp.last_error()
        for name in ref:
            assert np.array_equal(got[name], ref[name]), (call, name)


@pytest.mark.gpu
def test_noalloc_rejects_a_key_that_is_not_a_cell(built):
    import torch
    fn = _lib()
    G = 1000
    keys = np.arange(500, dtype=np.uint32) % G
    keys[123] = G  # neither a cell id below gridtotal nor GRID_UNDEF
    st, _ = _noalloc_call(fn, keys, G, torch)
    assert st == abi.ERR_INVALID_ARG
    assert "neither a cell id nor GRID_UNDEF" in sphmp.last_error()
    # the next call with valid keys works and is exact
    keys[123] = UNDEF
    st, got = _noalloc_call(fn, keys, G, torch)
    assert st == abi.OK, sphmp.last_error()
    ref = _stable_sort_reference(keys, G)
    for name in ref:
        assert np.array_equal(got[name], ref[name]), name


@pytest.mark.gpu
def test_noalloc_rejects_a_cell_above_4096_members(built):
    import torch
    fn = _lib()
    G = 100
    rng = np.random.default_rng(12)
    keys = rng.integers(0, G, 6000).astype(np.uint32)
    keys[:4097] = 42
    rng.shuffle(keys)
    assert (keys == 42).sum() >= 4097
    st, _ = _noalloc_call(fn, keys, G, torch)
    assert st == abi.ERR_CELL_OVERFLOW
    assert "4096" in sphmp.last_error()
