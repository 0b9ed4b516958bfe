"""Host-side logic of the C ABI that needs no GPU: the library loads and exports
every declared symbol, the parameter derivation matches the oracle's
restatement of the reference bit for bit, the particle generators follow the
reference's lattice rules, and bad parameters are rejected before any device call."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import sphmp
from oracle import oracle as O
from sphmp import abi, scenes

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(built):
    return sphmp.load()


def _declared_symbols():
    names = set()
    for h in ("sphmp.h", "sphmp_legacy.h", "sphmp_learned.h"):
        src = open(os.path.join(REPO, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src):
            name = m.group(1)
            if name not in ("if", "sizeof", "defined") and not name.isupper():
                names.add(name)
    return names


def test_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert set(abi.EXPORTED_SYMBOLS) <= declared | {"CarryParam"}
    for name in declared:
        if name == "CarryParam":
            continue
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", sphmp.LIB_PATH], capture_output=True, text=True).stdout
    assert "_Z10CarryParamR12ParamCarrier" in out  # C++ linkage, as in the reference
    for name in abi.EXPORTED_SYMBOLS:
        assert re.search(rf"\bT {name}$", out, re.M), name


def test_version(lib):
    assert lib.sphmp_version().decode().startswith("sphmp")


@pytest.mark.parametrize("h,simscale,vmin,vmax", [
    (0.02, 1.0, (-0.1, -0.1, -0.1), (0.74, 0.9, 0.74)),
    (0.01, 1.0, (-0.05, -0.05, -0.05), (1.33, 0.99, 0.69)),
    (0.015, 0.005, (-60.0, -20.0, -60.0), (60.0, 200.0, 60.0)),   # SPH_Solver/scene.xml values
    (0.0123, 0.37, (-1.7, 0.3, -2.2), (3.1, 4.4, 2.9)),
])
def test_constants_and_grid_match_oracle(lib, h, simscale, vmin, vmax):
    p = sphmp.params_default()
    p.smoothradius = h
    p.simscale = simscale
    for a in range(3):
        p.volmin[a], p.volmax[a] = vmin[a], vmax[a]
    q = p.copy()
    sphmp.setup_constants(p)
    sphmp.setup_grid(p)
    O.setup_constants(q)
    O.setup_grid(q)
    assert bytes(p) == bytes(q)
    assert p.gridtotal == p.gridres[0] * p.gridres[1] * p.gridres[2]
    assert p.neighborid[13] == 0 and p.neighborid[14] == 1 and p.neighborid[16] == p.gridres[0]
    assert p.neighborid[22] == p.gridres[0] * p.gridres[2]


def test_wall_lattice_follows_reference(lib):
    p = scenes.make_params(h=0.02, d=0.01, dt=1e-4, box_min=(0, 0, 0), box_max=(0.2, 0.2, 0.2), nphase=1,
                           dens=(1000.0,), visc=(0.2,))
    s = sphmp.boundary_spacing(p)
    assert abs(s - 0.01) < 1e-6
    disp, calc = sphmp.record_arrays(10000)
    mn, mx = (0.0, -0.015, 0.0), (0.1, 0.0, 0.07)
    n = sphmp.add_wall(p, disp, calc, 0, mn, mx)
    cntx = int(np.ceil(np.float32(0.1) / np.float32(s)))
    cntz = int(np.ceil(np.float32(0.07) / np.float32(s)))
    ys = []
    y = np.float32(mn[1])
    while y <= np.float32(mx[1]):
        ys.append(y)
        y = np.float32(y + np.float32(s))
    assert n == len(ys) * cntx * cntz
    assert np.all(disp["type"][:n] == abi.TYPE_BOUNDARY)
    assert np.allclose(calc["mass"][:n], p.bmass) and np.all(calc["restdens"][:n] == np.float32(p.bRestdensity))
    assert np.array_equal(calc["bornid"][:n], np.arange(n))
    # x walks fastest, then z, then y
    assert disp["pos"][1, 0] > disp["pos"][0, 0] and disp["pos"][cntx, 2] > disp["pos"][0, 2]


def test_fluid_volume_lattice(lib):
    p = scenes.make_params(h=0.02, d=0.01, dt=1e-4, box_min=(0, 0, 0), box_max=(0.3, 0.3, 0.3), nphase=2,
                           dens=(1000.0, 1.2), visc=(0.2, 0.1))
    disp, calc = sphmp.record_arrays(5000)
    n = sphmp.add_fluid_volume(p, disp, calc, 0, (0.005, 0.005, 0.005), (0.05, 0.035, 0.065), 0.01, phase=1,
                               jitter=0.001, seed=3)
    # the reference loops `for (int y = 0; y < cnts.y; y++)` with cnts = (max - min) / spacing in float
    cnts = (np.array((0.05, 0.035, 0.065), np.float32) - np.float32(0.005)) / np.float32(0.01)
    c = [int(np.ceil(v)) for v in cnts]
    assert n == c[0] * c[1] * c[2]
    assert np.all(disp["type"][:n] == 0)
    assert np.all(calc["restdens"][:n] == np.float32(1.2)) and np.all(calc["visc"][:n] == np.float32(0.1))
    base = np.array([[x, y, z] for y in range(c[1]) for z in range(c[2]) for x in range(c[0])],
                    np.float32) * 0.01 + 0.005
    assert np.max(np.abs(disp["pos"][:n] - base)) <= 0.0005 + 1e-6
    # the same seed gives the same jitter; another seed does not
    d2, c2 = sphmp.record_arrays(5000)
    sphmp.add_fluid_volume(p, d2, c2, 0, (0.005, 0.005, 0.005), (0.05, 0.035, 0.065), 0.01, phase=1, jitter=0.001,
                           seed=3)
    assert np.array_equal(d2["pos"][:n], disp["pos"][:n])
    sphmp.add_fluid_volume(p, d2, c2, 0, (0.005, 0.005, 0.005), (0.05, 0.035, 0.065), 0.01, phase=1, jitter=0.001,
                           seed=4)
    assert not np.array_equal(d2["pos"][:n], disp["pos"][:n])


def test_generator_capacity_error(lib):
    p = scenes.make_params(h=0.02, d=0.01, dt=1e-4, box_min=(0, 0, 0), box_max=(0.3, 0.3, 0.3), nphase=1,
                           dens=(1000.0,), visc=(0.2,))
    disp, calc = sphmp.record_arrays(10)
    with pytest.raises(sphmp.SphmpError) as e:
        sphmp.add_fluid_volume(p, disp, calc, 0, (0, 0, 0), (0.1, 0.1, 0.1), 0.01)
    assert e.value.status == abi.ERR_CAPACITY


def test_compute_num_blocks(lib):
    """computeNumBlocks, SPH_Solver/fluids/fluid_system_host.cu:70-76."""
    fn = lib.computeNumBlocks
    fn.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    for npnt, mx, eb, et in [(1000, 384, 3, 384), (384, 384, 1, 384), (10, 384, 1, 10), (0, 384, 1, 1),
                             (385, 384, 2, 384)]:
        b, t = C.c_int(), C.c_int()
        fn(npnt, mx, C.byref(b), C.byref(t))
        assert (b.value, t.value) == (eb, et), (npnt, mx)


def test_params_validation_before_device(lib):
    sc = scenes.small_block(seed=1, n=(4, 4, 4), walls=False)
    cases = []
    p = sc.params.copy(); p.nphase = 4; cases.append((p, abi.ERR_INVALID_ARG))
    p = sc.params.copy(); p.maxNum = 0; cases.append((p, abi.ERR_INVALID_ARG))
    p = sc.params.copy(); p.num = p.maxNum + 1; cases.append((p, abi.ERR_CAPACITY))
    p = sc.params.copy(); p.gridtotal += 1; cases.append((p, abi.ERR_GRID))
    p = sc.params.copy(); p.gridres[0] = 2; cases.append((p, abi.ERR_GRID))
    p = sc.params.copy(); p.smoothradius = float("nan"); cases.append((p, abi.ERR_NOT_FINITE))
    p = sc.params.copy(); p.eos = 7; cases.append((p, abi.ERR_INVALID_ARG))
    for p, code in cases:
        with pytest.raises(sphmp.SphmpError) as e:
            sphmp.Context(p)
        assert e.value.status == code


def test_no_device_is_reported_not_hidden(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    sc = scenes.small_block(seed=1, n=(4, 4, 4), walls=False)
    with pytest.raises(sphmp.SphmpError) as e:
        sphmp.Context(sc.params)
    assert e.value.status == abi.ERR_NO_DEVICE


def test_legacy_calls_without_setup_report_errors(lib):
    lib.GetParticleIndexCUDA.argtypes = []
    lib.GetParticleIndexCUDA()  # prints "CUDA ERROR: ..." and returns, like the reference
    assert "FluidSetupCUDA" in sphmp.last_error()
    assert lib.sphmp_legacy_context() is None


def test_param_carrier_prefix_layout():
    """The first 464 bytes of sphmp_params are the reference ParamCarrier."""
    offs = {"num": 68, "dt": 76, "smoothradius": 100, "massArr": 108, "kpoly6": 148, "bmass": 168,
            "cellsize": 180, "neighborid": 192, "gridmin": 300, "gridIdfac": 336, "gridres": 348,
            "gridtotal": 360, "surfaceTensionK": 452, "fBlending": 460, "nphase": 464}
    for k, v in offs.items():
        assert getattr(abi.Params, k).offset == v, k


@pytest.mark.parametrize("header", ["sphmp.h", "sphmp_legacy.h", "sphmp_learned.h"])
@pytest.mark.parametrize("lang,std", [("c", "-std=c99"), ("c++", "-std=c++11")])
def test_headers_compile_as_c_and_cpp(header, lang, std):
    cc = "gcc" if lang == "c" else "g++"
    r = subprocess.run([cc, "-x", lang, std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                        os.path.join(REPO, "include"), os.path.join(REPO, "include", header)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_host_links_and_fails_loudly_without_a_device(lib, tmp_path):
    """A C++ host in the reference's shape links against the library; with no GPU,
    FluidSetupCUDA reports it and the program stops (no CPU fallback)."""
    import torch

    from helpers import build_c_host, write_c_host_inputs
    exe = build_c_host(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (tests/test_gpu_legacy.py runs the program)")
    sc = scenes.small_block(seed=3, n=(4, 4, 4), walls=False)
    args = write_c_host_inputs(tmp_path, sc)
    r = subprocess.run([exe, *args, str(sc.n), "1", str(tmp_path / "out.bin")], capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert "CUDA ERROR: FluidSetupCUDA" in r.stderr and "no CUDA device" in r.stderr



@pytest.mark.parametrize("build", ["dam_break", "blobs"])
def test_oracle_generators_build_the_library_scenes(lib, build):
    """The oracle's restated generators (used where the CUDA library must not be
    loaded: the benchmark's reference arm) give the library's records byte for byte."""
    from oracle import oracle as O
    if build == "dam_break":
        make = lambda gen: scenes.dam_break_2phase(seed=5, n_side=20, gen=gen)  # noqa: E731
    else:
        make = lambda gen: scenes.blobs_3phase(seed=6, lattice=(40, 16, 24), gen=gen)  # noqa: E731
    a, b = make(scenes.LIBRARY), make(O.Generators)
    assert bytes(a.params) == bytes(b.params)
    assert a.n == b.n and a.n_fluid == b.n_fluid
    assert a.disp.tobytes() == b.disp.tobytes()
    assert a.calc.tobytes() == b.calc.tobytes()


def test_tiled_scenes_stay_apart_with_unique_ids(lib):
    """sphmp.scenes.tile (the batched solver's layout, also the source of the
    corrector's training pairs): every scene keeps its records in order, moved by
    a whole number of grid cells, born ids renumbered to stay unique, and no two
    scenes' particles within two cells of each other."""
    solo = [scenes.bubble_scene(seed=s, n_particles=1500) for s in (1, 2, 3)]
    big, layout = scenes.tile(solo)
    p = big.params
    cell = float(p.cellsize) / float(p.simscale)
    assert big.n == sum(s.n for s in solo) and big.n_fluid == sum(s.n_fluid for s in solo)
    ids = big.calc["bornid"][:big.n]
    assert len(np.unique(ids)) == big.n
    boxes = []
    for s, (first, count, off) in zip(solo, layout):
        assert count == s.n
        frac = np.asarray(off, np.float64) / cell
        assert np.allclose(frac, np.round(frac), atol=1e-4)
        pos = big.disp["pos"][first:first + count]
        assert np.allclose(pos, s.disp["pos"][:s.n] + off, atol=1e-6)
        assert np.array_equal(big.calc["restdens"][first:first + count], s.calc["restdens"][:s.n])
        boxes.append((pos.min(axis=0), pos.max(axis=0)))
    for i in range(len(boxes)):
        for j in range(i + 1, len(boxes)):
            (alo, ahi), (blo, bhi) = boxes[i], boxes[j]
            gap = np.maximum(blo - ahi, alo - bhi)  # per axis; positive where the boxes are apart
            assert gap.max() >= 2 * cell - 1e-6
