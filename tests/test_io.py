"""Particle data formats: the reference's text frame dump
(SPH_Solver/fluids/FluidIOUtility.cpp:17-38), its BINX-020 reader
(SPH_Solver/catpaw/BI2Reader.cpp:19-106) and shape import
(SPH_Solver/fluids/fluid_system.cpp:809-835), and the state checkpoint.

The expected outputs are restated here from those files: the frame text with
Python's %-formatting (the same conversions as C printf), .bi2 files written
field by field with `struct` in either byte order."""
import struct

import numpy as np
import pytest

import sphmp
from sphmp import abi, scenes


@pytest.fixture(scope="module", autouse=True)
def _lib(built):
    sphmp.load()


def test_frame_text_matches_reference_format(tmp_path):
    sc = scenes.small_block(seed=5, n=(5, 4, 3), nphase=2)
    path = tmp_path / "data_0000.txt"
    sphmp.write_frame_text(path, sc.disp, sc.calc)
    lines = path.read_text().splitlines()
    assert lines[0] == str(sc.n)
    for i in (0, 7, sc.n - 1):
        d, c = sc.disp[i], sc.calc[i]
        want = "%f %f %f %f %f %d" % (d["pos"][0], d["pos"][1], d["pos"][2], c["mass"], c["restdens"], d["type"])
        assert lines[1 + i] == want
    assert len(lines) == sc.n + 1


def _bi2_bytes(full, big, np_, nfixed, nmoving, nfloat, nfluidout, pos, vel, rhop, title=b"#File BINX-020 \0"):
    e = ">" if big else "<"
    out = title + bytes([20, 1 if big else 0, 1 if full else 0, 0])
    if full:
        out += struct.pack(e + "7f5if", 0.02, 0.01, 1.5, 1000.0, 7.0, 0.001, 0.002, np_, nfixed, nmoving, nfloat,
                           nfluidout, 0.25)
    else:
        out += struct.pack(e + "5if", np_, nfixed, nmoving, nfloat, nfluidout, 0.25)
    npok = np_ - nfluidout
    first = 0 if full else nfixed
    out += struct.pack(e + "%df" % (3 * (npok - first)), *pos[first:npok].ravel())
    out += struct.pack(e + "%df" % (3 * (npok - first)), *vel[first:npok].ravel())
    out += struct.pack(e + "%df" % npok, *rhop[:npok])
    return out


@pytest.mark.parametrize("full", [True, False], ids=["full", "short"])
@pytest.mark.parametrize("big", [False, True], ids=["little", "big"])
def test_bi2_reader(tmp_path, full, big):
    rng = np.random.default_rng(3)
    np_, nfixed, nmoving, nfloat, nout = 50, 12, 3, 2, 4
    pos = rng.normal(size=(np_, 3)).astype(np.float32)
    vel = rng.normal(size=(np_, 3)).astype(np.float32)
    rhop = rng.uniform(990, 1010, np_).astype(np.float32)
    path = tmp_path / "shape.bi2"
    path.write_bytes(_bi2_bytes(full, big, np_, nfixed, nmoving, nfloat, nout, pos, vel, rhop))
    info, p, v, r = sphmp.read_bi2(path)
    assert info["fmt"] == 20 and info["bitorder"] == (1 if big else 0) and info["full"] == int(full)
    assert (info["np"], info["nfixed"], info["nmoving"], info["nfloat"], info["nfluidout"]) == (np_, nfixed, nmoving,
                                                                                                  nfloat, nout)
    assert info["nbound"] == nfixed + nmoving + nfloat and info["nfluid"] == np_ - info["nbound"]
    assert info["time"] == np.float32(0.25)
    if full:
        assert info["h"] == np.float32(0.02) and info["dp"] == np.float32(0.01) and info["rhop0"] == 1000.0
    npok = np_ - nout
    first = 0 if full else nfixed
    assert np.array_equal(p[first:npok], pos[first:npok]) and np.array_equal(v[first:npok], vel[first:npok])
    assert np.array_equal(r[:npok], rhop[:npok])
    assert not p[npok:].any() and not p[:first].any() and not r[npok:].any()


def test_bi2_reader_rejects_bad_files(tmp_path):
    bad = tmp_path / "bad.bi2"
    bad.write_bytes(b"#File NOTBINX   " + bytes([20, 0, 2, 0]) + bytes(60))
    with pytest.raises(sphmp.SphmpError):
        sphmp.read_bi2(bad)
    short = tmp_path / "short.bi2"
    z = np.zeros((10, 3), np.float32)
    short.write_bytes(_bi2_bytes(True, False, 10, 0, 0, 0, 0, z, z, np.zeros(10, np.float32))[:-20])
    with pytest.raises(sphmp.SphmpError):
        sphmp.read_bi2(short)


def test_add_bi2_shape_follows_add_shape():
    p = scenes.make_params(h=0.02, d=0.01, dt=1e-4, box_min=(0, 0, 0), box_max=(1, 1, 1), nphase=3,
                           dens=(1000.0, 1.2, 800.0), visc=(0.2, 0.1, 0.3))
    pos = np.array([[0.001, 0.002, 0.003], [0.01, -0.02, 0.03]], np.float32)
    disp, calc = sphmp.record_arrays(10)
    n = sphmp.add_bi2_shape(p, disp, calc, 3, pos, offs=(1.0, 2.0, 3.0))
    assert n == 5
    for i in range(2):
        x, z, y = pos[i] / np.float32(0.005)
        assert np.array_equal(disp["pos"][3 + i], np.array([x + 1, y + 2, z + 3], np.float32))
    assert np.all(disp["type"][3:5] == abi.TYPE_FLUID)
    assert np.allclose(calc["vel"][3:5], [0, -1.5, 0])
    assert np.all(calc["restdens"][3:5] == np.float32(800.0)) and np.all(calc["visc"][3:5] == np.float32(0.3))
    assert np.array_equal(calc["bornid"][3:5], [3, 4])
    with pytest.raises(sphmp.SphmpError) as e:
        sphmp.add_bi2_shape(p, disp, calc, 9, pos)
    assert e.value.status == abi.ERR_CAPACITY


@pytest.mark.gpu
def test_checkpoint_continues_bit_for_bit(tmp_path):
    sc = scenes.small_block(seed=8, n=(14, 12, 10), nphase=3, eos=abi.EOS_TAIT, velocity_scale=0.3)
    a = sphmp.Context(sc.params)
    a.upload_aos(sc.disp, sc.calc)
    a.before_first_step()
    a.step(7, abi.SCHEDULE_FUSED, use_graph=True)
    path = tmp_path / "state.bin"
    a.save_state(path)
    b = sphmp.Context(sc.params)
    b.load_state(path)
    a.step(5, abi.SCHEDULE_FUSED, use_graph=True)
    b.step(5, abi.SCHEDULE_FUSED, use_graph=True)
    for f in (abi.F_POS, abi.F_VEL, abi.F_VELEVAL, abi.F_ALPHA, abi.F_DENS, abi.F_MGCELL, abi.F_MIDSORT):
        assert np.array_equal(a.download_field(f).view(np.uint32), b.download_field(f).view(np.uint32)), f
    a.close()
    b.close()
    wrong = sc.params.copy()
    wrong.nphase = 2
    c = sphmp.Context(wrong)
    with pytest.raises(sphmp.SphmpError):
        c.load_state(path)
    c.close()


@pytest.mark.gpu
def test_async_display_download_matches_sync():
    """Two contexts run the same steps; one downloads synchronously, the other
    through the asynchronous path into two alternating pinned buffers."""
    import torch
    sc = scenes.small_block(seed=9, n=(12, 10, 9), nphase=2, eos=abi.EOS_TAIT, velocity_scale=0.3)
    a = sphmp.Context(sc.params)
    b = sphmp.Context(sc.params)
    for ctx in (a, b):
        ctx.upload_aos(sc.disp, sc.calc)
        ctx.before_first_step()
    pinned = [torch.empty(sc.n * 32, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
    bufs = [t.numpy().view(abi.display_dtype()) for t in pinned]
    want = []
    for k in range(5):
        a.step(1, abi.SCHEDULE_FUSED, use_graph=True)
        want.append(a.download_aos(calc=False).copy())
    got = []
    for k in range(5):
        b.step(1, abi.SCHEDULE_FUSED, use_graph=True)
        b.download_display_async(bufs[k & 1])
        if k & 1:  # both buffers in flight: collect them
            b.download_wait()
            got += [bufs[0].copy(), bufs[1].copy()]
    b.download_wait()
    got.append(bufs[0].copy())
    for k in range(5):
        assert want[k].tobytes() == got[k].tobytes(), k
    a.close()
    b.close()


def test_emit_disk_follows_emit_particles():
    """EmitParticles (SPH_Solver/fluids/fluid_system.cpp:619-700): a disk normal to dir,
    two layers along +y, velocity dir * vel."""
    p = scenes.make_params(h=0.02, d=0.01, dt=1e-4, box_min=(0, 0, 0), box_max=(1, 1, 1), nphase=2,
                           dens=(1000.0, 800.0), visc=(0.2, 0.3))
    s, r = 0.01, 0.045
    disp, calc = sphmp.record_arrays(500)
    n = sphmp.emit_disk(p, disp, calc, 4, (0.5, 0.8, 0.5), (0, -1, 0), 1.0, r, s, layers=2, phase=1, frame=50,
                        jitter=0.0)
    res = int(np.float32(r) / np.float32(s))
    sites = [(i, j) for i in range(-res, res + 1) for j in range(-res, res + 1)
             if (np.float32(i * s)) ** 2 + (np.float32(j * s)) ** 2 <= np.float32(r) ** 2]
    assert n == 4 + 2 * len(sites)
    pos = disp["pos"][4:n]
    assert np.allclose(pos[:len(sites), 1], 0.8) and np.allclose(pos[len(sites):, 1], 0.81)
    assert np.allclose(np.sort(pos[:len(sites), 0] - 0.5), np.sort([i * s for i, _ in sites]), atol=1e-6)
    assert np.allclose(calc["vel"][4:n], [0, -1, 0]) and np.allclose(calc["veleval"][4:n], [0, -1, 0])
    assert np.allclose(disp["color"][4:n], [0.25, 0.5, 0.8, 0.5])
    assert np.all(calc["restdens"][4:n] == np.float32(800.0)) and np.all(calc["visc"][4:n] == np.float32(0.3))
    assert np.array_equal(calc["bornid"][4:n], np.arange(4, n))
    # a sideways emitter lays its disk in the plane normal to dir
    disp2, calc2 = sphmp.record_arrays(500)
    m = sphmp.emit_disk(p, disp2, calc2, 0, (0.3, 0.4, 0.5), (1, 0, 0), 2.0, r, s, layers=1, jitter=1.0, seed=7)
    assert m > 0 and np.all(disp2["pos"][:m, 0] == np.float32(0.3))
    assert np.all(np.sum((disp2["pos"][:m] - np.float32([0.3, 0.4, 0.5])) ** 2, axis=1) <= r * r * 1.0001)
    assert np.allclose(calc2["vel"][:m], [2, 0, 0])
    with pytest.raises(sphmp.SphmpError) as e:
        sphmp.emit_disk(p, disp2, calc2, 495, (0.3, 0.4, 0.5), (1, 0, 0), 2.0, r, s)
    assert e.value.status == abi.ERR_CAPACITY
