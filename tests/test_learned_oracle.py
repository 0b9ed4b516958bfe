"""The CPU oracle of the learned corrector (oracle/learned.py) checked on its own:
bf16 rounding, the parameter layout, the backward pass against finite
differences, the features on a hand-computed pair; and the corrector's C ABI
on a machine without a GPU (argument checks before any device use, loud
failure instead of a fallback). No GPU."""
import ctypes as C

import numpy as np
import pytest

from oracle import learned as OL
from sphmp import abi


def test_parameter_layout_matches_the_header():
    assert OL.PARAMS == abi.LC_PARAMS == 48 * 128 + 128 + 2 * (128 * 128 + 128) + 4 * 128 + 4
    p = OL.init_params(1)
    assert p.dtype == np.float32 and p.shape == (OL.PARAMS,)
    d = OL.unpack(p)
    assert d["W1"].shape == (128, 48) and d["W4"].shape == (4, 128) and d["b4"].shape == (4,)
    assert np.array_equal(OL.pack(d), p)
    assert np.abs(d["W1"]).max() <= 1 / np.sqrt(48) and np.abs(d["W2"]).max() <= 1 / np.sqrt(128)


def test_bf16_rounds_to_nearest_even():
    e = 2.0 ** -7  # bf16 spacing just above 1
    x = np.array([1.0, 1 + e / 2, 1 + 1.5 * e, 1 + 0.75 * e, -3.0, 0.0, 1e-30, 65504.0], np.float32)
    want = np.array([1.0, 1.0, 1 + 2 * e, 1 + e, -3.0, 0.0, None, None], object)
    got = OL.bf16(x)
    for g, w in zip(got[:6], want[:6]):
        assert g == np.float32(w)
    # every result has a zero low half
    assert np.all(got.view(np.uint32) & 0xFFFF == 0)
    assert abs(got[6] - 1e-30) / 1e-30 < 2 ** -8


def test_bf16_rounding_agrees_with_torch():
    import torch
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.standard_normal(100000).astype(np.float32) * 10.0 ** rng.integers(-20, 20, 100000),
                        np.array([0.0, -0.0, 1.0, 3.0e38, -1e-39], np.float32)]).astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(OL.bf16(x).view(np.uint32), ref.view(np.uint32))


def test_normalisation_standardises_inputs_and_outputs():
    import torch
    from sphmp import learned as SL
    rng = np.random.default_rng(10)
    X = torch.from_numpy((rng.standard_normal((5000, 48)) * 3 + 2).astype(np.float32))
    X[:, 7] = 0.0  # a constant feature (a phase that is absent): scale 1, not infinity
    T = (rng.standard_normal((5000, 4)) * [1e-4, 2e-4, 3e-4, 1e-2]).astype(np.float32)
    shift, scale, osc = SL.normalisation(X, T)
    Z = (X.numpy() - shift) * scale
    assert np.allclose(Z.mean(0), 0, atol=1e-4) and np.allclose(np.delete(Z.std(0), 7), 1, atol=1e-3)
    assert scale[7] == 1 and np.all(np.isfinite(scale))
    assert np.allclose(osc, T.std(0), rtol=1e-5)
    p = SL.init_params(3)
    assert p.shape == (abi.LC_PARAMS,) and np.abs(OL.unpack(p)["W4"]).max() <= 0.1 / np.sqrt(128)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(4)
    p = OL.init_params(5).astype(np.float64)
    X = rng.standard_normal((6, 48))
    T = rng.standard_normal((6, 4))
    ident = lambda a: np.asarray(a, np.float64)
    shift, scale = np.zeros(48), np.ones(48)
    g, loss = OL.mlp_backward(p, shift, scale, X, T, rnd=ident)

    def L(q):
        return OL.mlp_backward(q, shift, scale, X, T, rnd=ident)[1]

    idx = rng.choice(OL.PARAMS, 60, replace=False)
    idx = np.concatenate([idx, [OL.PARAMS - 1, OL.PARAMS - 5, 6144, 0]])  # b4, W4's last row, b1, W1
    eps = 1e-3
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp = L(q)
        q[i] -= 2 * eps
        lm = L(q)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 2e-3 * max(1e-2, abs(fd)), (i, fd, g[i])


def test_gpu_rounding_mode_stays_close_to_exact_gradients():
    """The oracle's GPU-rounding mode (bf16 operands, z saved in FP16, as the
    library's training kernels compute) against the exact float64 gradients of
    the same network: every parameter tensor within 2 % in norm, so the FP16
    save and the bf16 operands change the descent direction only slightly."""
    rng = np.random.default_rng(9)
    p = OL.init_params(6)
    X = rng.standard_normal((512, 48)).astype(np.float32)
    T = rng.standard_normal((512, 4)).astype(np.float32)
    shift, scale = np.zeros(48, np.float32), np.ones(48, np.float32)
    ident = lambda a: np.asarray(a, np.float64)
    g_gpu, l_gpu = OL.mlp_backward(p, shift, scale, X, T)
    g_ex, l_ex = OL.mlp_backward(p.astype(np.float64), shift, scale, X, T, rnd=ident)
    assert abs(l_gpu - l_ex) <= 1e-4 * l_ex
    G, R = OL.unpack(g_gpu), OL.unpack(g_ex.astype(np.float32))
    for k in R:
        assert np.linalg.norm(G[k] - R[k]) <= 1e-2 * np.linalg.norm(R[k]), k


def test_adam_first_step_moves_each_parameter_by_lr():
    p = np.zeros(5, np.float32)
    g = np.array([1.0, -2.0, 0.5, 1e-3, -1e-6], np.float32)
    q, m, v = OL.adam(p, g, np.zeros(5), np.zeros(5), 1, 1e-3)
    # bias-corrected first step: m/c1 = g, v/c2 = g^2
    assert np.allclose(q, -1e-3 * g / (np.abs(g) + 1e-8), rtol=1e-5)


def test_features_of_a_pair():
    h, ss = 0.02, 1.0
    pos = np.array([[0.1, 0.1, 0.1], [0.1 + 0.01, 0.1, 0.1], [0.1, 0.1 + 0.015, 0.1]], np.float32)
    vel = np.array([[0.0, 0.0, 0.0], [0.2, 0.0, 0.0], [0.0, 0.0, 0.0]], np.float32)
    dens = np.array([1000.0, 1010.0, 1.0], np.float32)
    pres = np.array([1.0, 3.0, 0.0], np.float32)
    alpha = np.array([[1, 0, 0], [0.5, 0.5, 0], [0, 0, 0]], np.float32)
    rest = np.array([1000.0, 1000.0, 1000.0], np.float32)
    gma = np.zeros((3, 3), np.float32)
    fluid = np.array([True, True, False])
    F = OL.features(pos, vel, dens, pres, alpha, rest, gma, fluid, np.ones(3, bool), 2, h, ss, (0, -9.81, 0), 8e-4)
    vs = np.sqrt(9.81 * h)
    r = 0.01
    w = (1 - (r / h) ** 2) ** 3
    g = (1 - r / h) ** 2
    f = F[0]
    assert np.isclose(f[11], w) and np.isclose(f[12], w * (-0.01) / h)
    assert np.isclose(f[15], w * 0.2 / vs)
    assert np.isclose(f[18], w * 0.01) and np.isclose(f[20], -0.5 * w) and np.isclose(f[21], 0.5 * w)
    assert np.isclose(f[29], -g) and np.isclose(f[32], g * (0.2 * -1) / vs)
    assert np.isclose(f[39], 1 / 32) and np.isclose(f[44], 1 / 32)
    rb = 0.015
    assert np.isclose(f[40], (1 - (rb / h) ** 2) ** 3)
    assert np.all(F[2] == 0)  # boundary particles carry no features


def _no_gpu():
    import torch
    return not torch.cuda.is_available()


@pytest.mark.skipif(not _no_gpu(), reason="checks the behaviour without a GPU")
def test_corrector_abi_without_a_device(built):
    import sphmp
    L = sphmp.load()
    out = C.c_void_p()
    # argument errors come first, then the missing device; nothing falls back to the CPU
    assert L.sphmp_corrector_create(100, None, C.byref(out)) == abi.ERR_INVALID_ARG
    assert L.sphmp_corrector_create(128, None, C.byref(out)) == abi.ERR_NO_DEVICE and not out.value
    assert L.sphmp_corrector_create(128, None, None) == abi.ERR_INVALID_ARG
    with pytest.raises(sphmp.SphmpError) as e:
        sphmp.Corrector(128)
    assert e.value.status == abi.ERR_NO_DEVICE
    for m, n, k in [(128, 24, 64), (128, 144, 64), (128, 32, 12), (0, 32, 64)]:
        assert L.sphmp_gemm_bf16_tn(C.c_void_p(16), 64, C.c_void_p(16), 64, C.c_void_p(16), m, n, k, 1,
                                    None) == abi.ERR_INVALID_ARG
    assert L.sphmp_step_large(None, None, 8, 1) == abi.ERR_INVALID_ARG
    assert L.sphmp_copy_state(None, None) == abi.ERR_INVALID_ARG
    assert L.sphmp_rollout(None, None, None, 8, 16, 16, 0.01, None) == abi.ERR_INVALID_ARG
    assert L.sphmp_compare_states(None, None, None, 5) == abi.ERR_INVALID_ARG
