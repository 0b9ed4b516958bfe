"""CPU oracle of the learned large-step corrector. TEST INFRASTRUCTURE ONLY:
tests/ and bench.py's checks use it; the library never does.

The corrector has no counterpart in the reference (it is a method on top of the
reference's step), so this module restates the library's own definitions in
numpy, with the same rounding points. Parity unpinned by reference vectors
(none can exist); the restatement is checked on its own instead: its backward
pass against finite differences, its features against a hand-computed pair
(tests/test_learned_oracle.py).

* mlp_forward / mlp_backward: the network 48 -> 128 -> 128 -> 128 -> 4 with
  SiLU. Inputs (features - shift) * scale, weights, hidden activations and the
  backward's dY / dZ are rounded to bf16 (round to nearest even) where the GPU
  feeds them to the tensor cores; products are summed in float64 here (FP32 in
  TMEM on the GPU), and SiLU is exact here (the GPU's forward pass computes it
  as z/2 (1 + tanh(z/2)) with the hardware tanh), so the two agree to the
  accumulation rounding and an occasional bf16 rounding step of an activation.
  The forward pass saves z of each hidden layer in FP16 for the backward pass,
  which multiplies dH by SiLU'(z) of that saved value (rounded to FP16 here too).
  Loss = sum over the batch and the 4 outputs of (y - t)^2, divided by the batch.
* adam: one Adam step with bias correction (beta1 0.9, beta2 0.999, eps 1e-8).
* features: the 48 per-particle features of include/sphmp_learned.h's large
  step, from the state after the step's density pass.
"""
import numpy as np

FEATURES = 48
HIDDEN = 128
OUTPUTS = 4
PARAMS = 39812

_SHAPES = [("W1", (HIDDEN, FEATURES)), ("b1", (HIDDEN,)), ("W2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
           ("W3", (HIDDEN, HIDDEN)), ("b3", (HIDDEN,)), ("W4", (OUTPUTS, HIDDEN)), ("b4", (OUTPUTS,))]


def unpack(p):
    """Flat FP32 parameters -> dict of arrays (PyTorch Linear layout W [out][in])."""
    out, o = {}, 0
    for name, shape in _SHAPES:
        k = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + k], np.float32).reshape(shape)
        o += k
    assert o == PARAMS
    return out


def _unpack64(p):
    out, o = {}, 0
    for name, shape in _SHAPES:
        k = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + k], np.float64).reshape(shape)
        o += k
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float32).reshape(-1) for name, _ in _SHAPES])


def init_params(seed):
    """U(-1/sqrt(in), 1/sqrt(in)) weights and biases (PyTorch's Linear default)."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in _SHAPES:
        fan_in = shape[1] if name.startswith("W") else {"b1": FEATURES}.get(name, HIDDEN)
        bound = 1.0 / np.sqrt(fan_in)
        d[name] = rng.uniform(-bound, bound, size=shape).astype(np.float32)
    return pack(d)


def bf16(x):
    """Round float32 values to bf16 (nearest, ties to even), returned as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(np.shape(x))


_bf16 = bf16


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def mlp_forward(params, shift, scale, X, rnd=None):
    """Network outputs y [n][4] and the intermediates the backward pass needs.
    `rnd` replaces the bf16 rounding (identity for a finite-difference check)."""
    bf16 = _bf16 if rnd is None else rnd
    f32 = np.float32 if rnd is None else np.float64  # the exact mode keeps float64 throughout
    P = unpack(params) if rnd is None else _unpack64(params)
    x = bf16((np.asarray(X, f32) - f32(shift)) * f32(scale))
    W = [np.asarray(bf16(P[f"W{i}"]), np.float64) for i in range(1, 5)]
    b = [P[f"b{i}"].astype(np.float64) for i in range(1, 5)]
    hs, zs = [x.astype(np.float64)], []
    h = hs[0]
    for i in range(3):
        z = (h @ W[i].T + b[i]).astype(f32)
        zs.append(z)
        h = np.asarray(bf16(silu(z)), np.float64)
        hs.append(h)
    y = (h @ W[3].T + b[3]).astype(f32)
    return y, {"h": hs, "z": zs, "W": W}


def mlp_backward(params, shift, scale, X, T, rnd=None):
    """(flat gradients, loss) of loss = sum((y - t)^2) / batch."""
    bf16 = _bf16 if rnd is None else rnd
    f32 = np.float32 if rnd is None else np.float64
    B = X.shape[0]
    y, c = mlp_forward(params, shift, scale, X, rnd)
    d = (y - np.asarray(T, f32)).astype(f32)
    loss = float(np.sum(d.astype(np.float64) ** 2) / B)
    dy = bf16(f32(2.0 / B) * d).astype(np.float64)
    hs, zs, W = c["h"], c["z"], c["W"]
    g = {"W4": dy.T @ hs[3], "b4": dy.sum(0)}
    dz = dy
    for i in (3, 2, 1):  # layer i + 1 back to layer 1
        dh = dz @ W[i]  # W[i] is layer (i + 1)'s weight
        z = zs[i - 1]
        if rnd is None:  # the forward pass saves z in FP16
            z = np.asarray(z, np.float32).astype(np.float16).astype(np.float32)
        dz = bf16((dh.astype(f32) * silu_grad(z)).astype(f32)).astype(np.float64)
        g[f"W{i}"] = dz.T @ hs[i - 1]
        g[f"b{i}"] = dz.sum(0)
    g["W1"] = g["W1"][:, :FEATURES]
    return np.concatenate([np.asarray(g[name], f32).reshape(-1) for name, _ in _SHAPES]), loss


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    p = p - lr * (m / c1) / (np.sqrt(v / c2) + eps)
    return p.astype(np.float32), m, v


def features(pos, vel, dens, pres, alpha, restdens, g_minus_a, fluid, in_grid, nphase, h, ss, gravity, dt_large):
    """The 48 features of every particle (zeros where not fluid or not in the
    grid). Positions in simulation units (x simscale = metres); `dens` is rho
    (not its inverse); boundary particles take part as neighbours through
    fluid == False."""
    from scipy.spatial import cKDTree
    n = len(pos)
    x = np.asarray(pos, np.float64) * ss
    v = np.asarray(vel, np.float64)
    vs = np.sqrt(max(np.linalg.norm(gravity), 1e-3) * h)
    F = np.zeros((n, FEATURES))
    inn = np.flatnonzero(in_grid)
    tree = cKDTree(x[inn])
    a = np.zeros((n, 3))
    a[:, :nphase] = np.asarray(alpha, np.float64)[:, :nphase]
    rel = np.asarray(dens, np.float64) / np.asarray(restdens, np.float64)
    for i in np.flatnonzero(fluid & in_grid):
        ips = 1.0 / (restdens[i] * vs * vs)
        f = F[i]
        f[0:3] = v[i] / vs
        f[3] = rel[i] - 1
        f[4] = pres[i] * ips
        f[5:8] = a[i]
        f[8:11] = np.asarray(g_minus_a[i], np.float64) * dt_large / vs
        for jj in tree.query_ball_point(x[i], h):
            j = inn[jj]
            dx = x[i] - x[j]
            r2 = dx @ dx
            if not (0 < r2 < h * h):
                continue
            r = np.sqrt(r2)
            w = (1 - r2 / (h * h)) ** 3
            g = (1 - r / h) ** 2
            u = dx / r
            if not fluid[j]:
                f[40] += w
                f[41:44] += w * dx / h
                f[44] += 1 / 32
                continue
            dv = v[j] - v[i]
            f[11] += w
            f[12:15] += w * dx / h
            f[15:18] += w * dv / vs
            f[18] += w * (rel[j] - rel[i])
            f[19] += w * (pres[j] - pres[i]) * ips
            f[20:23] += w * (a[j] - a[i])
            f[23:29] += w * np.array([dx[0] * dx[0], dx[1] * dx[1], dx[2] * dx[2], dx[0] * dx[1], dx[0] * dx[2],
                                      dx[1] * dx[2]]) / (h * h)
            f[29:32] += g * u
            f[32] += g * (dv @ u) / vs
            f[33:36] += g * np.cross(dv, u) / vs
            f[36:39] += g * (pres[i] + pres[j]) * ips * u
            f[39] += 1 / 32
            f[45:48] += g * (a[j, 0] - a[i, 0]) * u
    return F.astype(np.float32)
