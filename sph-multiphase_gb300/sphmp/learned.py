"""Training the learned large-step corrector from the plain solver's trajectories.

Host-side orchestration over the C ABI (include/sphmp_learned.h); device memory
for features and targets comes from torch. The pieces:

* generate_pairs: from states along a plain trajectory, the features of a large
  step (factor x dt) and its targets: the plain solver's result after `factor`
  steps against the uncorrected large step's, per particle (matched by bornid):
  the position difference over the large step's length (3, m/s) and the
  relative difference of the stored density.
* normalisation: feature shift / scale and output scale from the training set.
* train: Adam on random minibatches (the corrector's own tcgen05 kernels).
* step_errors: what one large step (corrected or not) misses against `factor`
  plain steps from the same state, densities recomputed at the final positions.
"""
import numpy as np

from . import Context, Corrector, abi


def _by_bornid(ctx):
    d = {k: ctx.download_field(f) for k, f in (("pos", abi.F_POS), ("dens", abi.F_DENS), ("bornid", abi.F_BORNID),
                                                ("type", abi.F_TYPE), ("mgcell", abi.F_MGCELL))}
    o = np.argsort(d["bornid"], kind="stable")
    return {k: v[o] for k, v in d.items()}


def zero_corrector():
    """A network whose outputs are all zero: its large step is the plain large
    step, with the features recorded."""
    return Corrector(0)


def generate_pairs(ctx, large, plain, factor, starts, gap):
    """Training pairs along the plain trajectory of `ctx` (advanced `gap` plain
    steps after each start). `large` and `plain` are scratch contexts with the
    same parameters. Returns (X torch [rows][48] on the device, T numpy [rows][4]
    physical targets)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    p = ctx.get_params()
    to_rate = np.float32(p.simscale) / np.float32(factor * p.dt)  # simulation units -> m/s over the step
    zero = zero_corrector()
    xs, ts = [], []
    for _ in range(starts):
        large.copy_state_from(ctx)
        plain.copy_state_from(ctx)
        large.step_large(factor, 1, zero)
        n = large.n
        feat = torch.empty((n, abi.LC_FEATURES), dtype=torch.float32, device=dev)
        ids = torch.empty(n, dtype=torch.int32, device=dev)
        rows = large.learned_features(feat, ids)
        plain.step(factor, abi.SCHEDULE_FUSED, use_graph=True)
        a, b = _by_bornid(plain), _by_bornid(large)
        ids_h = ids[:rows].cpu().numpy()
        keep = np.flatnonzero(ids_h >= 0)
        pa = np.searchsorted(a["bornid"], ids_h[keep])
        pb = np.searchsorted(b["bornid"], ids_h[keep])
        ok = (pa < len(a["bornid"])) & (pb < len(b["bornid"]))
        pa, pb, keep = pa[ok], pb[ok], keep[ok]
        ok = (a["bornid"][pa] == ids_h[keep]) & (b["bornid"][pb] == ids_h[keep]) & \
             (a["mgcell"][pa] != abi.GRID_UNDEF) & (b["mgcell"][pb] != abi.GRID_UNDEF)
        pa, pb, keep = pa[ok], pb[ok], keep[ok]
        t = np.empty((len(keep), 4), np.float32)
        t[:, :3] = (a["pos"][pa] - b["pos"][pb]) * to_rate
        t[:, 3] = b["dens"][pb] / a["dens"][pa] - 1.0  # stored inverses: rho_plain / rho_large - 1
        xs.append(feat[torch.from_numpy(keep).to(dev)])
        ts.append(t)
        ctx.step(gap, abi.SCHEDULE_FUSED, use_graph=True)
    zero.close()
    return torch.cat(xs), np.concatenate(ts)


def normalisation(X, T):
    """(feature shift, feature scale, output scale): standardised inputs and outputs."""
    x = X.double()
    mean = x.mean(0).cpu().numpy()
    std = x.std(0).cpu().numpy()
    scale = np.where(std > 1e-12, 1.0 / np.maximum(std, 1e-12), 1.0)
    ostd = T.astype(np.float64).std(0)
    out_scale = np.where(ostd > 0, ostd, 1.0)
    return mean.astype(np.float32), scale.astype(np.float32), out_scale.astype(np.float32)


def train(cor, X, T_net, steps, batch, lr, seed=0, log_every=0):
    """Adam on random minibatches of (X, T_net) (T_net in network units, a
    torch tensor on the device); returns [(step, loss)] every log_every steps."""
    import torch
    g = torch.Generator(device=X.device)
    g.manual_seed(seed)
    n = X.shape[0]
    log = []
    for k in range(steps):
        idx = torch.randint(0, n, (batch,), device=X.device, generator=g)
        xb = X[idx].contiguous()
        tb = T_net[idx].contiguous()
        want = log_every > 0 and (k % log_every == 0 or k == steps - 1)
        loss = cor.train_step(xb, tb, lr, want_loss=want)
        if want:
            log.append((k, loss))
    cor.sync()
    return log


def fit(params, ctx, factor, starts, gap, steps=400, batch=8192, lr=1e-3, seed=0, log_every=50):
    """Pairs along the plain trajectory of `ctx` (which advances starts x gap
    steps), normalisation, and a corrector trained on them; returns
    (corrector, training log, (X, T))."""
    import torch
    large, plain = Context(params), Context(params)
    try:
        X, T = generate_pairs(ctx, large, plain, factor, starts, gap)
    finally:
        large.close()
        plain.close()
    shift, scale, out_scale = normalisation(X, T)
    cor = Corrector(max_batch=batch)
    cor.set_params(init_params(seed))
    cor.set_normalisation(shift, scale, out_scale)
    T_net = torch.from_numpy(T / out_scale).to(X.device)
    log = train(cor, X, T_net, steps, batch, lr, seed, log_every)
    return cor, log, (X, T)


def init_params(seed):
    """U(-1/sqrt(in), 1/sqrt(in)) weights and biases (PyTorch's Linear default),
    the last layer scaled by 0.1 so that an untrained network corrects little."""
    rng = np.random.default_rng(seed)
    shapes = [(128, 48), (128,), (128, 128), (128,), (128, 128), (128,), (4, 128), (4,)]
    fans = [48, 48, 128, 128, 128, 128, 128, 128]
    out = []
    for i, (shape, fan) in enumerate(zip(shapes, fans)):
        b = 1.0 / np.sqrt(fan)
        a = rng.uniform(-b, b, size=shape).astype(np.float32)
        if i >= 6:
            a *= 0.1
        out.append(a.reshape(-1))
    p = np.concatenate(out)
    assert p.size == abi.LC_PARAMS
    return p


def step_errors(ctx, large, plain, factor, corrector=None):
    """From ctx's state: one large step (corrected when a corrector is given)
    against `factor` plain steps; densities recomputed at the final positions.
    Returns sphmp_compare_states' fields of the large step against the plain result."""
    large.copy_state_from(ctx)
    plain.copy_state_from(ctx)
    large.step_large(factor, 1, corrector)
    plain.step(factor, abi.SCHEDULE_FUSED, use_graph=False)
    for c in (large, plain):
        c.sort()
        c.compute_pressure()
    return large.compare_to(plain)
