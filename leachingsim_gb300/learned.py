"""The learned warm start of the pressure solve.

The network (the U-shaped 3D convolutional network of ls_lpnet_*, hand-written CUDA
kernels for its forward and backward passes and Adam) maps three fields of an assembled
pressure system to a start for the solve:

    mask  - 1 on the Pore rows (the unknowns), 0 elsewhere
    logk  - (log10 K + 15) / 3
    dist  - the Euclidean distance to the nearest voxel that carries the top pressure
            (ls_geom_distance on the half-resolution grid), over 100: the pressure of the
            Pore space falls off with it, on scales beyond the network's receptive field

and predicts the deviation of the pressure from the top pressure, d = 100 (1 - P / p_top),
on the Pore rows (the start is P / p_top = 1 - d / 100). The network runs at half
resolution: its inputs are the 2x2x2 block means of the mask and the log-permeability
(ls_field_pool2) and the distance computed on the half-resolution grid, its output is
repeated over each block (ls_field_up2); the deviation varies on the scale of
the distance to the inlet, and the half-resolution network costs an eighth of the
full-resolution one. The pressure of the Pore space
that the Air inlet reaches sits within a few percent of p_top, so this scaling gives the
network targets of order one. The loss covers the Pore voxels of the components anchored
to the inlet only: elsewhere the system is singular or nearly so, the solver keeps the
zero start's value, and what the network says there is discarded (the solver zeroes a
supplied start on unanchored components). It is trained only on solutions of the plain
solver (mixed-precision multigrid FCG with FP64 refinement) on seeded synthetic
geometries with porosity 0.15-0.40, correlation length 2-10 and mineral fraction
0.05-0.30, Air inlet planes as in the workload: 16 solves of 288 x 256 x 256 (the
workload's depth), each cut into 16 columns of 288 x 64 x 64. How far the pressure falls
depends on the Pore space behind and beside a voxel, which small domains of their own do
not show (96^3 patches, or narrow columns solved alone, train networks that help less at
the workload's size). At use, the start goes through
ls_pressure_solve_start: the FP64 refinement rescales it once by its minimal-residual
factor when that lowers the residual, judges it by the FP64 residual and finishes the
solve with the plain solver, so a poor start costs iterations, never accuracy.

    python -m leachingsim_gb300.learned train --samples 256 --epochs 64 --lr 2e-3 --seed 0

writes lpnet_weights.npy beside this file (the weights shipped here were made so).
"""
import argparse
import json
import math
import os
import sys
import time

import numpy as np

from . import _abi
from .geometry import grf_geometry

PATCH = (288, 64, 64)   # training crops (fine voxels)
WIDE = (288, 256, 256)   # the solves the crops are cut from
CROPS = 16               # crops per solve
DEV_SCALE = 100.0   # network output d = DEV_SCALE (1 - P / p_top)
DIST_SCALE = 100.0  # the distance input is dist / DIST_SCALE
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lpnet_weights.npy")
RAMP = 3600.0  # the top-pressure ramp of src/Simulation.cpp:662-670


def pad8(shape):
    return tuple(((int(v) + 7) // 8) * 8 for v in shape)


def pad16(shape):
    """The fine grid of the learned start: multiples of 16, so that the half-resolution
    network's grid is a multiple of 8."""
    return tuple(((int(v) + 15) // 16) * 16 for v in shape)


def coarse_inputs(m, k, bc):
    """The network's inputs from the fine fields (extents even): 2x2x2 block means of the
    mask and the log-permeability, and the distance input computed on the half-resolution
    grid itself (coarse_distance_input): an eighth of the work of a fine distance transform
    and within a voxel of the block mean of the fine distances."""
    from .runtime import field_pool2
    return field_pool2(m), field_pool2(k), coarse_distance_input(bc)


def top_pressure(params, t):
    """The effective (ramped) top pressure of the system assembled at time t."""
    top = params.top_pressure
    return top * (t / RAMP) + 1e-6 if t < RAMP else top


def solver_params(**kw):
    base = dict(c_sat=1.0, press_solver=_abi.PRESS_MIXED, press_rtol=1e-8)
    base.update(kw)
    return _abi.default_params(**base)


def patch_geometry(seed, shape=PATCH):
    """A seeded percolating patch with random porosity, correlation length and mineral
    fraction (parameters redrawn while a draw finds no percolating field)."""
    rng = np.random.default_rng(seed)
    for _ in range(32):
        por = rng.uniform(0.15, 0.40)
        corr = rng.uniform(2.0, 10.0)
        mineral = rng.uniform(0.05, 0.30)
        try:
            lab, used = grf_geometry(shape, porosity=por, corr_len=corr, mineral_fraction=mineral,
                                     seed=int(rng.integers(1 << 30)), air_inlet=True, max_tries=8)
        except RuntimeError:
            continue
        return lab, {"porosity": por, "corr_len": corr, "mineral_fraction": mineral, "seed": used}
    raise RuntimeError(f"no percolating patch from seed {seed}")


def _solution(ctx):
    """x of the last pressure solve (the P slots, shifted by one plane in the reference's
    write-back convention)."""
    Pp = ctx.download("pressure", padded=True).ravel()
    sh = ctx.J * ctx.K if ctx.params.compat_shift else 0
    return Pp[sh:sh + ctx.N].reshape(ctx.shape)


def make_sample(seed, shape=PATCH, t=RAMP, params=None):
    """One training sample from the plain solver, at the network's half resolution: the
    inputs (3 fields), the target d = DEV_SCALE (1 - P / p_top) averaged over the anchored
    Pore voxels of each block, and the loss mask (the blocks holding any)."""
    import torch
    from .runtime import Context
    params = params or solver_params()
    lab, meta = patch_geometry(seed, shape)
    ctx = Context(shape, params=params)
    try:
        ctx.upload("label", lab)
        ctx.init_all()
        ctx.props()
        ctx.pressure_setup(t)
        m, k, b = ctx.pressure_learned_inputs()
        ok, info = ctx.pressure_solve_start(torch.zeros(shape, dtype=torch.float32, device="cuda"), 0.0)
        if not ok:
            raise RuntimeError(f"plain solve failed on sample {seed}: {info}")
        tau = torch.from_numpy(np.ascontiguousarray(_solution(ctx) / top_pressure(params, t),
                                                    dtype=np.float32)).cuda()
        # the components anchored to the inlet: Pore voxels the solution lifted off the zero
        # start (the others keep 0)
        anchored = m * (tau > 0.5).float()
        target = DEV_SCALE * (1.0 - tau) * anchored
        from .runtime import field_pool2
        fs = pad16(shape)
        m, k, b, target, anchored = (_pad(v, fs) for v in (m, k, b, target, anchored))
        mc, kc, dc = coarse_inputs(m, k, b)
        tc = field_pool2(target, anchored)                   # mean over the anchored voxels
        ac = (field_pool2(anchored) > 0.0).float()           # blocks holding any
    finally:
        ctx.close()
    return (mc, kc, dc, tc, ac), dict(meta, iterations=info["iterations"],
                                      anchored=float(anchored.sum() / max(float(m.sum()), 1.0)))


def make_crops(seed, shape=WIDE, crop=PATCH, count=CROPS, t=RAMP, params=None):
    """Training samples cut from one wide solve: the plain solver on a seeded geometry of
    `shape`, the fields and target at half resolution, and `count` random crops of
    half of `crop` (a crop of a wide domain carries the pressure drop of the wide domain,
    which a narrow domain of its own would not)."""
    full, meta = make_sample(seed, shape, t, params)
    rng = np.random.default_rng(seed ^ 0x5EED)
    cs = tuple(v // 2 for v in pad16(crop))
    fs = full[0].shape
    out = []
    for _ in range(count):
        o = [int(rng.integers(0, fs[a] - cs[a] + 1)) for a in range(3)]
        sl = tuple(slice(o[a], o[a] + cs[a]) for a in range(3))
        out.append(tuple(v[sl].contiguous() for v in full))
    return out, meta


def coarse_distance_input(bc):
    """The third input, on the half-resolution grid: the distance (in fine voxels) from each
    2x2x2 block to the nearest block holding a voxel that carries the top pressure, over
    DIST_SCALE (0 where no voxel carries it); bc is the fine identity-row field, extents
    even."""
    from .runtime import field_pool2, geom_distance
    sites = (field_pool2(bc) > 0.0).float()
    d = geom_distance(sites)
    return (d.clamp_min(0.0) * (2.0 / DIST_SCALE)).contiguous()


def _pad(t, shape):
    import torch
    if tuple(t.shape) == tuple(shape):
        return t.contiguous()
    out = torch.zeros(shape, dtype=t.dtype, device=t.device)
    out[:t.shape[0], :t.shape[1], :t.shape[2]] = t
    return out


class LearnedStart:
    """A trained network for one grid: the grid padded to multiples of 16, the network at
    half of that."""

    def __init__(self, shape, params_flat):
        from .runtime import LPNet
        self.shape = tuple(shape)
        self.fine = pad16(shape)
        self.net = LPNet(tuple(v // 2 for v in self.fine))
        self.net.set_params(params_flat)

    def start(self, ctx):
        """The start (a torch CUDA float32 tensor of ctx's shape) for the system that
        ctx.pressure_setup(t) assembled."""
        from .runtime import field_up2
        m, k, b = ctx.pressure_learned_inputs()
        fs = self.fine
        mc, kc, dc = coarse_inputs(_pad(m, fs), _pad(k, fs), _pad(b, fs))
        d = field_up2(self.net.forward(mc, kc, dc))
        I, J, K = self.shape
        return ((1.0 - d[:I, :J, :K] / DEV_SCALE) * m).contiguous()

    def close(self):
        self.net.close()


def load_weights(path=WEIGHTS):
    return np.load(path) if os.path.exists(path) else None


def train(samples=256, epochs=64, lr=2e-3, seed=0, shape=PATCH, log=print, wide=None):
    """Generate samples with the plain solver and train a network on them; returns
    (flat parameters, history)."""
    from .runtime import LPNet
    t0 = time.time()
    data, metas = [], []
    if wide:
        for s in range((samples + CROPS - 1) // CROPS):
            d, meta = make_crops(seed * 100003 + s, wide, shape, CROPS)
            data.extend(d)
            metas.append(meta)
        data = data[:samples]
    else:
        for s in range(samples):
            d, meta = make_sample(seed * 100003 + s, shape)
            data.append(d)
            metas.append(meta)
    gen_s = time.time() - t0
    log(f"generated {len(data)} samples from {len(metas)} solves in {gen_s:.1f}s "
        f"(mean plain iterations {np.mean([m['iterations'] for m in metas]):.1f})")
    net = LPNet(tuple(v // 2 for v in pad16(shape)), seed=seed)
    rng = np.random.default_rng(seed)
    hist = []
    t1 = time.time()
    steps = epochs * samples
    for ep in range(epochs):
        order = rng.permutation(samples)
        losses = []
        for q, i in enumerate(order):
            step = ep * samples + q
            rate = lr * 0.5 * (1.0 + math.cos(math.pi * step / steps))  # cosine decay
            m, k, dist, tgt, anchored = data[i]
            losses.append(net.train_step(m, k, dist, tgt, anchored, lr=rate))
        hist.append(float(np.mean(losses)))
        log(f"epoch {ep}: mean loss {hist[-1]:.3e}")
    train_s = time.time() - t1
    flat = net.get_params()
    net.close()
    return flat, {"samples": samples, "epochs": epochs, "lr": lr, "generate_s": round(gen_s, 1),
                  "train_s": round(train_s, 1), "loss": hist}


# ---------------------------------------------------------------------------
# The learned coarse solver of the pressure multigrid (press_solver = PRESS_LEARNED): the
# same network, at 1/8 resolution, standing in for the V-cycle below the K-cycle levels.
# Its inputs are the member mask of multigrid level 4, the anchoring fraction e/d of each
# cell and the Jacobi-scaled residual D^-1/2 b / s (s = max |D^-1/2 b|); it predicts the
# Jacobi-scaled correction D^1/2 x / (s LPC_OUT_SCALE) with x ~ M^-1 b. It is trained on the
# level-4 operators of the plain solver's hierarchies for seeded geometries: for random
# errors x (white noise and Gaussian-smoothed noise of several correlation lengths, on the
# member cells) the input is b = M x and the target x itself, so no solve is needed.

PRECOND_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lpnet_precond_weights.npy")
LPC_LEVEL = 4
LPC_OUT_SCALE = 64.0   # kLpcOutScale of csrc/ls_mg.cu
LPC_SIGMAS = (0.0, 0.7, 1.5, 3.0, 6.0)


def level_apply(op, x):
    """M x of a multigrid level held as excess + links (float64): (M x)_i = e_i x_i +
    sum_j c_ij (x_i - x_j), f0/f1/f2 the links of the +i/+j/+k faces."""
    y = op["e"].astype(np.float64) * x
    for ax, f in enumerate(("f0", "f1", "f2")):
        c = np.asarray(op[f], np.float64)
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, -1)
        hi[ax] = slice(1, None)
        lo, hi = tuple(lo), tuple(hi)
        d = c[lo] * (x[lo] - x[hi])
        y[lo] += d
        y[hi] -= d
    return y


def level_diag(op):
    d = op["e"].astype(np.float64).copy()
    for ax, f in enumerate(("f0", "f1", "f2")):
        c = np.asarray(op[f], np.float64)
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, -1)
        hi[ax] = slice(1, None)
        d[tuple(lo)] += c[tuple(lo)]
        d[tuple(hi)] += c[tuple(lo)]
    return d


LPC_ANCHOR = 1e-3     # kLpcAnchor of csrc/ls_mg.cu


def precond_inputs(op):
    """Mask of the cells the network serves (members of components with a cell whose excess
    is above LPC_ANCHOR of its diagonal), anchoring fraction e/d and 1/sqrt(d) of those
    cells (float64 arrays)."""
    comp = op["comp"]
    m = comp >= 0
    d = level_diag(op)
    frac = np.where(m & (d > 0), op["e"] / np.where(d > 0, d, 1.0), 0.0)
    ids = np.unique(comp[m & (frac.astype(np.float32) > np.float32(LPC_ANCHOR))])
    ok = m & (d > 0) & np.isin(comp, ids)
    isd = np.where(ok, 1.0 / np.sqrt(np.where(ok, d, 1.0)), 0.0)
    anchor = np.where(ok, frac, 0.0)
    return ok, anchor, isd


def precond_samples(op, count, rng, net_shape):
    """count (mask, anchor, input, target) samples for one level operator, padded to the
    network grid."""
    from scipy.ndimage import gaussian_filter
    m, anchor, isd = precond_inputs(op)
    shape = m.shape

    def pad(a):
        out = np.zeros(net_shape, np.float32)
        out[:shape[0], :shape[1], :shape[2]] = a
        return out

    out = []
    while len(out) < count:
        sigma = float(rng.choice(LPC_SIGMAS))
        x = rng.standard_normal(shape)
        if sigma > 0:
            x = gaussian_filter(x, sigma, mode="nearest")
        x = x * m
        r = level_apply(op, x) * m
        rh = r * isd
        s = float(np.abs(rh).max())
        if not (s > 0):
            continue
        tgt = np.where(m, x / np.where(m, isd, 1.0) / (s * LPC_OUT_SCALE), 0.0)
        out.append((pad(m), pad(anchor), pad(rh / s), pad(tgt)))
    return out


def precond_level(seed, shape=WIDE, level=LPC_LEVEL, t=RAMP):
    """The level-`level` operator of the plain solver's hierarchy for one seeded geometry."""
    import torch
    from .runtime import Context
    lab, meta = patch_geometry(seed, shape)
    ctx = Context(shape, params=solver_params())
    try:
        ctx.upload("label", lab)
        ctx.init_all()
        ctx.props()
        ctx.pressure_setup(t)
        ok, info = ctx.pressure_solve_start(torch.zeros(shape, dtype=torch.float32, device="cuda"), 0.0)
        if not ok:
            raise RuntimeError(f"plain solve failed on geometry {seed}: {info}")
        op = ctx.mg_level(level)
    finally:
        ctx.close()
    return op, dict(meta, iterations=info["iterations"])


def train_precond(geometries=8, per_geometry=128, epochs=24, lr=2e-3, seed=0, shape=WIDE, log=print):
    """Train the learned coarse solver; returns (flat parameters, history)."""
    from .runtime import LPNet
    rng = np.random.default_rng(seed)
    t0 = time.time()
    data, metas, net_shape = [], [], None
    for g in range(geometries):
        op, meta = precond_level(seed * 100003 + 7919 * (g + 1), shape)
        ns = pad8(op["shape"])
        if net_shape is None:
            net_shape = ns
        if ns != net_shape:
            raise RuntimeError("training geometries must share the level grid")
        data.extend(precond_samples(op, per_geometry, rng, net_shape))
        metas.append(meta)
    gen_s = time.time() - t0
    log(f"generated {len(data)} samples from {len(metas)} level-{LPC_LEVEL} operators of {net_shape} "
        f"in {gen_s:.1f}s")
    import torch
    dev = [tuple(torch.from_numpy(a).cuda() for a in d) for d in data]
    net = LPNet(net_shape, seed=seed + 1)
    hist = []
    t1 = time.time()
    n = len(dev)
    steps = epochs * n
    for ep in range(epochs):
        order = rng.permutation(n)
        losses = []
        for q, i in enumerate(order):
            rate = lr * 0.5 * (1.0 + math.cos(math.pi * (ep * n + q) / steps))
            m, a, x, tgt = dev[i]
            losses.append(net.train_step(m, a, x, tgt, m, lr=rate))
        hist.append(float(np.mean(losses)))
        log(f"epoch {ep}: mean loss {hist[-1]:.3e}")
    train_s = time.time() - t1
    flat = net.get_params()
    net.close()
    return flat, {"geometries": geometries, "samples": n, "epochs": epochs, "lr": lr,
                  "net_shape": list(net_shape), "generate_s": round(gen_s, 1), "train_s": round(train_s, 1),
                  "loss": hist}


def precond_quality(flat, op, count=32, seed=1):
    """Mean relative error ||x - x_net|| / ||x|| (Jacobi-scaled) of the network on random
    samples of a level operator (random errors x as in training); flat None: the zero
    correction (error 1)."""
    from .runtime import LPNet
    rng = np.random.default_rng(seed)
    ns = pad8(op["shape"])
    samples = precond_samples(op, count, rng, ns)
    net = LPNet(ns)
    if flat is not None:
        net.set_params(flat)
    errs = []
    for m, a, x, tgt in samples:
        y = net.forward(m, a, x).cpu().numpy() * m
        errs.append(float(np.linalg.norm(y - tgt) / max(np.linalg.norm(tgt), 1e-30)))
    net.close()
    return float(np.mean(errs))


def load_precond_weights(path=PRECOND_WEIGHTS):
    return np.load(path) if os.path.exists(path) else None


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    tr = sub.add_parser("train")
    tr.add_argument("--samples", type=int, default=256)
    tr.add_argument("--epochs", type=int, default=64)
    tr.add_argument("--lr", type=float, default=2e-3)
    tr.add_argument("--seed", type=int, default=0)
    tr.add_argument("--out", default=WEIGHTS)
    tr.add_argument("--patches", action="store_true",
                    help="solve each sample on its own (default: cut the samples from wide solves)")
    tp = sub.add_parser("train-precond", help="train the learned coarse solver of the pressure multigrid")
    tp.add_argument("--geometries", type=int, default=8)
    tp.add_argument("--per-geometry", type=int, default=128)
    tp.add_argument("--epochs", type=int, default=24)
    tp.add_argument("--lr", type=float, default=2e-3)
    tp.add_argument("--seed", type=int, default=0)
    tp.add_argument("--out", default=PRECOND_WEIGHTS)
    fw = sub.add_parser("forward", help="time the network's forward pass on random inputs")
    fw.add_argument("--shape", default="144,176,176", help="network grid (multiples of 8)")
    fw.add_argument("--reps", type=int, default=5)
    ts = sub.add_parser("train-step", help="time the network's training step (forward, backward, Adam) on random inputs")
    ts.add_argument("--shape", default="144,32,32", help="network grid (multiples of 8)")
    ts.add_argument("--steps", type=int, default=20)
    a = ap.parse_args(argv)
    if a.cmd == "train-step":
        import torch
        from .runtime import LPNet
        shape = tuple(int(v) for v in a.shape.split(","))
        net = LPNet(shape, seed=1)
        g = torch.Generator(device="cuda")
        g.manual_seed(0)
        x = [torch.randn(shape, device="cuda", generator=g) for _ in range(4)]
        mask = torch.ones(shape, device="cuda")
        for _ in range(3):
            net.train_step(x[0], x[1], x[2], x[3], mask, lr=1e-4)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            net.train_step(x[0], x[1], x[2], x[3], mask, lr=1e-4)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / a.steps
        net.close()
        print(json.dumps({"shape": shape, "train_step_ms": round(ms, 3), "steps": a.steps}))
    if a.cmd == "forward":
        import torch
        from .runtime import LPNet
        shape = tuple(int(v) for v in a.shape.split(","))
        net = LPNet(shape)
        w = load_weights()
        if w is not None:
            net.set_params(w)
        x = [torch.rand(shape, device="cuda") for _ in range(3)]
        times = []
        for _ in range(a.reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            net.forward(*x)
            torch.cuda.synchronize()
            times.append((time.perf_counter() - t0) * 1e3)
        vox = shape[0] * shape[1] * shape[2]
        # multiply-adds of the eight convolutions: full, 1/8, 1/64, 1/512 of the voxels
        flops = 2 * 27 * vox * (16 * 16 * 2 + 16 * 16 + (16 * 32 + 32 * 16) / 8 + (32 * 64 + 64 * 32) / 64
                                + 64 * 64 / 512)
        best = min(times)
        print(json.dumps({"shape": shape, "ms": round(best, 3), "tflops": round(flops / best / 1e9, 1),
                          "times_ms": [round(t, 3) for t in times]}))
        net.close()
    if a.cmd == "train-precond":
        flat, hist = train_precond(a.geometries, a.per_geometry, a.epochs, a.lr, a.seed,
                                   log=lambda *x: print(*x, file=sys.stderr, flush=True))
        np.save(a.out, flat)
        print(json.dumps(hist))
    if a.cmd == "train":
        flat, hist = train(a.samples, a.epochs, a.lr, a.seed, log=lambda *x: print(*x, file=sys.stderr, flush=True),
                           wide=None if a.patches else WIDE)
        np.save(a.out, flat)
        print(json.dumps(hist))


if __name__ == "__main__":
    main()
