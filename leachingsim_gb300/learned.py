"""The learned warm start of the pressure solve.

The network (the U-shaped 3D convolutional network of ls_lpnet_*, hand-written CUDA
kernels for its forward and backward passes and Adam) maps three fields of an assembled
pressure system to a start for the solve:

    mask  - 1 on the Pore rows (the unknowns), 0 elsewhere
    logk  - (log10 K + 15) / 3
    dist  - the Euclidean distance to the nearest voxel that carries the top pressure
            (ls_geom_distance), over 100: the pressure of the Pore space falls off with
            it, on scales beyond the network's receptive field

and predicts the deviation of the pressure from the top pressure, d = 100 (1 - P / p_top),
on the Pore rows (the start is P / p_top = 1 - d / 100). The network runs at half
resolution: its inputs are the 2x2x2 block means of the three fields (ls_field_pool2), its
output is repeated over each block (ls_field_up2); the deviation varies on the scale of
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


def coarse_inputs(m, k, dist):
    """The network's inputs: 2x2x2 block means of the three fine fields (extents even)."""
    from .runtime import field_pool2
    return field_pool2(m), field_pool2(k), field_pool2(dist)


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
        dist = distance_input(b)
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
        m, k, dist, target, anchored = (_pad(v, fs) for v in (m, k, dist, target, anchored))
        mc, kc, dc = coarse_inputs(m, k, dist)
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


def distance_input(bc):
    """The third input: distance to the voxels carrying the top pressure, over DIST_SCALE
    (0 where no voxel carries it)."""
    from .runtime import geom_distance
    d = geom_distance((bc > 0.5).float())
    return (d.clamp_min(0.0) / DIST_SCALE).contiguous()


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
        mc, kc, dc = coarse_inputs(_pad(m, fs), _pad(k, fs), _pad(distance_input(b), fs))
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
    fw = sub.add_parser("forward", help="time the network's forward pass on random inputs")
    fw.add_argument("--shape", default="144,176,176", help="network grid (multiples of 8)")
    fw.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)
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
    if a.cmd == "train":
        flat, hist = train(a.samples, a.epochs, a.lr, a.seed, log=lambda *x: print(*x, file=sys.stderr, flush=True),
                           wide=None if a.patches else WIDE)
        np.save(a.out, flat)
        print(json.dumps(hist))


if __name__ == "__main__":
    main()
