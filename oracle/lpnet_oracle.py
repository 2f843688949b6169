"""CPU restatement of the learned pressure network, for the tests (the oracle).

Test infrastructure: only tests/ import this module, as the checker of the network kernels
in leachingsim_gb300/csrc/ls_learned.cu (forward, backward, Adam). The network has no
counterpart in the reference (it is the learned warm start / preconditioner of the
pressure solve), so there is nothing to pin against but the mathematics: the tests check
this module's gradients by finite differences and the GPU kernels against this module.

Layout and arithmetic, as on the GPU:
* activations are (D, H, W, C) arrays (channels innermost), stored as bfloat16 between
  layers (`bf16` rounds float32 to the nearest bfloat16, ties to even); the output layer
  is float32;
* a convolution is 3x3x3, stride 1, zero padding: out[z,y,x,co] = b[co] +
  sum_tap sum_ci w[tap,co,ci] in[z+dz,y+dy,x+dx,ci], tap = 9 (dz+1) + 3 (dy+1) + (dx+1);
  weights and inputs are bfloat16, sums are float32 on the GPU (float64 here);
* pooling is the 2x2x2 mean, upsampling repeats each voxel 2x2x2.

The U-shaped network (4 levels, 16-64 channels; input 16 channels of which the first
three are used, output channel 0 of 16):

    a0 = relu(conv(x, W0a))          16      s0 = relu(conv(a0, W0b))     16
    s1 = relu(conv(pool(s0), W1))    32      s2 = relu(conv(pool(s1), W2)) 64
    a3 = relu(conv(pool(s2), W3))    64
    b2 = relu(conv(up(a3) + s2, U2)) 32      b1 = relu(conv(up(b2) + s1, U1)) 16
    y  = conv(up(b1) + s0, U0)       16
"""
import numpy as np

LAYERS = [  # name, cin, cout, relu
    ("W0a", 16, 16, True), ("W0b", 16, 16, True), ("W1", 16, 32, True), ("W2", 32, 64, True),
    ("W3", 64, 64, True), ("U2", 64, 32, True), ("U1", 32, 16, True), ("U0", 16, 16, False)]


def bf16(a):
    """Round float32 values to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    nan = np.isnan(a)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).copy()
    out[nan] = np.nan
    return out


def init_params(seed=0):
    """He-normal float32 weights, zero biases."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, cin, cout, _ in LAYERS:
        std = np.sqrt(2.0 / (27 * cin))
        p[name] = (rng.standard_normal((27, cout, cin)) * std).astype(np.float32)
        p[name + "_b"] = np.zeros(cout, np.float32)
    return p


def _shift(a, dz, dy, dx):
    """out[z,y,x] = a[z+dz, y+dy, x+dx] with zeros outside."""
    out = np.zeros_like(a)
    D, H, W = a.shape[:3]
    zs, ys, xs = slice(max(0, -dz), min(D, D - dz)), slice(max(0, -dy), min(H, H - dy)), slice(max(0, -dx), min(W, W - dx))
    zd, yd, xd = slice(max(0, dz), min(D, D + dz)), slice(max(0, dy), min(H, H + dy)), slice(max(0, dx), min(W, W + dx))
    out[zs, ys, xs] = a[zd, yd, xd]
    return out


TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def conv(x, w, b):
    x = x.astype(np.float64)
    out = np.zeros(x.shape[:3] + (w.shape[1],), np.float64)
    for t, (dz, dy, dx) in enumerate(TAPS):
        out += _shift(x, dz, dy, dx) @ w[t].T.astype(np.float64)
    return out + b.astype(np.float64)


def conv_bwd_data(dy, w):
    dy = dy.astype(np.float64)
    out = np.zeros(dy.shape[:3] + (w.shape[2],), np.float64)
    for t, (dz, dy_, dx) in enumerate(TAPS):
        out += _shift(dy, -dz, -dy_, -dx) @ w[t].astype(np.float64)
    return out


def conv_bwd_w(x, dy):
    x = x.astype(np.float64)
    dy = dy.astype(np.float64)
    cin, cout = x.shape[3], dy.shape[3]
    dw = np.zeros((27, cout, cin), np.float64)
    for t, (dz, dy_, dx) in enumerate(TAPS):
        dw[t] = dy.reshape(-1, cout).T @ _shift(x, dz, dy_, dx).reshape(-1, cin)
    return dw, dy.reshape(-1, cout).sum(axis=0)


def pool(a):
    D, H, W, C = a.shape
    return a.reshape(D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(1, 3, 5))


def pool_bwd(d):
    return np.repeat(np.repeat(np.repeat(d, 2, 0), 2, 1), 2, 2) / 8.0


def up(a):
    return np.repeat(np.repeat(np.repeat(a, 2, 0), 2, 1), 2, 2)


def up_bwd(d):
    D, H, W, C = d.shape
    return d.reshape(D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(1, 3, 5))


def forward(p, x, round_bf16=True):
    """Returns the output (D, H, W, 16) and the cache of every layer input/output."""
    r = bf16 if round_bf16 else (lambda v: np.asarray(v, np.float64))
    wq = {n: r(p[n]) for n, *_ in LAYERS}
    c = {"x": r(x)}

    def layer(name, inp, relu, rnd=True):
        o = conv(inp, wq[name], p[name + "_b"])
        if relu:
            o = np.maximum(o, 0.0)
        return r(o) if rnd else o

    c["a0"] = layer("W0a", c["x"], True)
    c["s0"] = layer("W0b", c["a0"], True)
    c["p1"] = r(pool(c["s0"]))
    c["s1"] = layer("W1", c["p1"], True)
    c["p2"] = r(pool(c["s1"]))
    c["s2"] = layer("W2", c["p2"], True)
    c["p3"] = r(pool(c["s2"]))
    c["a3"] = layer("W3", c["p3"], True)
    c["u2"] = r(up(c["a3"]) + c["s2"])
    c["b2"] = layer("U2", c["u2"], True)
    c["u1"] = r(up(c["b2"]) + c["s1"])
    c["b1"] = layer("U1", c["u1"], True)
    c["u0"] = r(up(c["b1"]) + c["s0"])
    c["y"] = layer("U0", c["u0"], False, rnd=False)  # the output layer stays FP32
    c["wq"] = wq
    return c["y"], c


def backward(p, c, dy, round_bf16=True):
    """Gradients of every weight and bias for the output gradient dy (D, H, W, 16)."""
    r = bf16 if round_bf16 else (lambda v: np.asarray(v, np.float64))
    wq = c["wq"]
    g = {}

    def layer_bwd(name, inp, out, d, relu):
        if relu:
            d = d * (out > 0)
        d = r(d)
        g[name], g[name + "_b"] = conv_bwd_w(inp, d)
        return conv_bwd_data(d, wq[name])

    d_u0 = layer_bwd("U0", c["u0"], c["y"], dy, False)
    d_s0 = d_u0.copy()
    d_b1 = up_bwd(d_u0)
    d_u1 = layer_bwd("U1", c["u1"], c["b1"], d_b1, True)
    d_s1 = d_u1.copy()
    d_b2 = up_bwd(d_u1)
    d_u2 = layer_bwd("U2", c["u2"], c["b2"], d_b2, True)
    d_s2 = d_u2.copy()
    d_a3 = up_bwd(d_u2)
    d_p3 = layer_bwd("W3", c["p3"], c["a3"], d_a3, True)
    d_s2 = d_s2 + pool_bwd(d_p3)
    d_p2 = layer_bwd("W2", c["p2"], c["s2"], d_s2, True)
    d_s1 = d_s1 + pool_bwd(d_p2)
    d_p1 = layer_bwd("W1", c["p1"], c["s1"], d_s1, True)
    d_s0 = d_s0 + pool_bwd(d_p1)
    d_a0 = layer_bwd("W0b", c["a0"], c["s0"], d_s0, True)
    layer_bwd("W0a", c["x"], c["a0"], d_a0, True)
    return g


def mse_loss(y, target, mask):
    """Mean over masked voxels of (y[..., 0] - target)^2 and its gradient wrt y."""
    n = max(int(mask.sum()), 1)
    diff = (y[..., 0].astype(np.float64) - target) * mask
    dy = np.zeros(y.shape, np.float64)
    dy[..., 0] = 2.0 * diff / n
    return float((diff * diff).sum() / n), dy


def adam(p, g, state, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step on the float32 master parameters (state: m, v per parameter, t)."""
    state["t"] = state.get("t", 0) + 1
    t = state["t"]
    for k in g:
        m = state.setdefault("m_" + k, np.zeros_like(p[k]))
        v = state.setdefault("v_" + k, np.zeros_like(p[k]))
        gk = g[k].astype(np.float32)
        m[...] = b1 * m + (1 - b1) * gk
        v[...] = b2 * v + (1 - b2) * gk * gk
        mh = m / (1 - b1 ** t)
        vh = v / (1 - b2 ** t)
        p[k] = (p[k] - lr * mh / (np.sqrt(vh) + eps)).astype(np.float32)
    return p
