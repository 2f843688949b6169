"""The learned pressure network: the oracle (oracle/lpnet_oracle.py) against finite
differences on the CPU, and the GPU kernels behind ls_lpnet_* (tensor-core convolutions,
weight gradients, pooling, Adam) against the oracle.

Tolerances: the GPU rounds every activation to BF16 (8 significant bits) and sums in FP32;
the oracle rounds at the same points and sums in FP64, so a value can land one BF16 step
(0.4 %) away, and such differences travel through the layers. Forward outputs agree to 2 %
(relative L2), gradients to 5 %; Adam, an FP32 elementwise update, to 1e-5 of the rate.
"""
import numpy as np
import pytest

from oracle import lpnet_oracle as lo


def _rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _case(shape, seed):
    rng = np.random.default_rng(seed)
    p = lo.init_params(seed)
    for k in p:
        if k.endswith("_b"):
            p[k] = (rng.standard_normal(p[k].shape) * 0.1).astype(np.float32)
    mask = (rng.random(shape) < 0.6).astype(np.float32)
    c1 = rng.standard_normal(shape).astype(np.float32)
    c2 = rng.standard_normal(shape).astype(np.float32)
    target = rng.standard_normal(shape).astype(np.float32)
    return p, mask, c1, c2, target


def _x16(mask, c1, c2):
    x = np.zeros(mask.shape + (16,), np.float32)
    x[..., 0], x[..., 1], x[..., 2] = mask, c1, c2
    return x


def test_oracle_gradients_match_finite_differences():
    p, mask, c1, c2, target = _case((8, 8, 8), 0)
    p = {k: v.astype(np.float64) for k, v in p.items()}
    x = _x16(mask, c1, c2).astype(np.float64)

    def loss_of(q):
        y, _ = lo.forward(q, x, round_bf16=False)
        return lo.mse_loss(y, target, mask)

    _, dy = loss_of(p)
    _, cache = lo.forward(p, x, round_bf16=False)
    g = lo.backward(p, cache, dy, round_bf16=False)
    for name, idx in [("W0a", (13, 3, 1)), ("W2", (5, 10, 7)), ("U0", (26, 0, 15)), ("U1", (0, 4, 31)),
                      ("W0b_b", (7,)), ("U2_b", (3,)), ("W1", (22, 17, 9))]:
        q = {k: v.copy() for k, v in p.items()}
        eps = 1e-6
        q[name][idx] += eps
        lp, _ = loss_of(q)
        q[name][idx] -= 2 * eps
        lm, _ = loss_of(q)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[name][idx]) <= 1e-6 * max(abs(fd), 1e-3), (name, idx, fd, g[name][idx])


def test_parameter_layout_round_trip():
    from leachingsim_gb300.runtime import lpnet_flatten, lpnet_unflatten
    p = lo.init_params(3)
    q = lpnet_unflatten(lpnet_flatten(p))
    assert all(np.array_equal(p[k], q[k]) for k in p)
    assert lpnet_flatten(p).size == sum(27 * ci * co + co for _, ci, co, _ in lo.LAYERS)


# convolution paths (LS_LPNET_TC, read when a network is created): "tma" = the TMA-fed
# tcgen05 kernel streaming through z with the dz taps stacked along N, every layer (3, the
# default); "tc" = the first tcgen05 kernel for every layer with up to 32 input channels (2),
# "tc64" = that kernel on the 32 -> 64 layer alone (1), "mma" = mma.sync only (0)
PATHS = ["tma", "tc", "tc64", "mma"]


def _path(monkeypatch, path):
    monkeypatch.setenv("LS_LPNET_TC", {"tc": "2", "tma": "3", "tc64": "1", "mma": "0"}[path])


@pytest.mark.gpu
@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("shape", [(16, 16, 24), (24, 40, 8), (8, 24, 56)])
def test_gpu_forward_matches_oracle(shape, path, monkeypatch):
    """Grids whose extents are not multiples of the convolution tiles (16 x 8 x 1 for
    tcgen05, 16 x 4 x 2 for mma.sync), down to coarse levels of odd extent."""
    from leachingsim_gb300.runtime import LPNet, lpnet_flatten
    _path(monkeypatch, path)
    p, mask, c1, c2, _ = _case(shape, 1)
    net = LPNet(shape)
    net.set_params(lpnet_flatten(p))
    out = net.forward(mask, c1, c2).cpu().numpy()
    y, _ = lo.forward(p, _x16(mask, c1, c2))
    assert _rel(out, y[..., 0]) < 2e-2
    net.close()


@pytest.mark.gpu
@pytest.mark.parametrize("path", PATHS)
def test_gpu_gradients_match_oracle(path, monkeypatch):
    from leachingsim_gb300.runtime import LPNet, lpnet_flatten, lpnet_unflatten
    _path(monkeypatch, path)
    shape = (16, 24, 16)
    p, mask, c1, c2, target = _case(shape, 2)
    net = LPNet(shape)
    net.set_params(lpnet_flatten(p))
    loss = net.train_step(mask, c1, c2, target, mask, lr=0.0, update=False)
    g = lpnet_unflatten(net.get_grads())
    y, cache = lo.forward(p, _x16(mask, c1, c2))
    lref, dy = lo.mse_loss(y, target, mask)
    gref = lo.backward(p, cache, dy)
    assert abs(loss - lref) <= 1e-3 * lref
    for name, *_ in lo.LAYERS:
        assert _rel(g[name], gref[name]) < 5e-2, name
        assert _rel(g[name + "_b"], gref[name + "_b"]) < 5e-2, name + "_b"
    net.close()


@pytest.mark.gpu
def test_gpu_adam_step_matches_oracle():
    from leachingsim_gb300.runtime import LPNet, lpnet_flatten, lpnet_unflatten
    shape = (8, 8, 16)
    p, mask, c1, c2, target = _case(shape, 3)
    net = LPNet(shape)
    flat = lpnet_flatten(p)
    net.set_params(flat)
    net.train_step(mask, c1, c2, target, mask, lr=0.0, update=False)
    g = lpnet_unflatten(net.get_grads())
    net.set_params(flat)
    lr = 1e-3
    net.train_step(mask, c1, c2, target, mask, lr=lr, update=True)
    got = net.get_params()
    ref = lpnet_flatten(lo.adam({k: v.copy() for k, v in p.items()}, g, {}, lr=lr))
    # the first Adam step moves each weight by ~lr * sign(g); gradients recomputed in the
    # second call may differ in the last bits (atomic summation order), which matters only
    # where |g| is near zero
    gf = lpnet_flatten(g)
    big = np.abs(gf) > 1e-6
    np.testing.assert_allclose(got[big], ref[big], rtol=0, atol=1e-5 * lr + 1e-7)
    assert np.all(np.abs(got - flat) <= lr * 1.0001 + 1e-7)
    net.close()


@pytest.mark.gpu
def test_gpu_training_reduces_loss():
    """The network learns a smooth field of its inputs (a blurred channel times the mask)."""
    from scipy import ndimage
    from leachingsim_gb300.runtime import LPNet
    shape = (16, 16, 16)
    rng = np.random.default_rng(4)
    net = LPNet(shape, seed=5)
    losses = []
    for it in range(120):
        mask = (ndimage.gaussian_filter(rng.standard_normal(shape), 2.0) > -0.1).astype(np.float32)
        c1 = rng.standard_normal(shape).astype(np.float32)
        target = (ndimage.gaussian_filter(c1, 1.5) * 3.0 * mask).astype(np.float32)
        losses.append(net.train_step(mask, c1, np.zeros(shape, np.float32), target, mask, lr=2e-3))
    assert np.mean(losses[-10:]) < 0.3 * np.mean(losses[:10]), (losses[:10], losses[-10:])
    net.close()


@pytest.mark.gpu
def test_gpu_tcgen05_and_mma_sync_paths_agree(monkeypatch):
    """The convolution paths sum the same BF16 products in FP32, in different orders: the
    outputs agree far inside the oracle tolerance, at a size with many tiles per level."""
    from leachingsim_gb300.runtime import LPNet, lpnet_flatten
    shape = (32, 48, 80)
    p, mask, c1, c2, _ = _case(shape, 6)
    outs = {}
    for path in PATHS:
        _path(monkeypatch, path)
        net = LPNet(shape)
        net.set_params(lpnet_flatten(p))
        outs[path] = net.forward(mask, c1, c2).cpu().numpy()
        net.close()
    for path in ("tma", "tc", "tc64"):
        assert _rel(outs[path], outs["mma"]) < 5e-3, path


@pytest.mark.gpu
@pytest.mark.parametrize("path", ["tma", "tc"])
def test_gpu_tcgen05_timeout_falls_back_to_mma_sync(path, monkeypatch):
    """A tcgen05 wait that gives up (the library's timeout counter, here set by the host-side
    LS_LPNET_SIMULATE_TIMEOUT switch; nothing on the GPU waits less or is skipped) makes the
    network discard the pass, switch to its mma.sync kernels for good and recompute: the
    forward returns the fallback status with the mma.sync result, and later passes (the
    switch off again) still match it."""
    from leachingsim_gb300.runtime import LPNet, lpnet_flatten
    shape = (16, 24, 24)
    p, mask, c1, c2, _ = _case(shape, 7)
    _path(monkeypatch, "mma")
    ref_net = LPNet(shape)
    ref_net.set_params(lpnet_flatten(p))
    ref = ref_net.forward(mask, c1, c2).cpu().numpy()
    ref_net.close()
    _path(monkeypatch, path)
    net = LPNet(shape)
    net.set_params(lpnet_flatten(p))
    monkeypatch.setenv("LS_LPNET_SIMULATE_TIMEOUT", "1")
    out = net.forward(mask, c1, c2).cpu().numpy()
    assert net.last_status == 2
    monkeypatch.delenv("LS_LPNET_SIMULATE_TIMEOUT")
    again = net.forward(mask, c1, c2).cpu().numpy()
    assert net.last_status == 0
    net.close()
    np.testing.assert_array_equal(out, ref)
    np.testing.assert_array_equal(again, ref)
