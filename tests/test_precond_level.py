"""Host side of the learned coarse solver's training (leachingsim_gb300/learned.py): the
level operator in excess + Laplacian form against an assembled dense matrix, and the
training samples' scaling (input = D^-1/2 M x / s, target = D^1/2 x / (64 s))."""
import numpy as np

from leachingsim_gb300 import learned as L


def _op(shape=(6, 5, 7), seed=0):
    rng = np.random.default_rng(seed)
    op = {"shape": shape, "comp": np.where(rng.random(shape) < 0.8, 0, -1).astype(np.int32),
          "e": (rng.random(shape) * 0.1).astype(np.float32)}
    for f in ("f0", "f1", "f2"):
        op[f] = rng.random(shape).astype(np.float32)
    op["f0"][-1] = 0
    op["f1"][:, -1] = 0
    op["f2"][:, :, -1] = 0
    return op


def _dense(op):
    sh = op["shape"]
    n = int(np.prod(sh))
    A = np.zeros((n, n))
    idx = np.arange(n).reshape(sh)
    for i in range(sh[0]):
        for j in range(sh[1]):
            for k in range(sh[2]):
                r = idx[i, j, k]
                A[r, r] += op["e"][i, j, k]
                for di, dj, dk, f in ((1, 0, 0, "f0"), (0, 1, 0, "f1"), (0, 0, 1, "f2")):
                    ii, jj, kk = i + di, j + dj, k + dk
                    if ii < sh[0] and jj < sh[1] and kk < sh[2]:
                        c = op[f][i, j, k]
                        q = idx[ii, jj, kk]
                        A[r, r] += c
                        A[q, q] += c
                        A[r, q] -= c
                        A[q, r] -= c
    return A


def test_level_apply_and_diagonal_match_the_assembled_operator():
    op = _op()
    A = _dense(op)
    x = np.random.default_rng(1).standard_normal(op["shape"])
    np.testing.assert_allclose(L.level_apply(op, x).ravel(), A @ x.ravel(), rtol=0, atol=1e-13)
    np.testing.assert_allclose(L.level_diag(op).ravel(), np.diag(A), rtol=1e-15, atol=0)


def test_samples_scale_input_and_target_consistently():
    op = _op()
    rng = np.random.default_rng(2)
    m, anchor, isd = L.precond_inputs(op)
    A = _dense(op)
    for mask, anc, inp, tgt in L.precond_samples(op, 6, rng, (8, 8, 8)):
        sh = op["shape"]
        sl = (slice(0, sh[0]), slice(0, sh[1]), slice(0, sh[2]))
        assert np.array_equal(mask[sl] > 0, m)
        assert np.abs(inp).max() == np.float32(1.0)
        assert not mask[sh[0]:].any() and not inp[sh[0]:].any()
        # x = 64 s D^-1/2 target must reproduce the input: D^-1/2 M x / s = input
        x = np.where(m, tgt[sl].astype(np.float64) * isd, 0.0)  # = x / (64 s)
        rh = (A @ x.ravel()).reshape(sh) * isd * L.LPC_OUT_SCALE
        np.testing.assert_allclose(rh[m], inp[sl][m], rtol=1e-4, atol=1e-5)
        np.testing.assert_allclose(anc[sl], anchor, rtol=1e-6, atol=1e-7)
