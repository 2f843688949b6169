"""The learned start of the pressure solve (leachingsim_gb300/learned.py) and the solver
entry points behind it (ls_pressure_learned_inputs, ls_pressure_solve_start), plus the
switch between the FP64 and the mixed inner solver inside one context.

The start never changes what the solve converges to: every solve ends at the same FP64
relative residual (1e-8 here). A start is kept only on the components anchored to fixed
values (elsewhere the system is singular or nearly so and the zero start's value stays),
so solutions from different starts agree to ~1e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (32, 32, 40)


def _ctx(seed, shape=SHAPE, **kw):
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300.runtime import Context
    lab, _ = L.patch_geometry(seed, shape)
    ctx = Context(shape, params=L.solver_params(**kw))
    ctx.upload("label", lab)
    ctx.init_all()
    ctx.props()
    ctx.pressure_setup(L.RAMP)
    return ctx, lab


def _zero_solve(ctx):
    import torch
    from leachingsim_gb300 import learned as L
    ok, info = ctx.pressure_solve_start(torch.zeros(ctx.shape, dtype=torch.float32, device="cuda"), 0.0)
    assert ok, info
    return L._solution(ctx).copy(), info


def _rel(a, b):
    return np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel())


def test_learned_inputs_describe_the_system():
    from leachingsim_gb300.geometry import AIR, PORE
    ctx, lab = _ctx(1)
    m, k, b = (t.cpu().numpy() for t in ctx.pressure_learned_inputs())
    np.testing.assert_array_equal(m, (lab == PORE).astype(np.float32))
    K = ctx.download("permeability")
    np.testing.assert_allclose(k, (np.log10(np.maximum(K, 1e-30)) + 15.0) / 3.0, rtol=1e-6, atol=1e-6)
    assert set(np.unique(b)) <= {0.0, 1.0} and b.max() == 1.0
    assert np.all(lab[b == 1.0] == AIR)
    ctx.close()


def test_start_from_the_solution_needs_few_iterations():
    import torch
    from leachingsim_gb300 import learned as L
    ctx, lab = _ctx(2)
    x0, info0 = _zero_solve(ctx)
    start = torch.from_numpy((x0 / L.top_pressure(ctx.params, L.RAMP)).astype(np.float32)).cuda()
    ok, info1 = ctx.pressure_solve_start(start, 1.0)
    assert ok
    assert info1["iterations"] <= max(2, info0["iterations"] // 4), (info0, info1)
    assert _rel(L._solution(ctx), x0) < 1e-6
    ctx.close()


def test_untrained_network_start_still_converges_to_the_same_solution():
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300.runtime import LPNet
    ctx, _ = _ctx(3)
    x0, _ = _zero_solve(ctx)
    net = LPNet((8, 8, 8), seed=9)
    ls = L.LearnedStart(SHAPE, net.get_params())
    net.close()
    ok, info = ctx.pressure_solve_start(ls.start(ctx), 1.0)
    assert ok, info
    assert info["rel_residual"] <= 1e-8
    assert _rel(L._solution(ctx), x0) < 1e-5
    ls.close()
    ctx.close()


def test_trained_start_saves_iterations():
    """A network trained on a few plain-solver solutions (32x32x40 patches) gives a start
    from which the held-out solve takes fewer iterations than from zero."""
    from leachingsim_gb300 import learned as L
    flat, hist = L.train(samples=12, epochs=8, lr=2e-3, seed=1, shape=SHAPE, log=lambda *a: None)
    assert hist["loss"][-1] < hist["loss"][0]
    ctx, _ = _ctx(999)
    x0, info0 = _zero_solve(ctx)
    ls = L.LearnedStart(SHAPE, flat)
    ok, info1 = ctx.pressure_solve_start(ls.start(ctx), 1.0)
    assert ok
    assert info1["iterations"] < info0["iterations"], (info0, info1)
    assert info1["rel_residual"] <= 1e-8
    assert _rel(L._solution(ctx), x0) < 1e-5
    ls.close()
    ctx.close()


def test_inner_precision_switch_within_one_context():
    """Mixed -> FP64 -> mixed inner solver in one context (the inner arrays and the
    multigrid hierarchy are reallocated in the other precision) against fresh contexts."""
    from leachingsim_gb300._abi import PRESS_FP64, PRESS_MIXED
    from leachingsim_gb300 import learned as L
    ctx, _ = _ctx(4)
    xm, _ = _zero_solve(ctx)
    for solver in (PRESS_FP64, PRESS_MIXED, PRESS_FP64):
        ctx.set_params(L.solver_params(press_solver=solver))
        ctx.pressure_setup(L.RAMP)
        x, _ = _zero_solve(ctx)
        ref_ctx, _ = _ctx(4, press_solver=solver)
        xr, _ = _zero_solve(ref_ctx)
        ref_ctx.close()
        assert _rel(x, xr) < 1e-7, solver
        assert _rel(x, xm) < 1e-6, solver
    ctx.close()


def test_half_resolution_transfers():
    import torch
    from leachingsim_gb300.runtime import field_pool2, field_up2
    rng = np.random.default_rng(5)
    f = rng.standard_normal((6, 10, 4)).astype(np.float32)
    w = (rng.random((6, 10, 4)) < 0.5).astype(np.float32)
    blocks = lambda a: a.reshape(3, 2, 5, 2, 2, 2).transpose(0, 2, 4, 1, 3, 5).reshape(3, 5, 2, 8)
    ft, wt = torch.from_numpy(f).cuda(), torch.from_numpy(w).cuda()
    np.testing.assert_allclose(field_pool2(ft).cpu().numpy(), blocks(f).mean(-1), rtol=1e-6, atol=1e-6)
    sw = blocks(w).sum(-1)
    ref = np.where(sw > 0, (blocks(f) * blocks(w)).sum(-1) / np.maximum(sw, 1e-30), 0.0)
    np.testing.assert_allclose(field_pool2(ft, wt).cpu().numpy(), ref, rtol=1e-6, atol=1e-6)
    c = torch.from_numpy(rng.standard_normal((3, 5, 2)).astype(np.float32)).cuda()
    up = field_up2(c).cpu().numpy()
    np.testing.assert_array_equal(up, np.repeat(np.repeat(np.repeat(c.cpu().numpy(), 2, 0), 2, 1), 2, 2))
