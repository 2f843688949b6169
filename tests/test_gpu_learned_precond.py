"""The learned coarse solver of the pressure multigrid (press_solver = PRESS_LEARNED,
ls_pressure_set_precond_weights): the network stands in for the V-cycle below the K-cycle
levels inside the flexible CG, and the plain cycle takes over when that CG stagnates.

Whatever the network does, the solve ends at the requested FP64 relative residual and at the
plain solver's solution (to ~1e-6, the near-null modes of weakly anchored Pore clusters,
as for the learned start): a network whose activations overflow hands the solve to the plain
cycle at once, a network that outputs nothing (zero weights) once the CG slows down."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (96, 96, 96)  # multigrid level 4 (the learned one) is 6^3, the network grid 8^3


def _ctx(seed=11):
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300.runtime import Context
    lab, _ = L.patch_geometry(seed, SHAPE)
    ctx = Context(SHAPE, params=L.solver_params(press_rtol=1e-10))
    ctx.upload("label", lab)
    ctx.init_all()
    ctx.props()
    return ctx


def _solve(ctx, solver, weights=None):
    import torch
    from leachingsim_gb300 import learned as L
    p = L.solver_params(press_rtol=1e-10, press_solver=solver)
    ctx.set_params(p)
    if weights is not None:
        ctx.set_precond_weights(weights)
    ctx.upload("pressure", np.zeros(ctx.NP), padded=True)
    ctx.pressure_setup(L.RAMP)
    f0 = ctx.pressure_fallbacks()
    ok, info = ctx.pressure_solve_start(torch.zeros(SHAPE, dtype=torch.float32, device="cuda"), 0.0)
    assert ok, info
    assert info["rel_residual"] <= 1e-10
    return L._solution(ctx).copy(), info, ctx.pressure_fallbacks() - f0


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def plain():
    from leachingsim_gb300 import _abi
    ctx = _ctx()
    x, info, _ = _solve(ctx, _abi.PRESS_MIXED)
    ctx.close()
    return x, info


def test_shipped_weights_exist_and_fit_the_network():
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300.runtime import LPNet
    w = L.load_precond_weights()
    assert w is not None
    net = LPNet((16, 16, 16))
    assert w.size == net.n
    net.close()


def test_learned_solve_reaches_the_plain_solution(plain):
    from leachingsim_gb300 import _abi
    from leachingsim_gb300 import learned as L
    ctx = _ctx()
    x, info, _ = _solve(ctx, _abi.PRESS_LEARNED, L.load_precond_weights())
    ctx.close()
    assert _rel(x, plain[0]) < 1e-6


def test_overflowing_network_falls_back_at_once(plain):
    from leachingsim_gb300 import _abi
    from leachingsim_gb300 import learned as L
    ctx = _ctx()
    bad = np.full_like(L.load_precond_weights(), 3e38)
    x, info, fb = _solve(ctx, _abi.PRESS_LEARNED, bad)
    ctx.close()
    assert fb >= 1
    assert _rel(x, plain[0]) < 1e-6


def test_silent_network_falls_back_on_stagnation(plain):
    from leachingsim_gb300 import _abi
    from leachingsim_gb300 import learned as L
    ctx = _ctx()
    x, info, fb = _solve(ctx, _abi.PRESS_LEARNED, np.zeros_like(L.load_precond_weights()))
    ctx.close()
    assert fb >= 1
    assert _rel(x, plain[0]) < 1e-6


def test_learned_weights_need_a_learned_solver():
    from leachingsim_gb300 import _abi
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300.runtime import LsError
    ctx = _ctx()
    ctx.set_params(L.solver_params(press_solver=_abi.PRESS_LEARNED))
    ctx.set_precond_weights(np.zeros(0, np.float32))
    ctx.pressure_setup(L.RAMP)
    import torch
    with pytest.raises(LsError):
        ctx.pressure_solve_start(torch.zeros(SHAPE, dtype=torch.float32, device="cuda"), 0.0)
    ctx.close()


def test_trained_network_gains_over_no_network():
    """The trained network's Jacobi-scaled error on random errors of a level-4 operator it
    was not trained on, against no correction (error 1) and the untrained network."""
    from leachingsim_gb300 import _abi
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300.runtime import LPNet
    ctx = _ctx(seed=23)
    _solve(ctx, _abi.PRESS_MIXED)
    op = ctx.mg_level(L.LPC_LEVEL)
    ctx.close()
    trained = L.precond_quality(L.load_precond_weights(), op)
    net = LPNet(L.pad8(op["shape"]), seed=1)
    untrained = L.precond_quality(net.get_params(), op)
    net.close()
    print({"trained": trained, "untrained": untrained})
    assert trained < 0.99
    assert trained < untrained


def test_mg_level_hook_needs_an_fp32_hierarchy():
    from leachingsim_gb300 import _abi
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300.runtime import LsError
    ctx = _ctx()
    with pytest.raises(LsError):
        ctx.mg_level(1)            # no solve yet
    _solve(ctx, _abi.PRESS_MIXED)
    op = ctx.mg_level(1)
    assert op["shape"] == (48, 48, 48)
    members = op["comp"] >= 0
    assert members.any() and np.all(op["e"][members] >= 0) and np.all(op["f0"] >= 0)
    with pytest.raises(LsError):
        ctx.mg_level(99)
    ctx.close()
