"""The multigrid preconditioner captured into CUDA graphs (the default) against the same
cycle launched kernel by kernel (LS_MG_GRAPHS=0, read when a context is created): the
graph replays the very launches the capture recorded, so both solves take the same
iterations and give the same pressure bit for bit, for both inner precisions and for the
learned coarse solver, over solves that rebuild the hierarchy in place (the captured graphs
stay valid) and across a precision switch (which frees the hierarchy and its graphs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (48, 40, 40)


def _run(monkeypatch, graphs):
    import torch
    from leachingsim_gb300 import _abi
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300.runtime import Context
    monkeypatch.setenv("LS_MG_GRAPHS", "1" if graphs else "0")
    lab, _ = L.patch_geometry(5, SHAPE)
    ctx = Context(SHAPE, params=L.solver_params(press_rtol=1e-10))
    ctx.upload("label", lab)
    ctx.init_all()
    ctx.props()
    ctx.set_precond_weights(L.load_precond_weights())
    zero = torch.zeros(SHAPE, dtype=torch.float32, device="cuda")
    out = []
    for solver in (_abi.PRESS_MIXED, _abi.PRESS_MIXED, _abi.PRESS_FP64, _abi.PRESS_LEARNED, _abi.PRESS_MIXED):
        ctx.set_params(L.solver_params(press_rtol=1e-10, press_solver=solver))
        ctx.upload("pressure", np.zeros(ctx.NP), padded=True)
        ctx.pressure_setup(L.RAMP)
        ok, info = ctx.pressure_solve_start(zero, 0.0)
        assert ok, info
        out.append((info["iterations"], info["outer_iterations"], ctx.download("pressure", padded=True).copy()))
    ctx.close()
    return out


def test_captured_cycle_matches_kernel_by_kernel(monkeypatch):
    a = _run(monkeypatch, True)
    b = _run(monkeypatch, False)
    for (ia, oa, pa), (ib, ob, pb) in zip(a, b):
        assert (ia, oa) == (ib, ob)
        assert np.array_equal(pa, pb)


def _run_tail(monkeypatch, tail_cells):
    import torch
    from leachingsim_gb300 import _abi
    from leachingsim_gb300 import learned as L
    from leachingsim_gb300.runtime import Context
    monkeypatch.setenv("LS_MG_TAIL_CELLS", str(tail_cells))
    monkeypatch.setenv("LS_MG_GRAPHS", "0")  # count the launches one by one
    shape = (160, 128, 128)  # levels 4 (640 cells) and 5 (80) below the K-cycle levels
    lab, _ = L.patch_geometry(7, shape)
    ctx = Context(shape, params=L.solver_params(press_rtol=1e-10))
    ctx.upload("label", lab)
    ctx.init_all()
    ctx.props()
    zero = torch.zeros(shape, dtype=torch.float32, device="cuda")
    out = []
    for solver in (_abi.PRESS_MIXED, _abi.PRESS_FP64):
        ctx.set_params(L.solver_params(press_rtol=1e-10, press_solver=solver))
        ctx.upload("pressure", np.zeros(ctx.NP), padded=True)
        ctx.pressure_setup(L.RAMP)
        l0 = ctx.launches()
        ok, info = ctx.pressure_solve_start(zero, 0.0)
        assert ok, info
        out.append((info["iterations"], info["outer_iterations"], ctx.download("pressure", padded=True).copy(),
                    ctx.launches() - l0))
    ctx.close()
    return out


def test_one_block_coarse_tail_matches_level_kernels(monkeypatch):
    """The V-cycle over the small coarse levels run by one block (k_mg_tail) against the
    same cycle as one kernel per sweep (LS_MG_TAIL_CELLS=0): the same per-cell updates in
    the same order, so the same iterations and pressure bit for bit, with far fewer
    launches."""
    a = _run_tail(monkeypatch, 4096)
    b = _run_tail(monkeypatch, 0)
    for (ia, oa, pa, la), (ib, ob, pb, lb) in zip(a, b):
        assert (ia, oa) == (ib, ob)
        assert np.array_equal(pa, pb)
        assert la < lb
