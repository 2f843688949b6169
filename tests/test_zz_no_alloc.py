"""ls_saturation_noalloc: the explicit saturation update for callers that cannot let the
library allocate device memory (hosts that own all device memory through their own pool,
stepping loops that cannot take an allocation's synchronisation). It must give exactly what
the context entry point ls_saturation gives, call after call, with its scratch in a fixed
device array. Device buffers here belong to the caller (allocated by torch)."""
import ctypes as C

import numpy as np
import pytest

from helpers import params, small_grf
from leachingsim_gb300._abi import LS_BAD_ARG, LS_OK, LsSubstepInfo
from leachingsim_gb300.runtime import Context, load

pytestmark = pytest.mark.gpu


def _call(L, shape, label, fx, fy, fz, sat, dt, p):
    I, J, K = shape
    info = LsSubstepInfo()
    err = C.create_string_buffer(256)
    st = L.ls_saturation_noalloc(I, J, K, 1, label.data_ptr(), fx.data_ptr(), fy.data_ptr(),
                                 fz.data_ptr(), sat.data_ptr(), dt, p.dx, p.porosity,
                                 p.evaporative_flux, None, C.byref(info), err, 256)
    return st, info, err.value.decode()


def test_noalloc_matches_context_entry_point_twice():
    torch = pytest.importorskip("torch")
    L = load()
    lab = small_grf((24, 20, 18), seed=3)
    p = params(evaporative_flux=2e-3)
    ctx = Context(lab.shape, params=p)
    ctx.upload("label", lab)
    ctx.init_all()
    ok, _ = ctx.pressure(600.0)
    assert ok
    ctx.flux()
    dev = torch.device("cuda")
    fl = {}
    for f in ("flux_x", "flux_y", "flux_z"):
        v = ctx.download(f) * 1e9  # several sub-steps
        ctx.upload(f, v)
        fl[f] = torch.from_numpy(np.ascontiguousarray(v).ravel()).to(dev)
    label = torch.from_numpy(np.ascontiguousarray(lab).ravel()).to(dev)
    sat = torch.from_numpy(ctx.download("saturation", padded=True).ravel().copy()).to(dev)
    for call in range(2):
        st, info, msg = _call(L, lab.shape, label, fl["flux_x"], fl["flux_y"], fl["flux_z"], sat, 2.0, p)
        torch.cuda.synchronize()
        assert st == LS_OK, msg
        ref = ctx.saturation(2.0)
        assert info.num_steps == ref["num_steps"] > 1
        assert info.max_rate == ref["max_rate"]
        np.testing.assert_array_equal(sat.cpu().numpy(), ctx.download("saturation", padded=True).ravel(),
                                      err_msg=f"call {call}")
    ctx.close()


def test_noalloc_rejects_domains_above_its_scratch_limit():
    torch = pytest.importorskip("torch")
    L = load()
    t = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = params()
    st, info, msg = _call(L, (600, 600, 600), t, t, t, t, t, 1.0, p)
    assert st == LS_BAD_ARG
    assert "exceed" in msg and "134217728" in msg
