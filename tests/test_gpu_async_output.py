"""Asynchronous output copies (ls_download_fields_async) through the C-ABI.

The copies run on the context's copy stream from the state at the call while later steps go
on; a kernel family that writes a copied field waits on the device for that copy. So the
buffers must hold exactly the state at the call (compared with a twin context that stops
there), and the steps run meanwhile must give exactly the results of a run without output
(compared with a third context). Both the resident and the lean layout (whose snapshot
copies share the copy stream) are covered. The count of non-finite values that decides the
output writer's NaN scrub (src/Simulation.cpp:1487-1517) is checked on planted NaN/Inf.
"""
import numpy as np
import pytest

from helpers import params
from leachingsim_gb300._abi import BC_FLOW_I, MEM_LEAN, MEM_RESIDENT
from leachingsim_gb300.geometry import grf_geometry
from leachingsim_gb300.runtime import Context, load

pytestmark = pytest.mark.gpu

OUT = ["label", "conc", "pressure", "frac", "flux_x", "flux_y", "flux_z", "saturation", "cap_pressure",
       "rel_perm", "permeability", "acid", "precipitate"]


def make(lab, mode):
    p = params(bc_mode=BC_FLOW_I, acid_inlet=1.0, kreac=3.0, time_scalar=20.0, memory_mode=mode)
    g = Context(lab.shape, params=p)
    g.upload("label", lab)
    g.init_all()
    return g


def steps(g, t0, n):
    t = t0
    for _ in range(n):
        ok, _ = g.step(t, 1.0)
        assert ok
        t += 1.0
    return t


def pinned(g, name):
    import torch
    dt = {1: torch.uint8, 2: torch.uint16}.get(g.label_bytes, torch.uint8) if name == "label" else (
        torch.float32 if name in ("frac", "kmult") else torch.float64)
    return torch.empty(g.N, dtype=dt, pin_memory=True).numpy()


@pytest.mark.parametrize("mode", [MEM_RESIDENT, MEM_LEAN], ids=["resident", "lean"])
def test_async_copies_hold_the_state_at_the_call(mode):
    lab, _ = grf_geometry((40, 36, 34), porosity=0.3, corr_len=3.0, mineral_fraction=0.2, seed=9, air_inlet=False)
    a, b, c = make(lab, mode), make(lab, mode), make(lab, mode)
    t = 0.0
    for g in (a, b, c):
        steps(g, t, 3)
    a.props()
    b.props()
    c.props()
    bufs = [pinned(a, f) for f in OUT]
    pend = a.download_async(OUT, bufs)
    t = steps(a, 3.0, 3)  # the copies drain while these steps run
    got = pend.wait()
    for f, v in zip(OUT, got):
        np.testing.assert_array_equal(v.reshape(lab.shape), b.download(f), err_msg=f)
    steps(c, 3.0, 3)
    for f in OUT:
        np.testing.assert_array_equal(a.download(f, padded=True), c.download(f, padded=True), err_msg=f)
    for g in (a, b, c):
        g.close()


def test_count_nonfinite():
    lab, _ = grf_geometry((20, 18, 16), porosity=0.3, corr_len=3.0, mineral_fraction=0.2, seed=4, air_inlet=True)
    g = make(lab, MEM_RESIDENT)
    assert g.count_nonfinite("pressure") == 0
    P = g.download("pressure").copy()
    P.ravel()[[5, 77, 300]] = [np.nan, np.inf, -np.inf]
    g.upload("pressure", P)
    assert g.count_nonfinite("pressure") == 3
    pc = g.download("cap_pressure").copy()
    pc.ravel()[11] = np.nan
    g.upload("cap_pressure", pc)
    assert g.count_nonfinite("cap_pressure") == 1
    g.close()


def test_host_alloc_roundtrip():
    L = load()
    p = L.ls_host_alloc(1 << 20)
    assert p
    L.ls_host_free(p)
