"""The lean device layout (memory_mode = MEM_LEAN) against the resident one, through the C-ABI.

The lean layout releases the pressure solve's work arrays before each transport solve and
the transport's before each pressure assembly (through a stream-ordered pool that keeps the
memory), recomputes every voxel of the per-voxel FP64 kernels instead of tracking changes,
and keeps the retry snapshot (src/Simulation.cpp:2312-2353) in host memory. None of that
changes an arithmetic operation, so whole runs must match the resident layout bit for bit,
and a rollback must restore every field bit for bit. Its footprint is checked against the
bytes per voxel the layout is built for.
"""
import numpy as np
import pytest
import torch

from helpers import params
from leachingsim_gb300._abi import BC_FLOW_I, MEM_LEAN, MEM_RESIDENT, PRESS_FP64, PRESS_MIXED
from leachingsim_gb300.geometry import grf_geometry
from leachingsim_gb300.runtime import Context, LsError

pytestmark = pytest.mark.gpu

STATE = ("label", "frac", "precipitate", "saturation", "pressure", "conc", "acid", "flux_x", "flux_y", "flux_z",
         "permeability", "viscosity", "cap_pressure", "rel_perm")


def geometry(shape, seed, air, dtype=np.uint8):
    lab, _ = grf_geometry(shape, porosity=0.3, corr_len=3.0, mineral_fraction=0.2, seed=seed, air_inlet=air,
                          dtype=dtype)
    return lab


def run(lab, p, steps, kmult=None, lb=1):
    g = Context(lab.shape, label_bytes=lb, params=p)
    g.upload("label", lab)
    if kmult is not None:
        g.upload("kmult", kmult)
    g.init_all()
    infos = []
    t = 0.0
    for _ in range(steps):
        ok, info = g.step(t, 1.0)
        assert ok
        infos.append(info)
        t += 1.0
    out = {f: g.download(f, padded=True).copy() for f in STATE}
    return g, out, infos


CASES = [
    # flow-through model with acid inflow and a 1e4 permeability contrast, mixed precision
    ("flow_mixed", dict(bc_mode=BC_FLOW_I, acid_inlet=1.0, kreac=2.0, time_scalar=5.0, press_solver=PRESS_MIXED),
     False, True, 1),
    # the reference's Air-inlet model at FP64 settings, uint16 labels
    ("reference_fp64", dict(press_solver=PRESS_FP64, press_rtol=1e-12, conc_rtol=1e-12, kreac=3.0,
                            evaporative_flux=1e-7), True, False, 2),
]


@pytest.mark.parametrize("name,kw,air,contrast,lb", CASES, ids=[c[0] for c in CASES])
def test_lean_matches_resident_bit_for_bit(name, kw, air, contrast, lb):
    shape = (40, 36, 34)
    lab = geometry(shape, 5, air, np.uint8 if lb == 1 else np.uint16)
    km = None
    if contrast:
        rng = np.random.default_rng(2)
        km = np.where(rng.uniform(size=shape) < 0.05, 1e4, 1.0).astype(np.float32)
    res_ctx, res, res_info = run(lab, params(memory_mode=MEM_RESIDENT, **kw), 5, km, lb)
    lean_ctx, lean, lean_info = run(lab, params(memory_mode=MEM_LEAN, **kw), 5, km, lb)
    for f in STATE:
        np.testing.assert_array_equal(lean[f], res[f], err_msg=f)
    for a, b in zip(res_info, lean_info):
        assert a["pressure"]["iterations"] == b["pressure"]["iterations"]
        assert a["leached"] == b["leached"]
        assert a["budget"] == b["budget"]
    if name == "flow_mixed":
        assert sum(i["budget"]["acid_consumed"] for i in res_info) > 0  # the dissolution sweep ran
    # the lean snapshot lives on the host; the resident one on the device
    assert lean_ctx.host_bytes() > 0 and res_ctx.host_bytes() == 0
    res_ctx.close()
    lean_ctx.close()


def test_lean_rollback_restores_every_field():
    lab = geometry((24, 22, 20), 3, True)
    g = Context(lab.shape, params=params(memory_mode=MEM_LEAN, press_max_it=1, press_rtol=1e-12))
    g.upload("label", lab)
    g.init_all()
    ok, _ = g.step(0.0, 1.0)  # t = 0: the ramp's first pressure is tiny but nonzero
    before = {f: g.download(f, padded=True).copy() for f in STATE}
    ok, info = g.step(1.0, 1.0)
    assert not ok and info["pressure"]["converged"] == 0
    g.rollback()
    for f in STATE:
        np.testing.assert_array_equal(g.download(f, padded=True), before[f], err_msg=f)
    g.set_params(params(memory_mode=MEM_LEAN, press_rtol=1e-12))
    ok, _ = g.step(1.0, 1.0)
    assert ok
    g.close()


def test_lean_footprint_and_fixed_mode():
    """Device bytes per voxel: the lean layout's peak within 300 B/voxel for uint16 labels, the
    multiplier and mixed precision (~285 expected), against ~620 for the resident layout, and
    the device's free memory agreeing with it; the pressure system stays readable until the
    next transport solve; the memory mode cannot change after creation."""
    shape = (128, 128, 128)
    lab = geometry(shape, 7, False, np.uint16)
    km = np.ones(shape, np.float32)
    p = dict(bc_mode=BC_FLOW_I, acid_inlet=1.0, press_solver=PRESS_MIXED)
    peaks = {}
    for mode in (MEM_RESIDENT, MEM_LEAN):
        free0 = torch.cuda.mem_get_info()[0]
        g, _, _ = run(lab, params(memory_mode=mode, **p), 2, km, lb=2)
        peaks[mode] = g.device_peak_bytes() / lab.size
        # what the device lost is what the context holds (up to the allocation granularity)
        held = free0 - torch.cuda.mem_get_info()[0]
        assert abs(held - g.device_bytes()) < 160e6 + 0.05 * g.device_bytes(), (held, g.device_bytes())
        if mode == MEM_LEAN:
            with pytest.raises(LsError):
                g.set_params(params(memory_mode=MEM_RESIDENT, **p))
            g.pressure_setup(0.0)
            b = g.pressure_rhs()
            assert np.isfinite(b).all()
            g.transport_apply(1.0, np.zeros(lab.size))  # the transport takes the memory back
            with pytest.raises(LsError):
                g.pressure_rhs()
        g.close()
    assert peaks[MEM_LEAN] < 300.0, peaks
    assert peaks[MEM_RESIDENT] > 1.8 * peaks[MEM_LEAN], peaks
