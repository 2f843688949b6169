"""The flow-through boundary model, the permeability parameters and the FP64 step budget on
the GPU against the oracle, through the C-ABI.

The flow-through model (bc_mode = BC_FLOW_I; no counterpart in the reference, whose only
pressure driver is the ramped Air surface of src/Simulation.cpp:662-720) holds the Pore
voxels of plane i = 0 at p_inlet and of plane i = I-1 at p_outlet, and the fluid voxels of
plane i = 0 at conc_inlet / acid_inlet in the transport systems.

Tolerances:
  * assembled operators and right-hand sides: bit for bit (A x, b);
  * props with the permeability parameters and the multiplier: 1e-13 relative (pow);
  * whole runs at FP64 settings (FP64 inner multigrid-PCG to rtol 1e-12, transport rtol
    1e-13) against the oracle at rtol 1e-13: labels exact, pressure, velocity (the three
    face fluxes), concentration, acid and precipitate within rel-L2 1e-8;
  * the mixed-precision settings (FP32 inner solves, FP64 refinement to rtol 1e-8):
    pressure and velocity within 1e-6;
  * budget sums against the oracle's: 1e-12 relative (reduction order), counts exact.
"""
import numpy as np
import pytest

from helpers import params, rel_l2
from leachingsim_gb300 import _abi
from leachingsim_gb300._abi import BC_FLOW_I
from leachingsim_gb300.geometry import grf_geometry
from leachingsim_gb300.runtime import Context

pytestmark = pytest.mark.gpu

FIELDS = ("pressure", "flux_x", "flux_y", "flux_z", "conc", "acid", "precipitate")


def flow_geometry(shape, seed=0, porosity=0.30, corr_len=4.0, label_dtype=np.uint8):
    lab, _ = grf_geometry(shape, porosity=porosity, corr_len=corr_len, mineral_fraction=0.15, seed=seed,
                          air_inlet=False, dtype=label_dtype)
    return lab


def make_pair(oracle_mod, lab, p, lb=1, mode=None):
    o = oracle_mod.Oracle(lab.shape, label_bytes=lb, params=p,
                          mode=oracle_mod.SOLVE_PCG if mode is None else mode, rtol=1e-13, restart=200,
                          max_it=200000)
    o.load_labels(lab)
    o.init_all()
    g = Context(lab.shape, label_bytes=lb, params=p)
    g.upload("label", lab)
    g.init_all()
    return o, g


@pytest.mark.parametrize("lb", [1, 2])
def test_flow_operators_exact(oracle_mod, lb):
    lab = flow_geometry((18, 16, 14), seed=3, corr_len=2.0, label_dtype=np.uint8 if lb == 1 else np.uint16)
    p = params(bc_mode=BC_FLOW_I, p_inlet=1.5, p_outlet=0.25, conc_inlet=0.3, acid_inlet=0.8,
               pore_permeability=4e-12, rock_permeability=3e-17, alpha_transfer=0.2)
    o, g = make_pair(oracle_mod, lab, p, lb)
    rng = np.random.default_rng(7)
    km = np.where(rng.uniform(size=lab.shape) < 0.3, 1e4, 1.0).astype(np.float32)
    sat = rng.uniform(0.0, 1.0, lab.shape)
    for a in (o, g):
        (a.set if a is o else a.upload)("kmult", km)
        (a.set if a is o else a.upload)("saturation", sat)
        a.props()
    np.testing.assert_allclose(g.download("permeability"), o.get("permeability"), rtol=1e-13, atol=0)
    np.testing.assert_array_equal(g.download("kmult"), km)
    # exact operators on identical coefficients
    for f in ("permeability", "viscosity"):
        g.upload(f, o.get(f, padded=True), padded=True)
    x = rng.normal(size=lab.size)
    for t in (0.0, 7200.0):
        o.setup_pressure(t)
        g.pressure_setup(t)
        np.testing.assert_array_equal(g.pressure_rhs(), o.pressure_rhs())
        np.testing.assert_array_equal(g.pressure_apply(x), o.pressure_apply(x))
    I = lab.shape[0]
    for f in ("flux_x", "flux_y", "flux_z", "conc", "acid"):
        v = rng.normal(0, 1.0, (I + 1,) + lab.shape[1:])
        o.set(f, v, padded=True)
        g.upload(f, v, padded=True)
    o.setup_transport(0.7, 0)
    np.testing.assert_array_equal(g.transport_apply(0.7, x), o.transport_apply(x))
    # a two-right-hand-side solve: the inflow rows hold their values exactly
    ok, ci, ai = g.transport(0.7, 3)
    assert ok, (ci, ai)
    okc, _ = o.transport(0.7, 0)
    oka, _ = o.transport(0.7, 1)
    assert okc and oka
    for f in ("conc", "acid"):
        assert rel_l2(g.download(f, padded=True), o.get(f, padded=True)) < 1e-9, f
    conc = g.download("conc", padded=True)
    acid = g.download("acid", padded=True)
    fluid0 = (lab[0] == 2) | (lab[0] == 1)
    sh = 1  # compat_shift: row (0, j, k) lands in slot plane 1
    assert np.all(conc[sh][fluid0] == 0.3) and np.all(acid[sh][fluid0] == 0.8)
    g.close()
    o.close()


def _run_pair(oracle_mod, lab, p, steps, compare_at, tol):
    o, g = make_pair(oracle_mod, lab, p)
    errs = []
    for n in range(steps):
        ok_o, io = o.step(float(n), 1.0)
        ok_g, ig = g.step(float(n), 1.0)
        assert ok_o and ok_g, (io, ig)
        assert ig["leached"] == io["leached"]
        if n + 1 in compare_at:
            np.testing.assert_array_equal(g.download("label"), o.get("label").astype(lab.dtype))
            e = {f: rel_l2(g.download(f, padded=True), o.get(f, padded=True)) for f in FIELDS}
            errs.append((n + 1, e))
            for f in FIELDS:
                assert e[f] < tol[f], (n + 1, f, e)
    return o, g, errs


def test_c1_plain_configuration(oracle_mod):
    """The plain-method configuration exactly: 64^3 uint8 Gaussian random field (porosity
    0.30, correlation length 4, 15% of the solid reactive mineral, percolating along z), the
    flow-through pressure P = 1 at z = 0 and P = 0 at z = max with no-flow sides, FP64 solves,
    D = 1, kreac = 1, dt = 1, tmax = 10 (ten steps); outputs every nout = 5 steps are where the
    fields are compared (after steps 5 and 10), plus after step 1."""
    lab = flow_geometry((64, 64, 64), seed=0)
    p = params(bc_mode=BC_FLOW_I, p_inlet=1.0, p_outlet=0.0, D=1.0, kreac=1.0,
               press_solver=_abi.PRESS_FP64, press_rtol=1e-12, conc_rtol=1e-13)
    tol = {f: 1e-8 for f in FIELDS}
    o, g, errs = _run_pair(oracle_mod, lab, p, 10, (1, 5, 10), tol)
    print("c1_fp64", errs)
    g.close()
    o.close()


def test_c1_mixed_precision(oracle_mod):
    """The same configuration with the mixed-precision solvers (FP32 inner PCG/multigrid,
    FP64 refinement to rtol 1e-8): pressure and velocity within 1e-6 of the FP64 oracle."""
    lab = flow_geometry((64, 64, 64), seed=0)
    p = params(bc_mode=BC_FLOW_I, press_solver=_abi.PRESS_MIXED, press_rtol=1e-8, conc_rtol=1e-8)
    tol = {f: 1e-6 for f in FIELDS}
    o, g, errs = _run_pair(oracle_mod, lab, p, 10, (1, 10), tol)
    print("c1_mixed", errs)
    g.close()
    o.close()


def test_acid_inflow_run_and_budget(oracle_mod):
    """Acid flowing in at the inlet plane dissolves mineral: ten steps at FP64 settings with
    the fields, the leached counts and the FP64 budget of every step against the oracle."""
    lab = flow_geometry((32, 28, 30), seed=4, corr_len=3.0)
    p = params(bc_mode=BC_FLOW_I, acid_inlet=1.0, kreac=2.0, time_scalar=3.0, press_solver=_abi.PRESS_FP64,
               press_rtol=1e-12, conc_rtol=1e-13)
    o, g = make_pair(oracle_mod, lab, p)
    leached = 0
    for n in range(10):
        ok_o, io = o.step(float(n), 1.0)
        ok_g, ig = g.step(float(n), 1.0)
        assert ok_o and ok_g
        assert ig["leached"] == io["leached"]
        leached += ig["leached"]
        bo, bg = io["budget"], ig["budget"]
        for k in ("sulphide_voxels", "precipitate_voxels"):
            assert bg[k] == bo[k], (n, k)
        for k in ("conc", "acid", "mineral", "precipitate", "acid_consumed", "mineral_dissolved"):
            assert abs(bg[k] - bo[k]) <= 1e-12 * max(1.0, abs(bo[k])), (n, k, bg[k], bo[k])
    assert leached > 0
    np.testing.assert_array_equal(g.download("label"), o.get("label").astype(np.uint8))
    for f in FIELDS:
        assert rel_l2(g.download(f, padded=True), o.get(f, padded=True)) < 1e-8, f
    g.close()
    o.close()


def test_reference_model_untouched(oracle_mod):
    """bc_mode 0 (the default) with the default permeabilities: an Air-inlet geometry gives
    the same assembled pressure system as before the parameters existed (no identity rows for
    Pore voxels on the end planes)."""
    lab, _ = grf_geometry((16, 14, 12), porosity=0.35, corr_len=2.0, mineral_fraction=0.2, seed=1,
                          air_inlet=True)
    p = params()
    o, g = make_pair(oracle_mod, lab, p)
    o.setup_pressure(0.0)
    g.pressure_setup(0.0)
    kind = o.pressure_rowkind().reshape(lab.shape)
    assert np.all(kind[lab == 2] == 2)
    x = np.random.default_rng(2).normal(size=lab.size)
    np.testing.assert_array_equal(g.pressure_rhs(), o.pressure_rhs())
    np.testing.assert_array_equal(g.pressure_apply(x), o.pressure_apply(x))
    g.close()
    o.close()
