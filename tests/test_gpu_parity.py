"""CUDA path against the CPU oracle (and the direct-solve twin) through the C-ABI.

Each kernel is isolated by uploading the oracle's inputs, so that arithmetic
without transcendental functions can be required to match bit for bit.
Tolerances, where not exact:
  * props (CUDA pow/sqrt against glibc pow; the n = 2 van Genuchten exponents are
    evaluated with sqrt and products): 1e-13 relative
  * pressure solutions: the Pore system is conditioned near 1e18; rel-L2 1e-7 for
    the full field against a direct solve, 1e-8 Jacobi-scaled residual
  * transport solutions: rel-L2 1e-9 against a direct solve
"""
import numpy as np
import pytest

from helpers import case, params, random_labels, rel_l2, small_grf
from leachingsim_gb300 import _abi
from leachingsim_gb300.runtime import Context
from twin import Twin

pytestmark = pytest.mark.gpu

GEOMS = [
    ("random8", lambda: random_labels((17, 13, 11), 1), 1),
    ("random_u16", lambda: random_labels((12, 11, 13), 2, values=(0, 1, 2, 3, 4, 5, 9),
                                         dtype=np.uint16), 2),
    ("grf", lambda: small_grf((20, 18, 16), seed=5), 1),
    ("case0", lambda: case(24, 0), 1),
    ("case1", lambda: case(24, 1), 1),
]


def pair(oracle_mod, lab, p, lb, seed=0, randomize=True):
    o = oracle_mod.Oracle(lab.shape, label_bytes=lb, params=p, mode=oracle_mod.SOLVE_TIGHT,
                          rtol=1e-14, restart=200, max_it=50000)
    o.load_labels(lab)
    o.init_all()
    g = Context(lab.shape, label_bytes=lb, params=p)
    g.upload("label", lab)
    g.init_all()
    if randomize:
        rng = np.random.default_rng(seed)
        shp = lab.shape
        fields = {
            "saturation": rng.uniform(0.0, 1.0, shp),
            "precipitate": rng.uniform(-0.2, 1.2, shp),
            "frac": rng.uniform(0.0, 1.0, shp).astype(np.float32),
        }
        for name, arr in fields.items():
            o.set(name, arr)
            g.upload(name, arr)
        P = rng.normal(0, 100.0, (shp[0] + 1,) + shp[1:])
        o.set("pressure", P, padded=True)
        g.upload("pressure", P, padded=True)
        o.props()
        g.props()
    return o, g


def copy_fields(o, g, names, padded=True):
    for n in names:
        g.upload(n, o.get(n, padded=padded), padded=padded)


@pytest.mark.parametrize("name,geom,lb", GEOMS)
def test_props(oracle_mod, name, geom, lb):
    lab = geom()
    o, g = pair(oracle_mod, lab, params(), lb, seed=11)
    for f in ("rel_perm", "cap_pressure", "permeability"):
        np.testing.assert_allclose(g.download(f), o.get(f), rtol=1e-13, atol=0, err_msg=f)
    np.testing.assert_array_equal(g.download("viscosity"), o.get("viscosity"))
    g.close()


@pytest.mark.parametrize("name,geom,lb", GEOMS)
def test_flux_saturation_surface_exact(oracle_mod, name, geom, lb):
    lab = geom()
    o, g = pair(oracle_mod, lab, params(evaporative_flux=2e-3), lb, seed=13)
    copy_fields(o, g, ["permeability", "viscosity", "cap_pressure"])
    o.flux()
    g.flux()
    for f in ("flux_x", "flux_y", "flux_z"):
        np.testing.assert_array_equal(g.download(f), o.get(f), err_msg=f)
    for f in ("flux_x", "flux_y", "flux_z"):
        v = o.get(f) * 1e9
        o.set(f, v)
        g.upload(f, v)
    io = o.saturation(2.0)
    ig = g.saturation(2.0)
    assert io["num_steps"] == ig["num_steps"]
    assert io["max_rate"] == ig["max_rate"]
    np.testing.assert_array_equal(g.download("saturation", padded=True),
                                  o.get("saturation", padded=True))
    o.surface()
    g.surface()
    np.testing.assert_array_equal(g.download("label"), o.get("label"))
    np.testing.assert_array_equal(g.download("conc"), o.get("conc"))
    g.close()


@pytest.mark.parametrize("name,geom,lb", GEOMS)
def test_pressure_operator_exact(oracle_mod, name, geom, lb):
    lab = geom()
    o, g = pair(oracle_mod, lab, params(evaporative_flux=1e-7), lb, seed=12)
    copy_fields(o, g, ["permeability", "viscosity"])
    x = np.random.default_rng(3).normal(size=lab.size)
    for t in (0.0, 1800.0, 7200.0):
        o.setup_pressure(t)
        g.pressure_setup(t)
        np.testing.assert_array_equal(g.pressure_rhs(), o.pressure_rhs())
        np.testing.assert_array_equal(g.pressure_apply(x), o.pressure_apply(x))
    g.close()


@pytest.mark.parametrize("solver", [_abi.PRESS_JACOBI64, _abi.PRESS_FP64, _abi.PRESS_MIXED])
@pytest.mark.parametrize("name,geom,lb", GEOMS)
def test_pressure_solve(oracle_mod, name, geom, lb, solver):
    lab = geom()
    p = params(press_solver=solver, press_rtol=1e-10)
    o, g = pair(oracle_mod, lab, p, lb, seed=12, randomize=False)
    tw = Twin(lab, p)
    tw.init_all()
    for t in (600.0, 3600.0):
        ok, info = g.pressure(t)
        assert ok, info
        assert info["rel_residual"] <= 1e-10
        tw.pressure(t)
        P = g.download("pressure", padded=True)
        assert rel_l2(P, tw.P) < 1e-7, (t, rel_l2(P, tw.P))
    g.close()


@pytest.mark.parametrize("which", [3, 1])
@pytest.mark.parametrize("theta", [1.0, 0.5])
@pytest.mark.parametrize("name,geom,lb", GEOMS)
def test_transport_operator_and_solve(oracle_mod, name, geom, lb, theta, which):
    """which = 3: conc and acid as one two-right-hand-side solve; which = 1: conc alone (the
    single-right-hand-side kernels, paired-row when the row length K is even)."""
    lab = geom()
    p = params(theta=theta, alpha_transfer=0.3, Dpore_fac=2.0, conc_rtol=1e-13)
    o, g = pair(oracle_mod, lab, p, lb, seed=14)
    rng = np.random.default_rng(5)
    tw = Twin(lab, p)
    I = lab.shape[0]
    for f, tf in (("flux_x", tw.fx), ("flux_y", tw.fy), ("flux_z", tw.fz), ("conc", tw.conc),
                  ("acid", tw.acid)):
        v = rng.normal(0, 1.0, (I + 1,) + lab.shape[1:])
        o.set(f, v, padded=True)
        g.upload(f, v, padded=True)
        tf[:] = v
    tw.label[:I] = o.get("label")
    x = rng.normal(size=lab.size)
    o.setup_transport(0.7, 0)
    np.testing.assert_array_equal(g.transport_apply(0.7, x), o.transport_apply(x))
    acid_before = g.download("acid", padded=True)
    ok, ci, ai = g.transport(0.7, which)
    assert ok, (ci, ai)
    tw.transport(0.7)
    assert rel_l2(g.download("conc", padded=True), tw.conc) < 1e-9
    if which == 3:
        assert rel_l2(g.download("acid", padded=True), tw.acid) < 1e-9
    else:
        np.testing.assert_array_equal(g.download("acid", padded=True), acid_before)
    for f, tf in (("flux_x", tw.fx), ("flux_y", tw.fy), ("flux_z", tw.fz)):
        np.testing.assert_array_equal(g.download(f, padded=True), tf)
    g.close()


@pytest.mark.parametrize("name,geom,lb", GEOMS)
def test_precip_exact(oracle_mod, name, geom, lb):
    lab = geom()
    for instant in (0, 1):
        p = params(use_instant_precipitation=instant, solid_density=0.3, c_sat=0.6)
        o, g = pair(oracle_mod, lab, p, lb, seed=15)
        c = np.random.default_rng(6).uniform(0, 1.5, lab.shape)
        o.set("conc", c)
        g.upload("conc", c)
        o.precip()
        g.precip()
        for f in ("label", "conc", "precipitate"):
            np.testing.assert_array_equal(g.download(f), o.get(f), err_msg=f)
        g.close()


@pytest.mark.parametrize("name,geom,lb", GEOMS)
def test_dissolve_exact(oracle_mod, name, geom, lb):
    """Wavefront-parallel dissolution reproduces the sequential sweep bit for bit."""
    lab = geom()
    o, g = pair(oracle_mod, lab, params(kreac=50.0, time_scalar=3.0), lb, seed=16)
    acid = np.random.default_rng(7).uniform(0, 2.0, lab.shape)
    frac = np.where(lab == 4, np.random.default_rng(8).uniform(0, 0.3, lab.shape), 0.0).astype(np.float32)
    for n, a in (("acid", acid), ("frac", frac)):
        o.set(n, a)
        g.upload(n, a)
    copy_fields(o, g, ["conc", "precipitate"])
    no, io = o.dissolve(0.9)
    ng, ig = g.dissolve(0.9)
    assert (no, io["num_steps"]) == (ng, ig["num_steps"])
    assert io["max_rate"] == ig["max_rate"]
    for f in ("frac", "acid", "label", "conc", "precipitate"):
        np.testing.assert_array_equal(g.download(f), o.get(f), err_msg=f)
    g.close()


def test_dissolve_no_acid_is_identity(oracle_mod):
    lab = small_grf((16, 16, 16), seed=2)
    o, g = pair(oracle_mod, lab, params(), 1, randomize=False)
    before = {f: g.download(f) for f in ("frac", "label", "acid")}
    n, info = g.dissolve(1.0)
    assert n == 0 and info["num_steps"] == 1
    for f, v in before.items():
        np.testing.assert_array_equal(g.download(f), v)
    g.close()


# Pressure tolerance per inner precision: the FP64 residual meets rtol either way, but
# components of the error in near-null modes (clusters anchored only by weak links) are
# invisible to it and sit at the inner solver's precision.
@pytest.mark.parametrize("solver,ptol", [(_abi.PRESS_MIXED, 1e-6), (_abi.PRESS_FP64, 1e-7)])
@pytest.mark.parametrize("shift", [1, 0])
@pytest.mark.parametrize("name,geom,lb", GEOMS[2:])
def test_steps_against_twin(oracle_mod, name, geom, lb, shift, solver, ptol):
    lab = geom()
    p = params(compat_shift=shift, press_rtol=1e-11, conc_rtol=1e-13, press_solver=solver)
    g = Context(lab.shape, label_bytes=lb, params=p)
    g.upload("label", lab)
    g.init_all()
    tw = Twin(lab, p)
    tw.init_all()
    for n in range(5):
        ok, info = g.step(float(n), 1.0)
        assert ok, info
        tw.step(float(n), 1.0)
        np.testing.assert_array_equal(g.download("label"), tw.label[:lab.shape[0]])
        assert rel_l2(g.download("pressure", padded=True), tw.P) < ptol
        assert rel_l2(g.download("saturation", padded=True), tw.sat) < 1e-9
        assert rel_l2(g.download("conc", padded=True), tw.conc) < 1e-9
    g.close()


def test_steps_against_oracle_with_acid(oracle_mod):
    """Restart-style state with acid present (the reference's acid field has no source in
    a fresh run): several full steps, dissolution active."""
    lab = small_grf((20, 16, 16), seed=4)
    p = params(kreac=5.0, time_scalar=100.0, press_rtol=1e-11, conc_rtol=1e-13)
    o, g = pair(oracle_mod, lab, p, 1, randomize=False)
    acid = np.random.default_rng(1).uniform(0.0, 1.0, lab.shape)
    o.set("acid", acid)
    g.upload("acid", acid)
    total_o = total_g = 0
    for n in range(4):
        ok_o, io = o.step(float(n), 1.0)
        ok_g, ig = g.step(float(n), 1.0)
        assert ok_o and ok_g
        total_o += io["leached"]
        total_g += ig["leached"]
        assert io["leaching"]["num_steps"] == ig["leaching"]["num_steps"]
        np.testing.assert_array_equal(g.download("label"), o.get("label"))
        assert rel_l2(g.download("acid", padded=True), o.get("acid", padded=True)) < 1e-9
        assert rel_l2(g.download("frac"), o.get("frac")) < 1e-6
    assert total_o == total_g
    g.close()


def test_snapshot_rollback(oracle_mod):
    lab = small_grf((16, 14, 12), seed=6)
    g = Context(lab.shape, params=params())
    g.upload("label", lab)
    g.init_all()
    g.step(0.0, 1.0)
    names = ["label", "frac", "precipitate", "saturation", "pressure", "conc", "acid",
             "flux_x", "flux_y", "flux_z"]
    g.snapshot()
    before = {n: g.download(n, padded=True) for n in names}
    g.step(1.0, 1.0)   # snapshots again, then changes the state
    g.rollback()
    for n in names:
        np.testing.assert_array_equal(g.download(n, padded=True), before[n], err_msg=n)
    g.close()


@pytest.mark.parametrize("name,geom,lb", GEOMS[2:4])
def test_implicit_saturation(oracle_mod, name, geom, lb):
    lab = geom()
    p = params(use_implicit_saturation=1, press_rtol=1e-11, sat_rtol=1e-13, conc_rtol=1e-13)
    o, g = pair(oracle_mod, lab, p, lb, randomize=False)
    for n in range(2):
        ok_o, io = o.step(float(n), 1.0)
        ok_g, ig = g.step(float(n), 1.0)
        assert ok_o == ok_g
        if not ok_o:
            o.restore_state()
            g.rollback()
            continue
        np.testing.assert_array_equal(g.download("label"), o.get("label"))
        assert rel_l2(g.download("saturation", padded=True), o.get("saturation", padded=True)) < 1e-7
    g.close()


def test_bad_arguments_report_errors():
    g = Context((8, 8, 8))
    with pytest.raises(Exception):
        g.upload("saturation", np.zeros(10))
    with pytest.raises(Exception):
        g.saturation(-1.0)
    g.close()
