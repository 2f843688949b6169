"""Deferred work against immediate work, through the C-ABI.

* The fluxes of Rock and Precipitate voxels are zeroed after the transport solve
  (src/Simulation.cpp:1134-1149). The library defers that zeroing until the fluxes are
  next read: a transfer, a count, an asynchronous download, a saturation update. A
  saturation update called right after a transport, without a flux evaluation in between,
  must still see the zeros (compared with the oracle, which zeroes at once, bit for bit); a
  voxel that precipitation turns into Precipitate after the solve keeps its flux, as in the
  reference; a rollback must bring back fluxes that read as the zeroed ones of the step it
  returns to.
* Programmatic dependent launch (LS_PDL) changes when kernels are scheduled, not what they
  compute. Runs with it on and off must agree bit for bit, including steps whose pressure
  solves iterate.
"""
import numpy as np
import pytest

from helpers import PORE, PRECIPITATE, ROCK, params, small_grf
from leachingsim_gb300._abi import BC_FLOW_I
from leachingsim_gb300.geometry import grf_geometry
from leachingsim_gb300.runtime import Context

pytestmark = pytest.mark.gpu

FLUX = ("flux_x", "flux_y", "flux_z")


def _pair(oracle_mod, lab, p):
    o = oracle_mod.Oracle(lab.shape, label_bytes=1, params=p, mode=oracle_mod.SOLVE_TIGHT, rtol=1e-14,
                          restart=200, max_it=50000)
    o.load_labels(lab)
    o.init_all()
    g = Context(lab.shape, label_bytes=1, params=p)
    g.upload("label", lab)
    g.init_all()
    rng = np.random.default_rng(3)
    fields = {"saturation": rng.uniform(0.0, 1.0, lab.shape), "conc": rng.uniform(0.0, 1.0, lab.shape)}
    for name, arr in fields.items():
        o.set(name, arr)
        g.upload(name, arr)
    P = rng.normal(0, 100.0, (lab.shape[0] + 1,) + lab.shape[1:])
    o.set("pressure", P, padded=True)
    g.upload("pressure", P, padded=True)
    o.props()
    g.props()
    return o, g


def test_saturation_after_transport_sees_zeroed_solid_fluxes(oracle_mod):
    lab = small_grf((20, 18, 16), seed=5)
    p = params(conc_rtol=1e-13)
    o, g = _pair(oracle_mod, lab, p)
    # the flux inputs from the oracle (its pow-based properties differ in the last bits)
    for f in ("permeability", "viscosity", "cap_pressure"):
        g.upload(f, o.get(f, padded=True), padded=True)
    o.flux()
    g.flux()
    o.transport(0.7, 3)
    g.transport(0.7, 3)
    # no flux evaluation in between: the update reads the zeroed Rock / Precipitate fluxes
    io = o.saturation(2.0)
    ig = g.saturation(2.0)
    assert io["num_steps"] == ig["num_steps"]
    np.testing.assert_array_equal(g.download("saturation", padded=True), o.get("saturation", padded=True))
    for f in FLUX:
        np.testing.assert_array_equal(g.download(f, padded=True), o.get(f, padded=True), err_msg=f)
    g.close()
    o.close()


def test_rollback_brings_back_the_zeroed_fluxes():
    lab = small_grf((16, 14, 12), seed=6)
    p = params()
    a = Context(lab.shape, params=p)
    b = Context(lab.shape, params=p)
    for g in (a, b):
        g.upload("label", lab)
        g.init_all()
        ok, _ = g.step(0.0, 1.0)
        assert ok
    ref = {f: a.download(f, padded=True).copy() for f in FLUX}
    kind = a.download("label")
    solid = np.isin(kind, (ROCK, PRECIPITATE))
    for f in FLUX:
        assert not ref[f][: lab.shape[0]][solid].any(), f
    # b: the next step snapshots the fluxes while their zeroing is still pending, then rolls back
    ok, _ = b.step(1.0, 1.0)
    assert ok
    b.rollback()
    for f in FLUX:
        np.testing.assert_array_equal(b.download(f, padded=True), ref[f], err_msg=f)
    a.close()
    b.close()


def test_voxels_that_precipitate_after_the_transport_keep_their_flux(oracle_mod):
    """Instant precipitation after the transport makes Pore voxels Precipitate. The
    reference zeroed the solid fluxes before that, by the labels of the solve, so those
    voxels keep their flux; the deferred zeroing must work from the same labels."""
    lab = small_grf((20, 18, 16), seed=7)
    p = params(use_instant_precipitation=1, c_sat=0.5, conc_rtol=1e-13, press_rtol=1e-11)
    o = oracle_mod.Oracle(lab.shape, label_bytes=1, params=p, mode=oracle_mod.SOLVE_TIGHT, rtol=1e-14,
                          restart=200, max_it=50000)
    o.load_labels(lab)
    o.init_all()
    g = Context(lab.shape, label_bytes=1, params=p)
    g.upload("label", lab)
    g.init_all()
    conc = np.random.default_rng(4).uniform(0.0, 1.0, lab.shape)  # above c_sat in about half the Pore
    o.set("conc", conc)
    g.upload("conc", conc)
    pore0 = g.download("label") == PORE
    ok_o, io = o.step(0.0, 1.0)
    ok_g, ig = g.step(0.0, 1.0)
    assert ok_o and ok_g
    lab_after = g.download("label")
    np.testing.assert_array_equal(lab_after, o.get("label"))
    became = pore0 & (lab_after == PRECIPITATE)
    assert became.sum() > 0  # the case happens
    for f in FLUX:
        gv, ov = g.download(f), o.get(f)
        np.testing.assert_array_equal(gv == 0.0, ov == 0.0, err_msg=f)
        assert (ov[became] != 0.0).any(), f
        assert np.linalg.norm(gv - ov) <= 1e-9 * np.linalg.norm(ov), f
    g.close()
    o.close()


FIELDS = ("label", "frac", "pressure", "saturation", "conc", "acid", "precipitate") + FLUX


def _run(lab, p, steps):
    g = Context(lab.shape, params=p)
    g.upload("label", lab)
    g.init_all()
    its = []
    for n in range(steps):
        ok, info = g.step(float(n), 1.0)
        assert ok
        its.append(info["pressure"]["iterations"])
    out = {f: g.download(f, padded=True).copy() for f in FIELDS}
    g.close()
    return out, its


def test_programmatic_dependent_launch_changes_no_result(monkeypatch):
    lab, _ = grf_geometry((48, 40, 40), porosity=0.3, corr_len=3.0, mineral_fraction=0.2, seed=8,
                          air_inlet=False)
    p = params(bc_mode=BC_FLOW_I, acid_inlet=1.0, kreac=2.0, time_scalar=5.0)
    monkeypatch.setenv("LS_PDL", "1")
    on, its_on = _run(lab, p, 4)
    monkeypatch.setenv("LS_PDL", "0")
    off, its_off = _run(lab, p, 4)
    assert its_on == its_off and sum(its_on) > 0  # the pressure solves iterate
    for f in FIELDS:
        np.testing.assert_array_equal(on[f], off[f], err_msg=f)
