"""The flow-through boundary model, the permeability parameters and the FP64 step budget
in the oracle (CPU).

The flow-through model (bc_mode = BC_FLOW_I) has no counterpart in the reference, whose
only pressure driver is the ramped Air surface (src/Simulation.cpp:662-720): the Pore
voxels of the planes i = 0 and i = I-1 hold p_inlet and p_outlet, the fluid voxels of plane
i = 0 hold conc_inlet / acid_inlet in the transport systems. Everything else is the
reference's; the reference model stays the default.
"""
import numpy as np

from helpers import params
from leachingsim_gb300._abi import BC_FLOW_I
from leachingsim_gb300.geometry import grf_geometry

PORE, SULPHIDE = 2, 4


def flow_case(n=(16, 14, 12), seed=2):
    lab, _ = grf_geometry(n, porosity=0.3, corr_len=2.0, mineral_fraction=0.15, seed=seed, air_inlet=False)
    return lab


def test_flow_rows(oracle_mod):
    lab = flow_case()
    p = params(bc_mode=BC_FLOW_I, p_inlet=2.5, p_outlet=0.5, acid_inlet=0.7, conc_inlet=0.2)
    o = oracle_mod.Oracle(lab.shape, params=p, mode=oracle_mod.SOLVE_TIGHT)
    o.load_labels(lab)
    o.init_all()
    o.setup_pressure(0.0)
    kind = o.pressure_rowkind().reshape(lab.shape)
    b = o.pressure_rhs().reshape(lab.shape)
    pore = lab == PORE
    assert np.all(kind[0][pore[0]] == 1) and np.all(kind[-1][pore[-1]] == 1)
    assert np.all(b[0][pore[0]] == 2.5) and np.all(b[-1][pore[-1]] == 0.5)
    assert np.all(kind[1:-1][pore[1:-1]] == 2)
    # transport: identity rows holding the inflow value on the fluid voxels of plane 0
    for which, val in ((0, 0.2), (1, 0.7)):
        o.setup_transport(1.0, which)
        bt = o.transport_rhs().reshape(lab.shape)
        assert np.all(bt[0][pore[0]] == val)
        x = np.random.default_rng(1).normal(size=lab.size)
        y = o.transport_apply(x).reshape(lab.shape)
        np.testing.assert_array_equal(y[0][pore[0]], x.reshape(lab.shape)[0][pore[0]])
    o.close()


def test_reference_model_unchanged_by_default(oracle_mod):
    """Default parameters keep the reference's model: no identity rows for Pore voxels."""
    lab = flow_case()
    o = oracle_mod.Oracle(lab.shape, params=params(), mode=oracle_mod.SOLVE_TIGHT)
    o.load_labels(lab)
    o.init_all()
    o.setup_pressure(0.0)
    kind = o.pressure_rowkind().reshape(lab.shape)
    assert np.all(kind[lab == PORE] == 2)
    o.close()


def test_permeability_parameters_and_multiplier(oracle_mod):
    lab = flow_case()
    rng = np.random.default_rng(4)
    o0 = oracle_mod.Oracle(lab.shape, params=params(), mode=oracle_mod.SOLVE_TIGHT)
    o1 = oracle_mod.Oracle(lab.shape, params=params(pore_permeability=3e-11, rock_permeability=2e-16),
                           mode=oracle_mod.SOLVE_TIGHT)
    km = np.where(rng.uniform(size=lab.shape) < 0.2, 1e4, 1.0).astype(np.float32)
    for o in (o0, o1):
        o.load_labels(lab)
        o.init_all()
        o.set("saturation", np.full(lab.shape, 0.6))
    o1.set("kmult", km)
    o0.props()
    o1.props()
    k0, k1 = o0.get("permeability"), o1.get("permeability")
    kr = o0.get("rel_perm")
    rock = lab == 3
    np.testing.assert_array_equal(k0[rock], 1e-18 * np.maximum(kr[rock], 1e-15))
    np.testing.assert_array_equal(k1[rock], (2e-16 * km[rock].astype(np.float64)) * np.maximum(kr[rock], 1e-15))
    pore = lab == PORE
    np.testing.assert_allclose(k1[pore], 3e-11 * km[pore].astype(np.float64) * np.maximum(kr[pore], 1e-15),
                               rtol=1e-14)
    o0.close()
    o1.close()


def test_budget_closure_with_acid_inflow(oracle_mod):
    """Ten steps with acid flowing in: the FP64 budget's sums equal the fields' sums, the
    mineral the dissolution sweep removes equals the acid it consumes (times time_scalar) to
    the FP32 rounding of frac in steps where no voxel reaches the leach threshold; a leached
    voxel consumes acid for its whole last sub-step loss (<= 0.1, possibly past zero) and
    keeps none of the remainder (<= 1e-4) it had at the threshold."""
    lab = flow_case((20, 16, 16), seed=5)
    p = params(bc_mode=BC_FLOW_I, acid_inlet=1.0, kreac=2.0, time_scalar=3.0)
    o = oracle_mod.Oracle(lab.shape, params=p, mode=oracle_mod.SOLVE_PCG, rtol=1e-13)
    o.load_labels(lab)
    o.init_all()
    prev_frac = o.get("frac").astype(np.float64).sum()
    leached_any = consumed_any = False
    for n in range(10):
        ok, info = o.step(float(n), 1.0)
        assert ok
        b = info["budget"]
        assert abs(b["conc"] - o.get("conc").sum()) <= 1e-12 * max(1.0, abs(b["conc"]))
        assert abs(b["acid"] - o.get("acid").sum()) <= 1e-12 * max(1.0, abs(b["acid"]))
        frac = o.get("frac").astype(np.float64).sum()
        assert abs(b["mineral"] - frac) <= 1e-12 * max(1.0, frac)
        assert abs(b["mineral_dissolved"] - (prev_frac - frac)) <= 1e-9 * max(1.0, prev_frac)
        assert b["sulphide_voxels"] == int((o.get("label") == SULPHIDE).sum())
        diff = b["mineral_dissolved"] - 3.0 * b["acid_consumed"]
        if info["leached"] == 0:
            assert abs(diff) <= 1e-6 * max(1e-12, b["mineral_dissolved"]) + 1e-9
        else:
            leached_any = True
            assert -0.1 * info["leached"] - 1e-9 <= diff <= 1e-4 * info["leached"] + 1e-6 * b["mineral_dissolved"]
        consumed_any |= b["acid_consumed"] > 0
        prev_frac = frac
    assert consumed_any and leached_any
    o.close()
