"""Degenerate domains through whole time steps, against the oracle.

Empty systems (no Pore voxel: no pressure unknowns; no mineral: nothing to dissolve), a
domain of one phase, labels outside the reference's five (rows the reference leaves empty,
Q11), the smallest grid (2x2x2) and slabs one voxel pair thick along each axis, in the
reference model and the flow-through model, in the resident and the lean layout. The GPU
steps must succeed and match the oracle: labels exactly, the fields to the solves'
tolerance (here FP64 settings, so 1e-8 relative, or 1e-12 absolute for fields that stay
zero). The pressure is compared to 1e-5 of the system's pressure scale: these geometries
leave Pore clusters that clogging or unknown labels cut off from every fixed value, whose
pressure is free up to the weak links to fixed rows (a near-null mode), and a solve may
keep a warm start there that another drives to the exact solution (both to the FP64
residual tolerance); the fluxes, which see only its gradient, are compared tightly.
"""
import numpy as np
import pytest

from helpers import AIR, PORE, PRECIPITATE, ROCK, SULPHIDE, params, random_labels
from leachingsim_gb300._abi import BC_FLOW_I, BC_REFERENCE, MEM_LEAN, MEM_RESIDENT, PRESS_FP64
from leachingsim_gb300.runtime import Context

pytestmark = pytest.mark.gpu


def filled(shape, v, dtype=np.uint8):
    return np.full(shape, v, dtype=dtype)


def air_then(shape, v):
    lab = filled(shape, v)
    lab[:2] = AIR
    return lab


GEOMS = {
    "all_rock": lambda: filled((6, 5, 4), ROCK),
    "all_air": lambda: filled((5, 4, 6), AIR),
    "pore_no_mineral": lambda: air_then((8, 6, 5), PORE),
    "all_sulphide": lambda: filled((6, 6, 6), SULPHIDE),
    "all_precipitate": lambda: filled((4, 5, 6), PRECIPITATE),
    "unknown_labels": lambda: random_labels((7, 6, 5), 3, values=(0, 2, 4, 7, 9), dtype=np.uint16),
    "grid_2x2x2": lambda: random_labels((2, 2, 2), 5),
    "slab_i2": lambda: random_labels((2, 9, 7), 6),
    "slab_j2": lambda: random_labels((9, 2, 7), 7),
    "slab_k2": lambda: random_labels((9, 7, 2), 8),
}


def close(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(b) + 1e-12 * np.sqrt(b.size)


@pytest.mark.parametrize("mode", [MEM_RESIDENT, MEM_LEAN], ids=["resident", "lean"])
@pytest.mark.parametrize("bc", [BC_REFERENCE, BC_FLOW_I], ids=["reference", "flow"])
@pytest.mark.parametrize("name", list(GEOMS))
def test_degenerate_domain_steps(oracle_mod, name, bc, mode):
    lab = GEOMS[name]()
    lb = 2 if lab.dtype == np.uint16 else 1
    p = params(press_solver=PRESS_FP64, press_rtol=1e-12, conc_rtol=1e-13, kreac=3.0, time_scalar=50.0,
               bc_mode=bc, acid_inlet=1.0 if bc == BC_FLOW_I else 0.0, memory_mode=mode)
    o = oracle_mod.Oracle(lab.shape, label_bytes=lb, params=p, mode=oracle_mod.SOLVE_TIGHT, rtol=1e-14,
                          restart=200, max_it=50000)
    o.load_labels(lab)
    o.init_all()
    g = Context(lab.shape, label_bytes=lb, params=p)
    g.upload("label", lab)
    g.init_all()
    acid = np.random.default_rng(2).uniform(0.0, 1.0, lab.shape)
    o.set("acid", acid)
    g.upload("acid", acid)
    for n in range(3):
        ok_o, io = o.step(float(n), 1.0)
        ok_g, ig = g.step(float(n), 1.0)
        assert ok_o and ok_g, (io, ig)
        assert io["leached"] == ig["leached"]
        np.testing.assert_array_equal(g.download("label"), o.get("label"))
        assert ig["pressure"]["converged"] and ig["pressure"]["rel_residual"] <= 1e-12
        scale = max(p.p_inlet, p.p_outlet) if bc == BC_FLOW_I else p.top_pressure * min(n / 3600.0, 1.0) + 1e-6
        dp = np.abs(g.download("pressure", padded=True) - o.get("pressure", padded=True)).max()
        assert dp <= 1e-5 * scale, (n, dp, scale)
        for f in ("saturation", "conc", "acid", "precipitate", "flux_x", "flux_y", "flux_z"):
            assert close(g.download(f, padded=True), o.get(f, padded=True)), (n, f)
        np.testing.assert_allclose(g.download("frac"), o.get("frac"), rtol=1e-6, atol=1e-7)
    g.close()
    o.close()
