"""The dissolution sweep's sparse schedule against the oracle's sequential sweep.

The reference sweeps every voxel in (k, j, i) order, consuming acid in place
(src/Simulation.cpp:469-603). The GPU runs only the voxels that can change, levelled by
their dependencies, and redoes a call with the full wavefront schedule when a leach could
reach beyond them. Both must give the sequential sweep's result bit for bit.
"""
import numpy as np
import pytest

from helpers import params
from leachingsim_gb300.runtime import Context

pytestmark = pytest.mark.gpu

ROCK, SULPHIDE, PORE = 3, 4, 2


def run_both(oracle_mod, lab, frac, acid, p, dt=1.0):
    o = oracle_mod.Oracle(lab.shape, params=p, mode=oracle_mod.SOLVE_TIGHT)
    o.load_labels(lab)
    o.init_all()
    g = Context(lab.shape, params=p)
    g.upload("label", lab)
    g.init_all()
    for a in (o, g):
        (a.set if a is o else a.upload)("frac", frac)
        (a.set if a is o else a.upload)("acid", acid)
    n_o, io = o.dissolve(dt)
    n_g, ig = g.dissolve(dt)
    assert n_o == n_g
    assert io["num_steps"] == ig["num_steps"]
    np.testing.assert_array_equal(g.download("label"), o.get("label").astype(np.uint8))
    np.testing.assert_array_equal(g.download("frac"), o.get("frac"))
    for f in ("acid", "conc", "precipitate"):
        np.testing.assert_array_equal(g.download(f), o.get(f), err_msg=f)
    return g, n_g


def test_cascade_beyond_the_schedule_falls_back(oracle_mod):
    """A chain of mineral voxels along k (the sweep's outer loop, so each is swept after the
    previous): the first is at the leach threshold, the others just above it, each holding
    acid. In one sub-step each leach exposes the next voxel to the acid of the one before, so
    leaches run down the whole chain, beyond the two face steps the sparse schedule covers:
    the call must be redone with the full schedule and still match the sequential sweep."""
    shape = (6, 6, 14)
    lab = np.full(shape, ROCK, np.uint8)
    frac = np.zeros(shape, np.float32)
    acid = np.zeros(shape)
    for k in range(2, 10):
        lab[3, 3, k] = SULPHIDE
        frac[3, 3, k] = 2e-4
        acid[3, 3, k] = 1.0
    frac[3, 3, 2] = 5e-5
    g, n = run_both(oracle_mod, lab, frac, acid, params())
    assert n == 8
    assert g.dissolve_fallbacks() == 1
    g.close()


@pytest.mark.parametrize("seed", [0, 1])
def test_sparse_schedule_random(oracle_mod, seed):
    """Random mineral with acid near one face (the flow-through inlet's pattern): the sparse
    schedule runs and matches the sequential sweep, leaches included. With frac >= 0.8 and
    at most 0.1 lost per sub-step a leach needs 8 sub-steps, so with 15 sub-steps no chain of
    leaches reaches three steps and the call needs no fallback."""
    rng = np.random.default_rng(seed)
    shape = (24, 30, 28)
    lab = rng.choice(np.array([PORE, ROCK, SULPHIDE], np.uint8), size=shape, p=[0.3, 0.55, 0.15])
    frac = np.where(lab == SULPHIDE, rng.uniform(0.8, 1.0, shape), 0.0).astype(np.float32)
    acid = np.zeros(shape)
    acid[:5] = rng.uniform(0.5, 1.0, (5,) + shape[1:])
    p = params(kreac=1.0, time_scalar=1.0)
    g, n = run_both(oracle_mod, lab, frac, acid, p)
    assert n > 0
    assert g.dissolve_fallbacks() == 0
    g.close()
