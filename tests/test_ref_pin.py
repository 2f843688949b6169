"""The oracle (oracle/ls_oracle.c) pinned to the reference's own code.

oracle/_ref holds the reference's src/Simulation.cpp (with Domain.cpp, MPIDomain.cpp and
MPIDetails.cpp) compiled unchanged against single-rank stand-ins for MPI, PETSc and VTK
(oracle/build_ref.py, oracle/ref_shim/); its PETSc stand-in solves with restarted GMRES and
Jacobi preconditioning. Each function of the time step gets the same inputs in both and
must give the same outputs: bit for bit where no linear solve is involved (both run the
same FP64 expressions and libm on this host), to the solve tolerance where one is. The
reference's bounds-checked indexing throws for any non-solid voxel on a low face
(setupConcentrationEqns reads flux_x[Index(i-1,j,k)] before checking the index,
src/Simulation.cpp:1227-1231), and setupReactionRates (src/Simulation.cpp:109-125) for a
domain without Sulphide, so the geometries here have a Rock shell on the planes i, j, k = 0
and hold mineral. The library is built only where the reference's sources are present;
elsewhere these tests are skipped.
"""
import numpy as np
import pytest

from helpers import params, rel_l2
from leachingsim_gb300.geometry import grf_geometry

refsim = pytest.importorskip("oracle.refsim")
if not refsim.available():
    pytest.skip("the reference's sources are not present", allow_module_level=True)

AIR, PORE, ROCK, SULPHIDE, PRECIPITATE = 1, 2, 3, 4, 5


def shelled(shape, seed, air=True, dtype=np.uint8, porosity=0.35, corr=2.0):
    """GRF geometry (Air inlet planes i = 1, 2 when `air`), Rock on the planes i, j, k = 0."""
    lab, _ = grf_geometry(shape, porosity=porosity, corr_len=corr, mineral_fraction=0.2, seed=seed,
                          air_inlet=False, dtype=dtype)
    if air:
        lab[1:3] = AIR
    lab[0] = ROCK
    lab[:, 0] = ROCK
    lab[:, :, 0] = ROCK
    return lab


def pair(oracle_mod, lab, p, lb=1, seed=0, randomize=True):
    o = oracle_mod.Oracle(lab.shape, label_bytes=lb, params=p, mode=oracle_mod.SOLVE_TIGHT, rtol=1e-13,
                          restart=200, max_it=200000)
    r = refsim.RefSim(lab.shape, label_bytes=lb, params=p, rtol=1e-13, restart=200, max_it=200000)
    for a in (o, r):
        a.load_labels(lab)
        a.init_all()
    if randomize:
        rng = np.random.default_rng(seed)
        shp = lab.shape
        fields = {"saturation": rng.uniform(0.0, 1.0, shp), "precipitate": rng.uniform(-0.2, 1.2, shp),
                  "frac": rng.uniform(0.0, 1.0, shp).astype(np.float32)}
        for name, arr in fields.items():
            for a in (o, r):
                a.set(name, arr)
    return o, r


def same(a, b, name):
    np.testing.assert_array_equal(np.asarray(a), np.asarray(b), err_msg=name)


GEOMS = [("u8", np.uint8, 1, (14, 12, 11), 3), ("u16", np.uint16, 2, (12, 13, 10), 4)]


@pytest.mark.parametrize("name,dtype,lb,shape,seed", GEOMS)
def test_props_flux_saturation_surface_precip_exact(oracle_mod, name, dtype, lb, shape, seed):
    lab = shelled(shape, seed, dtype=dtype)
    p = params(evaporative_flux=2e-3)
    o, r = pair(oracle_mod, lab, p, lb, seed=seed)
    # updateRelativePermeability + updateCapillaryPressure + initProperties
    o.props()
    r.props()
    for f in ("rel_perm", "cap_pressure", "permeability", "viscosity"):
        same(o.get(f, padded=True), r.get(f, padded=True), f)
    # calculateFlux on a random pressure
    P = np.random.default_rng(seed + 1).normal(0, 100.0, (shape[0] + 1,) + shape[1:])
    for a in (o, r):
        a.set("pressure", P, padded=True)
    o.flux()
    r.call("calculateFlux")
    for f in ("flux_x", "flux_y", "flux_z"):
        same(o.get(f, padded=True), r.get(f, padded=True), f)
    # updateSaturation (explicit sub-steps) on scaled fluxes
    for f in ("flux_x", "flux_y", "flux_z"):
        v = o.get(f, padded=True) * 1e9
        o.set(f, v, padded=True)
        r.set(f, v, padded=True)
    o.saturation(2.0)
    r.call("updateSaturation", 2.0)
    same(o.get("saturation", padded=True), r.get("saturation", padded=True), "saturation")
    # handleSurfaceEffects
    o.surface()
    r.call("handleSurfaceEffects")
    same(o.get("label"), r.get("label"), "label")
    same(o.get("conc", padded=True), r.get("conc", padded=True), "conc")
    # handlePrecipitation, both modes
    c = np.random.default_rng(seed + 2).uniform(0.0, 1.5, shape)
    for instant in (0, 1):
        p2 = params(c_sat=0.6, solid_density=0.3, use_instant_precipitation=instant)
        o2, r2 = pair(oracle_mod, lab, p2, lb, seed=seed + 3)
        for a in (o2, r2):
            a.set("conc", c)
        o2.precip()
        r2.call("handlePrecipitation")
        for f in ("label", "conc", "precipitate"):
            same(o2.get(f, padded=f != "label"), r2.get(f, padded=f != "label"), f"{f} instant={instant}")
        o2.close()
        r2.close()
    o.close()
    r.close()


@pytest.mark.parametrize("name,dtype,lb,shape,seed", GEOMS)
def test_dissolution_exact(oracle_mod, name, dtype, lb, shape, seed):
    """updateFrac: the sequential in-place sweep with its sub-steps, leaches included."""
    lab = shelled(shape, seed, dtype=dtype)
    p = params(kreac=5.0, time_scalar=50.0)
    o, r = pair(oracle_mod, lab, p, lb, seed=seed)
    acid = np.random.default_rng(seed + 5).uniform(0.0, 1.0, (shape[0] + 1,) + shape[1:])
    for a in (o, r):
        a.set("acid", acid, padded=True)
    n_o, _ = o.dissolve(1.0)
    n_r = r.call("updateFrac", 1.0)
    assert n_o == n_r and n_o > 0
    for f in ("label", "frac", "acid", "conc", "precipitate"):
        same(o.get(f, padded=True), r.get(f, padded=True), f)
    o.close()
    r.close()


@pytest.mark.parametrize("name,dtype,lb,shape,seed", GEOMS)
def test_solves_and_the_write_back_offset(oracle_mod, name, dtype, lb, shape, seed):
    """setupPressureEqns + solvePressure, and the two transport solves: the solutions to the
    tolerance of two tight GMRES solves of the same system, written one i-plane up (the
    solution vector placed at data + pad_size, src/Simulation.cpp:808,1247,2173) with plane
    0 keeping what it held."""
    lab = shelled(shape, seed, dtype=dtype)
    p = params(evaporative_flux=1e-7, alpha_transfer=0.3, Dpore_fac=2.0)
    o, r = pair(oracle_mod, lab, p, lb, seed=seed)
    rng = np.random.default_rng(seed + 7)
    P0 = rng.normal(0, 1.0, (shape[0] + 1,) + shape[1:])
    for a in (o, r):
        a.props()
        a.set("pressure", P0, padded=True)
    o.pressure(1800.0)
    r.call("setupPressureEqns", 1800.0)
    assert r.call("solvePressure") == 1
    Po, Pr = o.get("pressure", padded=True), r.get("pressure", padded=True)
    same(Po[0], P0[0], "pressure plane 0 (oracle)")
    same(Pr[0], P0[0], "pressure plane 0 (reference)")
    # near-null modes of the floored Pore clusters: two solves to rtol 1e-13 differ there by up
    # to ~1.3e-7 (the oracle's OpenMP reductions make its own runs differ by as much)
    assert rel_l2(Po, Pr) < 1e-6
    for f in ("flux_x", "flux_y", "flux_z", "conc", "acid"):
        v = rng.normal(0, 1.0, (shape[0] + 1,) + shape[1:])
        for a in (o, r):
            a.set(f, v, padded=True)
    conc0, acid0 = o.get("conc", padded=True), o.get("acid", padded=True)
    o.transport(0.7, 0)
    r.call("setupConcentrationEqns_conc", 0.7)
    assert r.call("solveConc") == 1
    o.transport(0.7, 1)
    r.call("setupConcentrationEqns_acid", 0.7)
    assert r.call("solveAcid") == 1
    for f, f0 in (("conc", conc0), ("acid", acid0)):
        a, b = o.get(f, padded=True), r.get(f, padded=True)
        same(a[0], f0[0], f"{f} plane 0")
        same(b[0], f0[0], f"{f} plane 0 (reference)")
        assert rel_l2(a, b) < 1e-11, f
    # the fluxes the transport setup zeroes on Rock and Precipitate
    for f in ("flux_x", "flux_y", "flux_z"):
        same(o.get(f, padded=True), r.get(f, padded=True), f)
    o.close()
    r.close()


@pytest.mark.parametrize("name,dtype,lb,shape,seed", GEOMS)
def test_whole_steps(oracle_mod, name, dtype, lb, shape, seed):
    """Four whole steps of src/main.cpp:303-432 from a fresh start with acid present (the
    reference has no acid source, so it is put in as a restart state would): labels, leach
    counts and mineral fractions exact, fields to the solve tolerance."""
    lab = shelled(shape, seed, dtype=dtype)
    p = params(kreac=5.0, time_scalar=100.0)
    o, r = pair(oracle_mod, lab, p, lb, randomize=False)
    acid = np.random.default_rng(seed + 11).uniform(0.0, 1.0, shape)
    for a in (o, r):
        a.set("acid", acid)
    for n in range(4):
        ok_o, info = o.step(float(n), 1.0)
        ok_r, n_r = r.step(float(n), 1.0)
        assert ok_o and ok_r
        assert info["leached"] == n_r
    same(o.get("label"), r.get("label"), "label")
    same(o.get("frac"), r.get("frac"), "frac")
    for f, tol in (("pressure", 1e-8), ("saturation", 1e-10), ("conc", 1e-10), ("acid", 1e-10),
                   ("flux_x", 1e-8)):
        assert rel_l2(o.get(f, padded=True), r.get(f, padded=True)) < tol, f
    # where conc sits at c_sat = 1 to within the solves' rounding, one side may precipitate
    # ~1e-17 that the other does not: compared by the largest absolute difference
    assert np.abs(o.get("precipitate", padded=True) - r.get("precipitate", padded=True)).max() < 1e-12
    o.close()
    r.close()


def test_implicit_saturation(oracle_mod):
    """setupSaturationEqns + solveSaturation (src/Simulation.cpp:1858-2053), with its physics
    check and clamp."""
    lab = shelled((12, 11, 10), 6)
    p = params()
    o, r = pair(oracle_mod, lab, p, 1, seed=6)
    rng = np.random.default_rng(8)
    for f in ("flux_x", "flux_y", "flux_z"):
        v = rng.normal(0, 1e-3, (13, 11, 10))
        for a in (o, r):
            a.set(f, v, padded=True)
    ok_o, valid_o, _ = o.saturation_implicit(1.0)
    r.call("setupSaturationEqns", 1.0)
    ok_r = r.call("solveSaturation")
    assert bool(ok_o) == bool(ok_r)
    assert valid_o == bool(r.call("physics_valid"))
    assert rel_l2(o.get("saturation", padded=True), r.get("saturation", padded=True)) < 1e-10
    o.close()
    r.close()
