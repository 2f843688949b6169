"""Geometry pre-processing: coarsening (coarsen_grid.py), cleaning (clean_micro_ct.py),
micro-fracture drilling (micro_fracture.py) and grey-level classification.

CPU: the oracle (oracle/geometry_oracle.py) reproduces the fixtures made by running the
reference's own scripts (tests/golden/make_geometry_golden.py). GPU: the kernels behind the
C-ABI (ls_geom_*) reproduce the fixtures and the oracle exactly (integer label work).
"""
import os

import numpy as np
import pytest

from oracle import geometry_oracle as go

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "geometry.npz"))
CLEAN_CASES = [(t, m) for t in ("a", "b") for m in ("agglomerate", "core_sample")]


def test_oracle_coarsen_matches_reference_script():
    np.testing.assert_array_equal(go.coarsen(GOLD["coarsen_in"]), GOLD["coarsen_out"])


@pytest.mark.parametrize("tag,mode", CLEAN_CASES)
def test_oracle_clean_matches_reference_script(tag, mode):
    out, _ = go.clean(GOLD[f"clean_{tag}_in"], mode)
    np.testing.assert_array_equal(out, GOLD[f"clean_{tag}_{mode}"])


def test_oracle_classify():
    g = np.array([0, 99, 100, 101, 5000, 65535], dtype=np.uint16).reshape(1, 1, 6)
    out = go.classify(g, [100, 5000], [2, 3, 4])
    assert out.ravel().tolist() == [2, 2, 3, 3, 4, 4]


@pytest.mark.parametrize("tag", ["a", "b"])
def test_oracle_fracture_matches_reference_script(tag):
    out, n, n_enc = go.fracture(GOLD[f"fracture_{tag}_in"])
    np.testing.assert_array_equal(out, GOLD[f"fracture_{tag}_out"])
    assert n == int(((GOLD[f"fracture_{tag}_in"] == 3) & (out == 2)).sum()) and n_enc > 0


@pytest.mark.parametrize("seed", range(6))
def test_feature_transform_restatement_matches_scipy(seed):
    """The pass order and tie rule of the GPU feature transform give scipy's nearest sites."""
    from scipy import ndimage
    rng = np.random.default_rng(seed)
    for _ in range(5):
        shape = tuple(int(v) for v in rng.integers(1, 9, size=3))
        m = rng.random(shape) < rng.uniform(0.03, 0.3)
        m.flat[int(rng.integers(m.size))] = True
        _, ind = ndimage.distance_transform_edt(~m, return_indices=True)
        np.testing.assert_array_equal(go.feature_transform(m), ind)


def _random_labels(shape, seed, p=(0.1, 0.45, 0.3, 0.15)):
    rng = np.random.default_rng(seed)
    return rng.choice([1, 2, 3, 4], size=shape, p=list(p)).astype(np.uint8)


@pytest.mark.gpu
def test_gpu_coarsen_matches_reference_script():
    from leachingsim_gb300.runtime import geom_coarsen
    np.testing.assert_array_equal(geom_coarsen(GOLD["coarsen_in"]), GOLD["coarsen_out"])


@pytest.mark.gpu
@pytest.mark.parametrize("tag,mode", CLEAN_CASES)
def test_gpu_clean_matches_reference_script(tag, mode):
    from leachingsim_gb300.runtime import geom_clean
    lab = GOLD[f"clean_{tag}_in"]
    out, n = geom_clean(lab, mode)
    np.testing.assert_array_equal(out, GOLD[f"clean_{tag}_{mode}"])
    assert n == int(((lab == 2) & (out == 3)).sum())


@pytest.mark.gpu
@pytest.mark.parametrize("shape,seed", [((33, 40, 46), 1), ((16, 18, 20), 2), ((1, 8, 6), 3)])
def test_gpu_geometry_against_oracle(shape, seed):
    from leachingsim_gb300.runtime import geom_clean, geom_coarsen
    from leachingsim_gb300.geometry import grf_geometry
    lab = _random_labels(shape, seed) if min(shape) < 4 else grf_geometry(
        shape, porosity=0.4, corr_len=2.0, mineral_fraction=0.2, seed=seed)[0]
    for mode in ("agglomerate", "core_sample"):
        ref, nref = go.clean(lab, mode)
        out, n = geom_clean(lab, mode)
        np.testing.assert_array_equal(out, ref)
        assert n == nref
        ref16, _ = go.clean(lab.astype(np.uint16), mode)
        out16, _ = geom_clean(lab.astype(np.uint16), mode)
        np.testing.assert_array_equal(out16, ref16)
    if shape[1] % 2 == 0 and shape[2] % 2 == 0:
        np.testing.assert_array_equal(geom_coarsen(lab), go.coarsen(lab))


@pytest.mark.gpu
def test_gpu_classify_against_oracle():
    from leachingsim_gb300.runtime import geom_classify
    from leachingsim_gb300.geometry import grey_levels
    g = grey_levels((24, 30, 28), corr_len=3.0, seed=4)
    thr, labs = [21000, 47000], [2, 3, 4]
    for lb in (1, 2):
        np.testing.assert_array_equal(geom_classify(g, thr, labs, lb), go.classify(g, thr, labs))
    np.testing.assert_array_equal(geom_classify(g, [], [3], 1), np.full(g.shape, 3, np.uint8))


@pytest.mark.gpu
def test_gpu_geometry_bad_arguments():
    from leachingsim_gb300.runtime import geom_classify, geom_coarsen
    with pytest.raises(ValueError):
        geom_coarsen(np.zeros((4, 5, 6), np.uint8))  # odd y
    with pytest.raises(RuntimeError):
        geom_classify(np.zeros((2, 2, 2), np.uint16), [5, 3], [1, 2, 3])  # thresholds not ascending


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["a", "b"])
def test_gpu_fracture_matches_reference_script(tag):
    from leachingsim_gb300.runtime import geom_fracture
    lab = GOLD[f"fracture_{tag}_in"]
    out, n, n_enc = geom_fracture(lab)
    np.testing.assert_array_equal(out, GOLD[f"fracture_{tag}_out"])
    _, nref, eref = go.fracture(lab)
    assert (n, n_enc) == (nref, eref)
    out16, _, _ = geom_fracture(lab.astype(np.uint16))
    np.testing.assert_array_equal(out16, GOLD[f"fracture_{tag}_out"])


@pytest.mark.gpu
@pytest.mark.parametrize("shape,seed,por", [((40, 36, 50), 1, 0.12), ((1, 30, 28), 2, 0.2), ((25, 1, 33), 3, 0.2),
                                            ((31, 29, 1), 4, 0.2), ((64, 48, 72), 5, 0.12)])
def test_gpu_fracture_against_oracle(shape, seed, por):
    from leachingsim_gb300.geometry import grf_geometry
    from leachingsim_gb300.runtime import geom_fracture
    if min(shape) == 1:
        lab = _random_labels(shape, seed, p=(0.05, por, 0.55, 0.4 - por))
    else:
        lab = grf_geometry(shape, porosity=por, corr_len=2.0, mineral_fraction=0.3, seed=seed)[0]
    ref, nref, eref = go.fracture(lab)
    out, n, n_enc = geom_fracture(lab)
    np.testing.assert_array_equal(out, ref)
    assert (n, n_enc) == (nref, eref)


@pytest.mark.gpu
def test_gpu_fracture_edge_cases():
    from leachingsim_gb300.runtime import geom_fracture
    # every Sulphide voxel touches Pore: nothing changes
    lab = np.full((4, 5, 6), 3, np.uint8)
    lab[:, :, ::2] = 2
    lab[:, :, 1] = 4
    out, n, n_enc = geom_fracture(lab)
    assert (n, n_enc) == (0, 0)
    np.testing.assert_array_equal(out, lab)
    # a single Pore voxel far from a single Sulphide voxel: one straight drilled line
    lab = np.full((3, 3, 20), 3, np.uint8)
    lab[1, 1, 0] = 2
    lab[1, 1, 19] = 4
    ref, nref, _ = go.fracture(lab)
    out, n, n_enc = geom_fracture(lab)
    np.testing.assert_array_equal(out, ref)
    assert n == nref and n_enc == 1
    # no Pore voxel at all: refused
    with pytest.raises(RuntimeError):
        geom_fracture(np.full((3, 4, 5), 4, np.uint8))


@pytest.mark.gpu
@pytest.mark.parametrize("shape,seed", [((20, 17, 33), 1), ((1, 40, 9), 2), ((12, 12, 12), 3)])
def test_gpu_distance_matches_scipy(shape, seed):
    import torch
    from scipy import ndimage
    from leachingsim_gb300.runtime import geom_distance
    rng = np.random.default_rng(seed)
    sites = (rng.random(shape) < 0.05).astype(np.float32)
    sites.flat[0] = 1.0
    d = geom_distance(torch.from_numpy(sites).cuda()).cpu().numpy()
    ref = ndimage.distance_transform_edt(sites < 0.5)
    np.testing.assert_allclose(d, ref, rtol=1e-6, atol=1e-6)
    assert np.all(geom_distance(torch.zeros(shape).cuda()).cpu().numpy() == -1.0)
