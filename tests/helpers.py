"""Shared test helpers: small seeded geometries and field fillers."""
import numpy as np

from leachingsim_gb300._abi import default_params
from leachingsim_gb300.geometry import grf_geometry, reference_case

AIR, PORE, ROCK, SULPHIDE, PRECIPITATE = 1, 2, 3, 4, 5


def random_labels(shape, seed, values=(1, 2, 3, 4, 5), weights=None, dtype=np.uint8):
    rng = np.random.default_rng(seed)
    return rng.choice(np.asarray(values), size=shape, p=weights).astype(dtype)


def small_grf(shape=(20, 18, 16), seed=3, porosity=0.35):
    lab, _ = grf_geometry(shape, porosity=porosity, corr_len=2.0, mineral_fraction=0.2,
                          seed=seed, air_inlet=True)
    return lab


def case(n=24, which=1):
    return reference_case(which, n=n)


def params(**kw):
    base = dict(c_sat=1.0)
    base.update(kw)
    return default_params(**base)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    return num / den if den > 0 else num
