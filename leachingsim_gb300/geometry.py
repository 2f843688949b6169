"""Synthetic voxel geometries (labels in the reference's (z, y, x) = (i, j, k) order).

* ``reference_case(0|1)``: the two 50^3 inputs of the reference's
  generate_input.py (case 0: pore channel with a sulphide block, Air slabs at
  both ends; case 1: sulphide vein with a pore channel, Air slabs at both
  ends), rebuilt from their description.
* ``grf_geometry``: a seeded Gaussian random field thresholded to a target
  porosity, kept only if the pore phase percolates along i (reseeding s+1
  otherwise), with a second field choosing which solid voxels are reactive
  mineral (Sulphide). With ``air_inlet`` the first two i-planes become Air,
  the reference's only pressure driver (an irrigated surface).
* ``write_raw`` / ``read_raw``: the headerless .raw format of
  src/MPIRawLoader.h:49-107 (uint8 or uint16, k fastest).
"""
import numpy as np

AIR, PORE, ROCK, SULPHIDE, PRECIPITATE = 1, 2, 3, 4, 5


def reference_case(case=1, n=50, dtype=np.uint8):
    """Inputs of generate_input.py:24-70 (shape (z, y, x) = (n, n, n), scaled from 50)."""
    def s(v):
        return int(round(v * n / 50.0))

    d = np.full((n, n, n), ROCK, dtype=dtype)
    if case == 0:
        d[:, s(20):s(30), s(20):s(30)] = PORE
        d[s(20):s(30), s(22):s(28), s(22):s(28)] = SULPHIDE
        d[0:2, :, :] = AIR
        d[n - 2:, :, :] = AIR
    elif case == 1:
        d[2:n - 2, s(22):s(28), s(22):s(28)] = SULPHIDE
        d[:, s(24):s(26), s(24):s(26)] = PORE
        d[0:2, :, :] = AIR
        d[n - 2:n, :, :] = AIR
    else:
        raise ValueError("case must be 0 or 1")
    return d


def _smooth_field(shape, sigma, rng):
    from scipy import ndimage
    noise = rng.standard_normal(shape, dtype=np.float32)
    return ndimage.gaussian_filter(noise, sigma=sigma, mode="wrap", truncate=3.0)


def _percolates(pore_mask):
    """True if one 6-connected pore cluster touches both i=0 and i=I-1."""
    from scipy import ndimage
    lab, n = ndimage.label(pore_mask)
    if n == 0:
        return False
    top = np.unique(lab[0][lab[0] > 0])
    bot = np.unique(lab[-1][lab[-1] > 0])
    return np.intersect1d(top, bot).size > 0


def grf_geometry(shape, porosity=0.30, corr_len=4.0, mineral_fraction=0.15, seed=0,
                 air_inlet=True, dtype=np.uint8, max_tries=64):
    """Seeded Gaussian-random-field geometry.

    Pore = field below its ``porosity`` quantile; the rest is solid. Of the solid,
    the ``mineral_fraction`` voxels with the lowest value of a second field of half
    the correlation length become Sulphide, the others Rock. Reseeds (seed+1, ...)
    until the pore phase percolates along i. Returns (labels, seed_used).
    """
    shape = tuple(int(v) for v in shape)
    for attempt in range(max_tries):
        s = seed + attempt
        rng = np.random.Generator(np.random.PCG64(s))
        f = _smooth_field(shape, corr_len, rng)
        thr = np.quantile(f, porosity)
        pore = f <= thr
        if not _percolates(pore):
            continue
        labels = np.full(shape, ROCK, dtype=dtype)
        labels[pore] = PORE
        if mineral_fraction > 0:
            g = _smooth_field(shape, max(corr_len / 2.0, 1.0), rng)
            solid = ~pore
            gs = g[solid]
            if gs.size:
                gthr = np.quantile(gs, mineral_fraction)
                mineral = solid & (g <= gthr)
                labels[mineral] = SULPHIDE
        if air_inlet:
            labels[0:2] = AIR
        return labels, s
    raise RuntimeError(f"no percolating geometry in {max_tries} seeds from {seed}")


def grey_levels(shape, corr_len=6.0, seed=0, n_fractures=4, aperture=(1, 3)):
    """uint16 grey-level image (0..65535) from a seeded random field with planar
    fractures of random orientation stamped in at a fixed dark level."""
    shape = tuple(int(v) for v in shape)
    rng = np.random.Generator(np.random.PCG64(seed))
    f = _smooth_field(shape, corr_len, rng)
    lo, hi = float(f.min()), float(f.max())
    grey = ((f - lo) / max(hi - lo, 1e-30) * 65535.0).astype(np.uint16)
    ii, jj, kk = np.meshgrid(*[np.arange(n, dtype=np.float32) for n in shape], indexing="ij")
    centre = np.array(shape, dtype=np.float32) / 2.0
    for _ in range(n_fractures):
        normal = rng.standard_normal(3).astype(np.float32)
        normal /= np.linalg.norm(normal)
        offset = rng.uniform(-0.3, 0.3) * min(shape)
        half = rng.integers(aperture[0], aperture[1] + 1) / 2.0
        dist = ((ii - centre[0]) * normal[0] + (jj - centre[1]) * normal[1]
                + (kk - centre[2]) * normal[2] - offset)
        grey[np.abs(dist) <= half] = 0
    return grey


def write_raw(path, labels):
    np.ascontiguousarray(labels).tofile(path)


def read_raw(path, shape, dtype=np.uint8, header=0):
    """Read a headerless-or-skipped .raw image in (z, y, x) order (MPIRawLoader semantics)."""
    I, J, K = shape
    count = I * J * K
    with open(path, "rb") as fh:
        fh.seek(header)
        data = np.fromfile(fh, dtype=dtype, count=count)
    if data.size != count:
        raise ValueError(f"{path}: expected {count} voxels, read {data.size}")
    return data.reshape(shape)
