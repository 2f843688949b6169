"""CPU restatement of the reference's geometry pre-processing, for the tests (the oracle).

Test infrastructure: only tests/ import this module, as the checker of the GPU kernels in
leachingsim_gb300/csrc/ls_geometry.cu. Parity unpinned: the reference ships these steps as
stand-alone numpy/scipy scripts without tests or sample data; the restatement follows their
steps and is checked on seeded inputs.

* coarsen  - coarsen_grid.py:20-62: pad the slowest axis (z) with one Air plane when it is
  odd (the script pads unconditionally and only runs for odd z), then each 2x2x2 block takes
  the label of ranked priority voting: Sulphide if any voxel is Sulphide, else Air if any is
  Air, else Pore if any is Pore, else Rock.
* clean    - clean_micro_ct.py:33-114: morphological opening of the Pore mask with the
  6-neighbour structuring element (erosion, then dilation; voxels outside the image count
  as background), 6-connected components of the opened pores; 'agglomerate' mode keeps the
  components touching the one-voxel dilation of the largest 6-connected Air component
  (the largest by voxel count, ties to the component met first in raster order; with no Air
  at all the script's argmax falls on its background label, i.e. every non-Air voxel);
  'core_sample' mode keeps the components touching the x = 0 face. Pore voxels outside the
  kept opened components become Rock.
* fracture - micro_fracture.py:21-93: Sulphide voxels with no Pore among their six face
  neighbours are encapsulated; from each, a centre line runs to its nearest Pore voxel (the
  feature transform of scipy.ndimage.distance_transform_edt over the non-Pore mask, which
  the script calls), sampled at ceil(distance) + 1 points by numpy's linspace and rounded
  half to even; Rock voxels on the lines form the fracture mask, which is dilated with the
  full 3x3x3 element, and the Rock voxels inside the dilation become Pore. With no Pore
  voxel at all the script's transform has no feature to point at; the restatement refuses
  that input.
* classify - threshold classification of a grey-level image: label = labels[i] with i the
  number of thresholds <= the grey value.
"""
import numpy as np

AIR, PORE, ROCK, SULPHIDE = 1, 2, 3, 4


def _shift_or(m):
    """m OR its six face neighbours (outside the image: False)."""
    out = m.copy()
    out[1:] |= m[:-1]
    out[:-1] |= m[1:]
    out[:, 1:] |= m[:, :-1]
    out[:, :-1] |= m[:, 1:]
    out[:, :, 1:] |= m[:, :, :-1]
    out[:, :, :-1] |= m[:, :, 1:]
    return out


def _erode6(m):
    """m AND its six face neighbours (outside the image: False)."""
    out = m.copy()
    out[0] = False
    out[-1] = False
    out[:, 0] = False
    out[:, -1] = False
    out[:, :, 0] = False
    out[:, :, -1] = False
    out[1:] &= m[:-1]
    out[:-1] &= m[1:]
    out[:, 1:] &= m[:, :-1]
    out[:, :-1] &= m[:, 1:]
    out[:, :, 1:] &= m[:, :, :-1]
    out[:, :, :-1] &= m[:, :, 1:]
    return out


def _components6(mask):
    """6-connected component label per voxel: 0 background, else the raster index + 1 of
    the component's first voxel (so ordering by label is raster order of first voxels)."""
    from scipy import ndimage
    lab, n = ndimage.label(mask, structure=ndimage.generate_binary_structure(3, 1))
    if n == 0:
        return lab.astype(np.int64)
    flat = lab.ravel()
    first = np.full(n + 1, -1, dtype=np.int64)
    idx = np.nonzero(flat)[0]
    # first occurrence of each label in raster order
    order = np.unique(flat[idx], return_index=True)
    first[order[0]] = idx[order[1]]
    out = np.where(flat > 0, first[flat] + 1, 0)
    return out.reshape(mask.shape)


def coarsen(labels):
    labels = np.asarray(labels)
    Z, Y, X = labels.shape
    if Y % 2 or X % 2:
        raise ValueError("coarsening needs even y and x extents")
    if Z % 2:
        pad = np.full((1, Y, X), AIR, dtype=labels.dtype)
        labels = np.concatenate([labels, pad], axis=0)
        Z += 1
    b = labels.reshape(Z // 2, 2, Y // 2, 2, X // 2, 2)
    has = lambda v: (b == v).any(axis=(1, 3, 5))
    out = np.full((Z // 2, Y // 2, X // 2), ROCK, dtype=labels.dtype)
    out[has(PORE)] = PORE
    out[has(AIR)] = AIR
    out[has(SULPHIDE)] = SULPHIDE
    return out


def clean(labels, mode="agglomerate"):
    labels = np.asarray(labels)
    pore = labels == PORE
    opened = _shift_or(_erode6(pore))
    comp = _components6(opened)
    if mode == "agglomerate":
        air = _components6(labels == AIR)
        ids, counts = np.unique(air[air > 0], return_counts=True)
        if ids.size:
            amb = air == ids[np.lexsort((ids, -counts))[0]]
        else:
            amb = labels != AIR
        env = _shift_or(amb)
        valid = np.unique(comp[env & opened])
    elif mode == "core_sample":
        valid = np.unique(comp[:, :, 0])
    else:
        raise ValueError(mode)
    valid = valid[valid > 0]
    keep = np.isin(comp, valid) & (comp > 0)
    out = labels.copy()
    change = pore & ~keep
    out[change] = ROCK
    return out, int(change.sum())


def classify(grey, thresholds, labels):
    grey = np.asarray(grey)
    t = np.asarray(thresholds)
    idx = np.searchsorted(t, grey, side="right")
    return np.asarray(labels)[idx]


def fracture(labels):
    """Returns (labels after drilling, number of Rock voxels turned to Pore, number of
    encapsulated Sulphide voxels)."""
    from scipy import ndimage
    data = np.array(labels, copy=True)
    pore = data == PORE
    if not pore.any():
        raise ValueError("no Pore voxel: the distance transform has no feature")
    sul = data == SULPHIDE
    encaps = sul & ~_shift_or(pore)
    n_enc = int(encaps.sum())
    if n_enc == 0:
        return data, 0, 0
    dist, ind = ndimage.distance_transform_edt(~pore, return_indices=True)
    frac = np.zeros(data.shape, dtype=bool)
    for s in np.argwhere(encaps):
        p = ind[:, s[0], s[1], s[2]]
        num = int(np.ceil(dist[tuple(s)])) + 1
        if num > 1:
            pts = [np.round(np.linspace(s[a], p[a], num)).astype(int) for a in range(3)]
            on = data[pts[0], pts[1], pts[2]] == ROCK
            frac[pts[0][on], pts[1][on], pts[2][on]] = True
    wide = ndimage.binary_dilation(frac, structure=ndimage.generate_binary_structure(3, 3))
    new = wide & (data == ROCK)
    data[new] = PORE
    return data, int(new.sum()), n_enc


def feature_transform(sites):
    """Nearest site (True voxel) of every voxel, as an index array of shape (3,) + shape, by
    the separable algorithm of Maurer, Qi and Raghavan (IEEE PAMI 25(2), 2003) in the pass
    order and tie rule of the GPU kernel (slowest axis first; a position keeps the earlier
    site unless a later one is strictly closer). Pure Python, for small images: the tests
    check it against scipy.ndimage.distance_transform_edt(~sites, return_indices=True), the
    call micro_fracture.py makes."""
    sites = np.asarray(sites, dtype=bool)
    shape = sites.shape
    feat = np.full(shape + (3,), -1, dtype=np.int64)
    feat[sites] = np.argwhere(sites)
    for ax in range(3):
        moved = np.moveaxis(feat, ax, 0)  # view: lines along axis 0 of `moved`
        n = shape[ax]
        for idx in np.ndindex(*moved.shape[1:-1]):
            line = moved[(slice(None),) + idx]
            fixed = list(idx)
            stack = []  # (site, position, squared distance off the line)
            for q in range(n):
                f = line[q]
                if f[0] < 0:
                    continue
                perp = sum(int(f[a] - fixed[b]) ** 2 for b, a in enumerate(x for x in range(3) if x != ax)
                           if a < ax)
                while len(stack) >= 2:
                    (_, pu, du), (_, pv, dv) = stack[-2], stack[-1]
                    a, b = pv - pu, q - pv
                    c = a + b
                    if c * dv - b * du - a * perp - a * b * c > 0:
                        stack.pop()
                    else:
                        break
                stack.append((f.copy(), q, perp))
            if not stack:
                continue
            l = 0
            for q in range(n):
                while l + 1 < len(stack):
                    d0 = stack[l][2] + (stack[l][1] - q) ** 2
                    d1 = stack[l + 1][2] + (stack[l + 1][1] - q) ** 2
                    if d0 > d1:
                        l += 1
                    else:
                        break
                line[q] = stack[l][0]
    return np.moveaxis(feat, -1, 0)
