"""Golden fixtures for the geometry pre-processing, made by running the reference's own
scripts (coarsen_grid.py, clean_micro_ct.py, micro_fracture.py) on small seeded label
images.

The scripts keep their file names and shapes as module constants and do their work in
main(); this runs each script's source with those constants replaced by a small seeded
input, in a temporary directory, and stores input and output as tests/golden/geometry.npz.
It needs the reference checkout (its path in the environment variable LEACHINGSIM_REF) and
scipy; the fixture it writes is what the tests use.

Run:  python tests/golden/make_geometry_golden.py
"""
import os
import runpy
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.environ.get("LEACHINGSIM_REF")
if not REF:
    sys.exit("set LEACHINGSIM_REF to the reference checkout (its Python scripts are run from there)")

from leachingsim_gb300.geometry import grf_geometry  # noqa: E402


def run_script(name, overrides, data, out_shape, dtype):
    with tempfile.TemporaryDirectory(dir=HERE) as tmp:
        cwd = os.getcwd()
        os.chdir(tmp)
        try:
            data.tofile(overrides["INPUT_FILE"])
            g = runpy.run_path(os.path.join(REF, name), run_name="reference_script")
            g.update(overrides)
            g["main"].__globals__.update(overrides)
            g["main"]()
            return np.fromfile(overrides["OUTPUT_FILE"], dtype=dtype).reshape(out_shape)
        finally:
            os.chdir(cwd)


def sample(shape, seed, porosity, air):
    lab, _ = grf_geometry(shape, porosity=porosity, corr_len=2.5, mineral_fraction=0.2, seed=seed,
                          air_inlet=bool(air))
    if air:  # an Air envelope on two sides, plus a detached Air pocket
        lab[:, :, -2:] = 1
        lab[shape[0] // 2, 3:5, 3:5] = 1
    return lab


def main():
    arrays = {}
    # coarsening: odd z (the script pads z by one Air plane), even y and x
    c_in = sample((23, 26, 30), 3, 0.35, 2)
    arrays["coarsen_in"] = c_in
    arrays["coarsen_out"] = run_script(
        "coarsen_grid.py", {"INPUT_FILE": "in.raw", "OUTPUT_FILE": "out.raw", "ORIGINAL_SHAPE": c_in.shape},
        c_in, ((c_in.shape[0] + 1) // 2, c_in.shape[1] // 2, c_in.shape[2] // 2), np.uint8)
    # cleaning, both modes, on two geometries (with and without an Air envelope)
    for tag, (shape, seed, por, air) in {"a": ((20, 22, 24), 5, 0.4, 2), "b": ((18, 20, 16), 6, 0.45, 0)}.items():
        lab = sample(shape, seed, por, air)
        arrays[f"clean_{tag}_in"] = lab
        for mode in ("agglomerate", "core_sample"):
            arrays[f"clean_{tag}_{mode}"] = run_script(
                "clean_micro_ct.py",
                {"INPUT_FILE": "in.raw", "OUTPUT_FILE": "out.raw", "SHAPE": lab.shape, "MODE": mode},
                lab, lab.shape, np.uint8)
    # micro-fracture drilling: low porosity and a high mineral fraction, so that many
    # Sulphide voxels are encapsulated in Rock
    for tag, (shape, seed, por, frac) in {"a": ((20, 22, 24), 5, 0.15, 0.3), "b": ((17, 13, 26), 8, 0.1, 0.4)}.items():
        lab, _ = grf_geometry(shape, porosity=por, corr_len=2.5, mineral_fraction=frac, seed=seed)
        arrays[f"fracture_{tag}_in"] = lab
        arrays[f"fracture_{tag}_out"] = run_script(
            "micro_fracture.py", {"INPUT_FILE": "in.raw", "OUTPUT_FILE": "out.raw", "SHAPE": lab.shape},
            lab, lab.shape, np.uint8)
    np.savez_compressed(os.path.join(HERE, "geometry.npz"), **arrays)
    for k, v in arrays.items():
        print(k, v.shape, np.bincount(v.ravel(), minlength=6).tolist())


if __name__ == "__main__":
    main()
