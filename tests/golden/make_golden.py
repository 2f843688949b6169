"""Generate the golden fixtures of tests/golden/.

Oracle cases (the CPU oracle, tight solves): the reference's two generate_input.py recipes
scaled to 20^3 (Air slabs at both ends) and a small seeded Gaussian-random-field geometry,
each run from a fresh start for 4 steps of dt = 1 (csat = 1, like the reference's job
scripts), plus one restart-style case with acid present so the dissolution sweep is
exercised.

Reference cases (source "reference"): produced by the reference's own code, the parity
library oracle/_ref (src/Simulation.cpp compiled unchanged against single-rank MPI / PETSc /
VTK stand-ins, tight GMRES solves), stepped in the order of src/main.cpp:303-432. The
reference throws on non-solid voxels of a low face and on a domain without mineral, so these
geometries have a Rock shell on the planes i, j, k = 0 and Air inlet planes i = 1, 2; one is
uint8, one uint16 with acid present. They need the reference's sources (oracle/build_ref.py)
and are skipped by this script where those are absent.

Saved per case: the inputs, the parameters, the per-step summaries and the final fields
(padded (I+1)*J*K arrays, the reference's np=1 layout).

Run:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from leachingsim_gb300._abi import default_params  # noqa: E402
from leachingsim_gb300.geometry import grf_geometry, reference_case  # noqa: E402
from oracle import oracle as om  # noqa: E402

FIELDS = ["label", "frac", "pressure", "conc", "acid", "flux_x", "flux_y", "flux_z", "saturation",
          "cap_pressure", "rel_perm", "permeability", "precipitate"]


def cases():
    yield "case0_20", reference_case(0, n=20), dict(c_sat=1.0), None
    yield "case1_20", reference_case(1, n=20), dict(c_sat=1.0), None
    lab, _ = grf_geometry((18, 16, 14), porosity=0.32, corr_len=2.0, mineral_fraction=0.2, seed=7)
    yield "grf_18x16x14", lab, dict(c_sat=1.0), None
    acid = np.random.default_rng(11).uniform(0.0, 1.0, lab.shape)
    yield "grf_acid_18x16x14", lab, dict(c_sat=1.0, kreac=5.0, time_scalar=100.0), acid


def shelled(shape, seed, dtype):
    """GRF geometry with Air inlet planes i = 1, 2 and Rock on the planes i, j, k = 0."""
    lab, _ = grf_geometry(shape, porosity=0.35, corr_len=2.0, mineral_fraction=0.2, seed=seed, air_inlet=False,
                          dtype=dtype)
    lab[1:3] = 1
    lab[0] = 3
    lab[:, 0] = 3
    lab[:, :, 0] = 3
    return lab


def reference_cases():
    yield "ref_u8_16x14x12", shelled((16, 14, 12), 21, np.uint8), dict(c_sat=1.0), None
    lab = shelled((14, 15, 12), 22, np.uint16)
    acid = np.random.default_rng(23).uniform(0.0, 1.0, lab.shape)
    yield "ref_u16_acid_14x15x12", lab, dict(c_sat=1.0, kreac=5.0, time_scalar=100.0), acid


def run_reference(lab, pover, acid, steps=4):
    from oracle import refsim
    lb = 2 if lab.dtype == np.uint16 else 1
    p = default_params(press_rtol=1e-13, conc_rtol=1e-13, **pover)
    r = refsim.RefSim(lab.shape, label_bytes=lb, params=p, rtol=1e-14, restart=200, max_it=200000)
    r.load_labels(lab)
    r.init_all()
    if acid is not None:
        r.set("acid", acid)
    infos = []
    for n in range(steps):
        ok, leached = r.step(float(n), 1.0)
        assert ok
        infos.append({"leached": int(leached)})
    out = {f: r.get(f, padded=True) for f in FIELDS}
    r.close()
    return p, infos, out


def run_case(lab, pover, acid, steps=4):
    p = default_params(press_rtol=1e-13, conc_rtol=1e-13, **pover)
    o = om.Oracle(lab.shape, params=p, mode=om.SOLVE_TIGHT, rtol=1e-14, restart=200, max_it=200000)
    o.load_labels(lab)
    o.init_all()
    if acid is not None:
        o.set("acid", acid)
    infos = []
    for n in range(steps):
        ok, info = o.step(float(n), 1.0)
        assert ok, info
        infos.append({"leached": info["leached"], "sat_steps": info["saturation"]["num_steps"],
                      "sat_max_rate": info["saturation"]["max_rate"],
                      "leach_steps": info["leaching"]["num_steps"],
                      "leach_max_rate": info["leaching"]["max_rate"]})
    out = {f: o.get(f, padded=True) for f in FIELDS}
    return p, infos, out


def save(manifest, name, lab, acid, p, infos, out, source):
    arrays = {"in_label": lab}
    if acid is not None:
        arrays["in_acid"] = acid
    for f, v in out.items():
        arrays[f] = v
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
    manifest[name] = {"shape": list(lab.shape), "params": {k: v for k, v in p.as_dict().items()},
                      "steps": len(infos), "infos": infos, "source": source,
                      "label_bytes": 2 if lab.dtype == np.uint16 else 1}
    print(name, source, lab.shape, [i["leached"] for i in infos])


def main():
    manifest = {}
    old = os.path.join(HERE, "manifest.json")
    if os.path.exists(old):
        manifest = json.load(open(old))
    for name, lab, pover, acid in cases():
        p, infos, out = run_case(lab, pover, acid)
        save(manifest, name, lab, acid, p, infos, out, "oracle")
    from oracle import refsim
    if refsim.available():
        for name, lab, pover, acid in reference_cases():
            p, infos, out = run_reference(lab, pover, acid)
            save(manifest, name, lab, acid, p, infos, out, "reference")
    else:
        print("the reference's sources are not present: reference cases kept as they are")
    with open(os.path.join(HERE, "manifest.json"), "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
