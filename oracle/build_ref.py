"""Build the parity library oracle/_ref/liblsref_u{8,16}.so from the reference's own sources.

TEST INFRASTRUCTURE ONLY. The reference's per-time-step code (src/Simulation.cpp with
src/Domain.cpp, src/MPIDomain.cpp and src/MPIDetails.cpp) is compiled unchanged, where it
lies, against this directory's single-rank stand-ins for MPI, PETSc and VTK (ref_shim/) and
the C entry points of ref_driver.cpp. The reference's own build (its Makefile, mpicxx, PETSc,
VTK, Boost) is not used; its compile flags are mirrored (-O3 -std=c++17, and -DUSE_UINT8 /
-DDATA_TYPE for the two label widths). Output goes only to oracle/_ref/ (git-ignored).

The sources are looked for in $LEACHINGSIM_REF/src, else in /root/reference/src (the
reference checkout of the build container); where neither exists, nothing is built and the
tests that need the library are skipped.

Run:  python oracle/build_ref.py [--force]
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
SOURCES = ["Simulation.cpp", "Domain.cpp", "MPIDomain.cpp", "MPIDetails.cpp"]
VARIANTS = {
    "u8": ["-DMPI_RAW_TYPE=MPI_UNSIGNED_CHAR", "-DDATA_TYPE=8", "-DUSE_UINT8"],
    "u16": ["-DMPI_RAW_TYPE=MPI_UNSIGNED_SHORT", "-DDATA_TYPE=16", "-DX_ZY=1"],
}


def ref_src():
    for base in (os.environ.get("LEACHINGSIM_REF"), "/root/reference"):
        if base and all(os.path.exists(os.path.join(base, "src", f)) for f in SOURCES):
            return os.path.join(base, "src")
    return None


def lib_path(variant):
    return os.path.join(OUT, f"liblsref_{variant}.so")


def build(force=False):
    """Compile both variants; returns the directory of the libraries, or None when the
    reference's sources are not present."""
    src = ref_src()
    if src is None:
        return None
    os.makedirs(OUT, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim")
    own = [os.path.join(shim, "ref_shim.cpp"), os.path.join(HERE, "ref_driver.cpp")]
    deps = [os.path.join(src, f) for f in SOURCES] + own + [os.path.join(shim, f) for f in os.listdir(shim)]
    deps.append(os.path.abspath(__file__))
    cxx = shutil.which("g++") or "g++"
    for name, defs in VARIANTS.items():
        target = lib_path(name)
        if not force and os.path.exists(target) and os.path.getmtime(target) >= max(os.path.getmtime(d) for d in deps):
            continue
        cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w", *defs,
               "-I" + shim, "-I" + src, "-I" + os.path.join(ROOT, "include"),
               *[os.path.join(src, f) for f in SOURCES], *own, "-Wl,-Bsymbolic", "-o", target + ".tmp"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"building {target} failed:\n{res.stdout}\n{res.stderr}")
        os.replace(target + ".tmp", target)
    return OUT


if __name__ == "__main__":
    out = build(force="--force" in sys.argv)
    print(out if out else "reference sources not found: nothing built")
