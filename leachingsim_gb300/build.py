"""Build the CUDA library libleachingsim_gb300.so in-tree for sm_103a.

Each .cu under csrc/ is compiled in parallel with nvcc and linked into one shared
library exposing the C-ABI of include/leachingsim.h. The library is compiled
without FMA contraction (-fmad=false) so FP64 expressions round like the
reference's x86-64 build.

Usage: python -m leachingsim_gb300.build [--force]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libleachingsim_gb300.so")
HOST = os.path.join(HERE, "host")
CLI = os.path.join(HERE, "leachingsim")
HOST_SOURCES = ["Simulation.cpp", "vtk_writer.cpp", "main.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["ls_api.cu", "ls_pointwise.cu", "ls_pressure.cu", "ls_mg.cu", "ls_transport.cu",
           "ls_dissolve.cu", "ls_geometry.cu", "ls_learned.cu"]


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-O2", "-I" + os.path.join(ROOT, "include"), *extra]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(HOST, f) for f in os.listdir(HOST)]
    files.append(os.path.join(ROOT, "include", "leachingsim.h"))
    files.append(os.path.abspath(__file__))
    return files


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, extra=()):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc(), *_flags(extra), "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build_cli():
    """The command-line driver (host C++ over the C-ABI), linked to the library in-tree."""
    cxx = shutil.which("g++") or "g++"
    srcs = [os.path.join(HOST, s) for s in HOST_SOURCES]
    tmp = CLI + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I" + os.path.join(ROOT, "include"), "-I" + HOST,
           *srcs, "-o", tmp, "-L" + HERE, "-lleachingsim_gb300", "-Wl,-rpath,$ORIGIN", "-pthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"host build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, CLI)
    return CLI


def build(force=False, verbose=False, extra=()):
    deps = _deps()
    if not force and not _stale(LIB, deps) and not _stale(CLI, deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=(["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
    print(LIB)
