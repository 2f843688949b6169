"""ctypes front end of the parity library oracle/_ref/liblsref_u{8,16}.so: the reference's own
Simulation (src/Simulation.cpp, compiled unchanged against single-rank MPI / PETSc / VTK
stand-ins by oracle/build_ref.py).

TEST INFRASTRUCTURE ONLY: imported by tests/ to pin oracle/ls_oracle.c to the reference's
code. The library exists only where the reference's sources were present at build time;
`available()` says whether it is here.
"""
import ctypes as C
import os

import numpy as np

from leachingsim_gb300._abi import FIELDS, LsParams

from . import build_ref

_libs = {}


def available():
    try:
        return build_ref.build() is not None
    except RuntimeError:
        return False


def lib(label_bytes):
    name = "u8" if label_bytes == 1 else "u16"
    if name not in _libs:
        if build_ref.build() is None:
            raise RuntimeError("the reference's sources are not present: no parity library")
        L = C.CDLL(build_ref.lib_path(name))
        vp, d, i = C.c_void_p, C.c_double, C.c_int
        for fn, res, args in (("lsref_last_error", C.c_char_p, []), ("lsref_label_bytes", i, []),
                              ("lsref_create", vp, [i, i, i, C.POINTER(LsParams)]), ("lsref_destroy", None, [vp]),
                              ("lsref_option", None, [C.c_char_p, C.c_char_p]),
                              ("lsref_field", vp, [vp, i, C.POINTER(C.c_int)]), ("lsref_init", i, [vp]),
                              ("lsref_initial_sulphide_count", C.c_ulonglong, [vp]),
                              ("lsref_call", i, [vp, C.c_char_p, d, C.POINTER(C.c_int)]),
                              ("lsref_checkpoint", i, [vp, C.c_char_p, i, i])):
            f = getattr(L, fn)
            f.restype = res
            f.argtypes = args
        _libs[name] = L
    return _libs[name]


class RefSim:
    """The reference's Simulation on one rank, with the oracle's field and method names."""

    def __init__(self, shape, label_bytes=1, params=None, rtol=1e-13, restart=200, max_it=200000):
        self.shape = tuple(int(v) for v in shape)
        self.I, self.J, self.K = self.shape
        self.N = self.I * self.J * self.K
        self.NP = (self.I + 1) * self.J * self.K
        self.label_bytes = label_bytes
        self.L = lib(label_bytes)
        # the reference's PETSc command-line options for all four solvers (src/Simulation.cpp
        # :814, 1253, 1982, 2179 set the prefixes)
        for pre in ("press_", "conc_", "acid_", "sat_"):
            self.L.lsref_option(f"{pre}ksp_rtol".encode(), repr(float(rtol)).encode())
            self.L.lsref_option(f"{pre}ksp_max_it".encode(), str(int(max_it)).encode())
            self.L.lsref_option(f"{pre}ksp_gmres_restart".encode(), str(int(restart)).encode())
        self.params = params if params is not None else LsParams()
        self.h = self.L.lsref_create(self.I, self.J, self.K, C.byref(self.params))
        if not self.h:
            raise RuntimeError(self.L.lsref_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.lsref_destroy(self.h)
            self.h = None

    __del__ = close

    def _array(self, name):
        eb = C.c_int(0)
        ptr = self.L.lsref_field(self.h, FIELDS[name], C.byref(eb))
        if not ptr:
            raise ValueError(name)
        dt = {1: np.uint8, 2: np.uint16, 4: np.float32, 8: np.float64}[eb.value]
        buf = (C.c_char * (self.NP * eb.value)).from_address(ptr)
        return np.frombuffer(buf, dtype=dt).reshape((self.I + 1, self.J, self.K))

    def get(self, name, padded=False):
        a = self._array(name).copy()
        return a if padded else a[: self.I]

    def set(self, name, arr, padded=False):
        a = self._array(name)
        v = np.asarray(arr).reshape((self.I + (1 if padded else 0), self.J, self.K))
        if padded:
            a[...] = v
        else:
            a[: self.I] = v

    def call(self, method, arg=0.0):
        r = C.c_int(0)
        if self.L.lsref_call(self.h, method.encode(), float(arg), C.byref(r)) != 0:
            raise RuntimeError(f"{method}: {self.L.lsref_last_error().decode()}")
        return r.value

    def write_checkpoint(self, directory, step):
        """Simulation::writeCheckpoint: <directory>/checkpoint_rank0_<step>.bin"""
        if self.L.lsref_checkpoint(self.h, str(directory).encode(), int(step), 1) != 0:
            raise RuntimeError(self.L.lsref_last_error().decode())

    def load_checkpoint(self, directory, step):
        if self.L.lsref_checkpoint(self.h, str(directory).encode(), int(step), 0) != 0:
            raise RuntimeError(self.L.lsref_last_error().decode())

    def load_labels(self, labels):
        self.set("label", np.asarray(labels))

    def init_all(self):
        if self.L.lsref_init(self.h) != 0:
            raise RuntimeError(self.L.lsref_last_error().decode())
        return int(self.L.lsref_initial_sulphide_count(self.h))

    def props(self):
        for m in ("updateRelativePermeability", "updateCapillaryPressure", "initProperties"):
            self.call(m)

    def step(self, t, dt):
        """One attempt of src/main.cpp:303-432 with explicit saturation (no retry)."""
        self.call("saveState")
        self.props()
        self.call("setupPressureEqns", t)
        if not self.call("solvePressure"):
            return False, 0
        self.call("calculateFlux")
        self.call("updateSaturation", dt)
        self.call("handleSurfaceEffects")
        self.call("setupConcentrationEqns_conc", dt)
        if not self.call("solveConc"):
            return False, 0
        self.call("setupConcentrationEqns_acid", dt)
        if not self.call("solveAcid"):
            return False, 0
        self.call("handlePrecipitation")
        return True, self.call("updateFrac", dt)
