"""ctypes front end of the CPU oracle (oracle/ls_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package. Its parity with the
reference's own code is checked by tests/test_ref_pin.py; see ls_oracle.h.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from leachingsim_gb300._abi import (FIELDS, LsParams, LsSolveInfo, LsStepInfo,
                                    LsSubstepInfo, default_params)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblsoracle.so")

SOLVE_REFERENCE = 0
SOLVE_TIGHT = 1
SOLVE_PCG = 2
SOLVE_PRODUCTION = 3


def build(force=False):
    """Compile the oracle with the system C compiler (no FMA contraction, OpenMP)."""
    src = os.path.join(_HERE, "ls_oracle.c")
    deps = [src, os.path.join(_HERE, "ls_oracle.h"),
            os.path.join(os.path.dirname(_HERE), "include", "leachingsim.h")]
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(d) for d in deps):
        return LIB_PATH
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-Wall", "-o", LIB_PATH + ".tmp", src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class LsoSolverCfg(C.Structure):
    _fields_ = [("mode", C.c_int), ("restart", C.c_int), ("rtol", C.c_double),
                ("max_it", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, d, i, sz = C.c_void_p, C.c_double, C.c_int, C.c_size_t
        sigs = {
            "lso_params_default": (None, [C.POINTER(LsParams)]),
            "lso_create": (vp, [i, i, i, i, C.POINTER(LsParams)]),
            "lso_destroy": (None, [vp]),
            "lso_set_params": (None, [vp, C.POINTER(LsParams)]),
            "lso_set_solver": (None, [vp, C.POINTER(LsoSolverCfg)]),
            "lso_num_threads": (i, []),
            "lso_set_num_threads": (None, [i]),
            "lso_set_field": (i, [vp, i, vp, sz, i]),
            "lso_get_field": (i, [vp, i, vp, sz, i]),
            "lso_init_fields": (None, [vp]),
            "lso_init_frac": (C.c_ulonglong, [vp]),
            "lso_init_saturation": (None, [vp]),
            "lso_init_acid": (None, [vp]),
            "lso_update_relperm": (None, [vp]),
            "lso_update_cap": (None, [vp]),
            "lso_init_properties": (None, [vp]),
            "lso_setup_pressure": (None, [vp, d]),
            "lso_solve_pressure": (i, [vp, C.POINTER(LsSolveInfo)]),
            "lso_pressure_apply": (None, [vp, vp, vp]),
            "lso_pressure_rhs": (None, [vp, vp]),
            "lso_pressure_rowkind": (None, [vp, vp]),
            "lso_pressure_diag": (None, [vp, vp]),
            "lso_calculate_flux": (None, [vp]),
            "lso_update_saturation": (None, [vp, d, C.POINTER(LsSubstepInfo)]),
            "lso_setup_saturation": (None, [vp, d]),
            "lso_solve_saturation": (i, [vp, C.POINTER(LsSolveInfo), C.POINTER(C.c_int)]),
            "lso_handle_surface": (None, [vp]),
            "lso_setup_conc": (None, [vp, d, i]),
            "lso_solve_conc": (i, [vp, i, C.POINTER(LsSolveInfo)]),
            "lso_transport_apply": (None, [vp, vp, vp]),
            "lso_transport_rhs": (None, [vp, vp]),
            "lso_handle_precip": (None, [vp]),
            "lso_update_frac": (i, [vp, d, C.POINTER(LsSubstepInfo)]),
            "lso_save_state": (None, [vp]),
            "lso_restore_state": (None, [vp]),
            "lso_step": (i, [vp, d, d, C.POINTER(LsStepInfo)]),
            "lso_initial_sulphide_count": (C.c_ulonglong, [vp]),
            "lso_write_checkpoint": (i, [vp, C.c_char_p]),
            "lso_load_checkpoint": (i, [vp, C.c_char_p]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """One simulation domain on the CPU, restating the reference's np=1 semantics."""

    def __init__(self, shape, label_bytes=1, params=None, mode=SOLVE_TIGHT, rtol=1e-13,
                 restart=60, max_it=200000, threads=None):
        self.shape = tuple(int(v) for v in shape)
        I, J, K = self.shape
        self.I, self.J, self.K = I, J, K
        self.N = I * J * K
        self.NP = (I + 1) * J * K
        self.label_bytes = label_bytes
        self.params = params if params is not None else default_params()
        L = lib()
        if threads is not None:
            L.lso_set_num_threads(int(threads))
        self.h = L.lso_create(I, J, K, label_bytes, C.byref(self.params))
        if not self.h:
            raise ValueError(f"oracle rejected shape {shape} / label_bytes {label_bytes}")
        self.set_solver(mode, rtol=rtol, restart=restart, max_it=max_it)

    def close(self):
        if getattr(self, "h", None):
            lib().lso_destroy(self.h)
            self.h = None

    __del__ = close

    def set_solver(self, mode, rtol=-1.0, restart=30, max_it=-1):
        cfg = LsoSolverCfg(mode, restart, rtol, max_it)
        lib().lso_set_solver(self.h, C.byref(cfg))

    def set_params(self, params):
        self.params = params
        lib().lso_set_params(self.h, C.byref(params))

    # fields -------------------------------------------------------------
    def _dtype(self, fid):
        if fid == 0:
            return np.uint16
        if fid in (1, 14):
            return np.float32
        return np.float64

    def get(self, name, padded=False):
        fid = FIELDS[name]
        n = self.NP if padded else self.N
        out = np.empty(n, dtype=self._dtype(fid))
        if lib().lso_get_field(self.h, fid, _ptr(out), n, int(padded)) != 0:
            raise ValueError(name)
        shape = (self.I + (1 if padded else 0), self.J, self.K)
        return out.reshape(shape)

    def set(self, name, arr, padded=False):
        fid = FIELDS[name]
        a = np.ascontiguousarray(np.asarray(arr).reshape(-1), dtype=self._dtype(fid))
        if lib().lso_set_field(self.h, fid, _ptr(a), a.size, int(padded)) != 0:
            raise ValueError(f"{name}: bad size {a.size}")

    # initialisation -------------------------------------------------------
    def load_labels(self, labels):
        self.set("label", np.asarray(labels).astype(np.uint16))

    def init_all(self):
        """Fresh start of src/main.cpp:189-206."""
        L = lib()
        L.lso_init_fields(self.h)
        count = L.lso_init_frac(self.h)
        L.lso_init_saturation(self.h)
        L.lso_init_acid(self.h)
        self.props()
        return count

    def props(self):
        L = lib()
        L.lso_update_relperm(self.h)
        L.lso_update_cap(self.h)
        L.lso_init_properties(self.h)

    # hot path pieces ------------------------------------------------------
    def pressure(self, t):
        info = LsSolveInfo()
        lib().lso_setup_pressure(self.h, float(t))
        ok = lib().lso_solve_pressure(self.h, C.byref(info))
        return bool(ok), info.as_dict()

    def setup_pressure(self, t):
        lib().lso_setup_pressure(self.h, float(t))

    def pressure_apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        y = np.empty_like(x)
        lib().lso_pressure_apply(self.h, _ptr(x), _ptr(y))
        return y

    def pressure_rhs(self):
        b = np.empty(self.N)
        lib().lso_pressure_rhs(self.h, _ptr(b))
        return b

    def pressure_rowkind(self):
        k = np.empty(self.N, dtype=np.int8)
        lib().lso_pressure_rowkind(self.h, _ptr(k))
        return k

    def pressure_diag(self):
        d = np.empty(self.N)
        lib().lso_pressure_diag(self.h, _ptr(d))
        return d

    def flux(self):
        lib().lso_calculate_flux(self.h)

    def saturation(self, dt):
        info = LsSubstepInfo()
        lib().lso_update_saturation(self.h, float(dt), C.byref(info))
        return info.as_dict()

    def saturation_implicit(self, dt):
        info = LsSolveInfo()
        valid = C.c_int(1)
        lib().lso_setup_saturation(self.h, float(dt))
        ok = lib().lso_solve_saturation(self.h, C.byref(info), C.byref(valid))
        return bool(ok), bool(valid.value), info.as_dict()

    def surface(self):
        lib().lso_handle_surface(self.h)

    def transport(self, dt, which):
        info = LsSolveInfo()
        lib().lso_setup_conc(self.h, float(dt), int(which))
        ok = lib().lso_solve_conc(self.h, int(which), C.byref(info))
        return bool(ok), info.as_dict()

    def setup_transport(self, dt, which):
        lib().lso_setup_conc(self.h, float(dt), int(which))

    def transport_apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        y = np.empty_like(x)
        lib().lso_transport_apply(self.h, _ptr(x), _ptr(y))
        return y

    def transport_rhs(self):
        b = np.empty(self.N)
        lib().lso_transport_rhs(self.h, _ptr(b))
        return b

    def precip(self):
        lib().lso_handle_precip(self.h)

    def dissolve(self, dt):
        info = LsSubstepInfo()
        n = lib().lso_update_frac(self.h, float(dt), C.byref(info))
        return n, info.as_dict()

    def save_state(self):
        lib().lso_save_state(self.h)

    def restore_state(self):
        lib().lso_restore_state(self.h)

    def step(self, t, dt):
        info = LsStepInfo()
        ok = lib().lso_step(self.h, float(t), float(dt), C.byref(info))
        return bool(ok), info.as_dict()

    def write_checkpoint(self, path):
        return lib().lso_write_checkpoint(self.h, path.encode())

    def load_checkpoint(self, path):
        return lib().lso_load_checkpoint(self.h, path.encode())

    def run(self, tmax, dt, t0=0.0, n0=0, on_step=None):
        """Time loop of src/main.cpp:293-558 with the retry manager and dt ramp
        (no output files). Returns the list of per-step info dicts."""
        t, n = t0, n0
        dt_target = dt
        current_dt = min(60.0, dt_target) if n0 == 0 else dt_target
        log = []
        while True:
            while True:
                ok, info = self.step(t, current_dt)
                if ok:
                    break
                self.restore_state()
                current_dt *= 0.5
                if current_dt < 1e-3:
                    raise RuntimeError("time step shrank below 1 ms")
            info["t"], info["n"], info["dt"] = t, n, current_dt
            log.append(info)
            if on_step is not None:
                on_step(n, t, self)
            t += current_dt
            n += 1
            if current_dt < dt_target:
                current_dt = min(current_dt * 1.5, dt_target)
            if not (t < tmax):
                break
        return log
