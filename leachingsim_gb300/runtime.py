"""ctypes binding of libleachingsim_gb300.so (the C-ABI of include/leachingsim.h).

There is no fallback: if the CUDA library cannot be loaded, or no GPU is
present, creating a Context raises.
"""
import ctypes as C
import os

import numpy as np

from . import _abi
from ._abi import FIELDS, LsParams, LsSolveInfo, LsStepInfo, LsSubstepInfo, TIMERS

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libleachingsim_gb300.so")

SYMBOLS = {
    # name: (restype, argtypes)
    "ls_params_default": (None, [C.POINTER(LsParams)]),
    "ls_abi_version": (C.c_int, []),
    "ls_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_int,
                            C.POINTER(LsParams)]),
    "ls_destroy": (C.c_int, [C.c_void_p]),
    "ls_last_error": (C.c_char_p, [C.c_void_p]),
    "ls_set_params": (C.c_int, [C.c_void_p, C.POINTER(LsParams)]),
    "ls_get_params": (C.c_int, [C.c_void_p, C.POINTER(LsParams)]),
    "ls_stream": (C.c_void_p, [C.c_void_p]),
    "ls_synchronize": (C.c_int, [C.c_void_p]),
    "ls_device_bytes": (C.c_size_t, [C.c_void_p]),
    "ls_device_peak_bytes": (C.c_size_t, [C.c_void_p]),
    "ls_host_bytes": (C.c_size_t, [C.c_void_p]),
    "ls_upload_field": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_int]),
    "ls_download_field": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_int]),
    "ls_upload_field_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_int]),
    "ls_download_field_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_int]),
    "ls_download_fields_async": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                           C.POINTER(C.c_void_p)]),
    "ls_event_wait": (C.c_int, [C.c_void_p]),
    "ls_event_release": (None, [C.c_void_p]),
    "ls_host_alloc": (C.c_void_p, [C.c_size_t]),
    "ls_host_free": (None, [C.c_void_p]),
    "ls_count_nonfinite": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_longlong)]),
    "ls_init_fields": (C.c_int, [C.c_void_p]),
    "ls_init_frac": (C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong)]),
    "ls_init_saturation": (C.c_int, [C.c_void_p]),
    "ls_init_acid": (C.c_int, [C.c_void_p]),
    "ls_props": (C.c_int, [C.c_void_p]),
    "ls_pressure_step": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(LsSolveInfo)]),
    "ls_flux": (C.c_int, [C.c_void_p]),
    "ls_saturation": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(LsSubstepInfo)]),
    "ls_saturation_implicit": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(LsSolveInfo)]),
    "ls_saturation_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                        C.c_double, C.c_double, C.c_void_p, C.POINTER(LsSubstepInfo),
                                        C.c_char_p, C.c_size_t]),
    "ls_surface": (C.c_int, [C.c_void_p]),
    "ls_transport": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.POINTER(LsSolveInfo),
                               C.POINTER(LsSolveInfo)]),
    "ls_precip": (C.c_int, [C.c_void_p]),
    "ls_dissolve": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_int),
                              C.POINTER(LsSubstepInfo)]),
    "ls_snapshot": (C.c_int, [C.c_void_p]),
    "ls_rollback": (C.c_int, [C.c_void_p]),
    "ls_step": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.POINTER(LsStepInfo)]),
    "ls_pressure_setup": (C.c_int, [C.c_void_p, C.c_double]),
    "ls_pressure_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "ls_pressure_rhs": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ls_transport_apply": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]),
    "ls_geom_coarsen": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "ls_geom_clean": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p]),
    "ls_lpnet_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "ls_lpnet_destroy": (C.c_int, [C.c_void_p]),
    "ls_lpnet_last_error": (C.c_char_p, [C.c_void_p]),
    "ls_lpnet_param_count": (C.c_longlong, [C.c_void_p]),
    "ls_lpnet_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "ls_lpnet_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "ls_lpnet_get_grads": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "ls_lpnet_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ls_lpnet_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_longlong, C.c_float, C.c_int, C.POINTER(C.c_double)]),
    "ls_pressure_learned_inputs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ls_pressure_solve_start": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.POINTER(LsSolveInfo)]),
    "ls_pressure_set_precond_weights": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "ls_pressure_fallbacks": (C.c_longlong, [C.c_void_p]),
    "ls_dissolve_fallbacks": (C.c_longlong, [C.c_void_p]),
    "ls_pressure_mg_level": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]),
    "ls_field_pool2": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ls_field_up2": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "ls_geom_distance": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "ls_geom_fracture": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ls_geom_classify": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                   C.c_int, C.c_void_p]),
    "ls_timing_enable": (C.c_int, [C.c_void_p, C.c_int]),
    "ls_timing_reset": (C.c_int, [C.c_void_p]),
    "ls_timing_get": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                C.POINTER(C.c_longlong)]),
    "ls_timing_bytes": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "ls_kernel_launches": (C.c_longlong, [C.c_void_p]),
}

_lib = None


def load(build_if_missing=True):
    """Load the CUDA library (building it in-tree first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build
        build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run python -m leachingsim_gb300.build")
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SYMBOLS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class LsError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{_abi.STATUS_NAMES.get(status, status)}: {message}")


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


_LABEL_DTYPES = {1: np.uint8, 2: np.uint16}


def _geom_check(st, what):
    if st != 0:
        raise RuntimeError(f"{what} failed with status {st}")


def geom_coarsen(labels):
    """coarsen_grid.py on the GPU: 2x2x2 ranked priority voting (Sulphide > Air > Pore >
    Rock); an odd slowest extent is padded with one Air plane."""
    lab = np.ascontiguousarray(labels)
    if lab.dtype not in (np.uint8, np.uint16) or lab.ndim != 3:
        raise ValueError("labels must be a 3-D uint8 or uint16 array")
    I, J, K = lab.shape
    if J % 2 or K % 2:
        raise ValueError("coarsening needs even y and x extents")
    out = np.empty(((I + 1) // 2, J // 2, K // 2), dtype=lab.dtype)
    _geom_check(load().ls_geom_coarsen(I, J, K, lab.itemsize, _p(lab), _p(out)), "ls_geom_coarsen")
    return out


def geom_clean(labels, mode="agglomerate"):
    """clean_micro_ct.py on the GPU; returns (cleaned labels, number of Pore voxels turned to
    Rock). mode: 'agglomerate' or 'core_sample'."""
    modes = {"agglomerate": 0, "core_sample": 1}
    if mode not in modes:
        raise ValueError(f"mode must be one of {sorted(modes)}")
    lab = np.array(labels, copy=True, order="C")
    if lab.dtype not in (np.uint8, np.uint16) or lab.ndim != 3:
        raise ValueError("labels must be a 3-D uint8 or uint16 array")
    n = C.c_longlong(0)
    _geom_check(load().ls_geom_clean(*lab.shape, lab.itemsize, _p(lab), modes[mode], C.byref(n)),
                "ls_geom_clean")
    return lab, int(n.value)


def geom_fracture(labels):
    """micro_fracture.py on the GPU; returns (labels after drilling, number of Rock voxels
    turned to Pore, number of encapsulated Sulphide voxels)."""
    lab = np.array(labels, copy=True, order="C")
    if lab.dtype not in (np.uint8, np.uint16) or lab.ndim != 3:
        raise ValueError("labels must be a 3-D uint8 or uint16 array")
    n, ne = C.c_longlong(0), C.c_longlong(0)
    _geom_check(load().ls_geom_fracture(*lab.shape, lab.itemsize, _p(lab), C.byref(n), C.byref(ne)),
                "ls_geom_fracture")
    return lab, int(n.value), int(ne.value)


def geom_distance(sites):
    """Euclidean distance to the nearest site (sites > 0.5) of a torch CUDA float32 (I, J, K)
    tensor; -1 where there is no site."""
    import torch
    t = sites.to(device="cuda", dtype=torch.float32).contiguous()
    out = torch.empty_like(t)
    torch.cuda.synchronize()
    _geom_check(load().ls_geom_distance(*t.shape, C.c_void_p(t.data_ptr()), C.c_void_p(out.data_ptr())),
                "ls_geom_distance")
    return out


def field_pool2(fine, weight=None):
    """(Weighted) 2x2x2 block means of a torch CUDA float32 (D, H, W) field (even extents)."""
    import torch
    f = fine.contiguous()
    w = weight.contiguous() if weight is not None else None
    D, H, W = f.shape
    out = torch.empty((D // 2, H // 2, W // 2), dtype=torch.float32, device=f.device)
    torch.cuda.synchronize()
    _geom_check(load().ls_field_pool2(D, H, W, C.c_void_p(f.data_ptr()),
                                      C.c_void_p(w.data_ptr()) if w is not None else None,
                                      C.c_void_p(out.data_ptr())), "ls_field_pool2")
    return out


def field_up2(coarse):
    """Each value of a torch CUDA float32 (D, H, W) field repeated over a 2x2x2 block."""
    import torch
    c = coarse.contiguous()
    D, H, W = (2 * v for v in c.shape)
    out = torch.empty((D, H, W), dtype=torch.float32, device=c.device)
    torch.cuda.synchronize()
    _geom_check(load().ls_field_up2(D, H, W, C.c_void_p(c.data_ptr()), C.c_void_p(out.data_ptr())),
                "ls_field_up2")
    return out


def geom_classify(grey, thresholds, labels, label_bytes=1):
    """Threshold classification of a uint16 grey-level image on the GPU: label = labels[i],
    i = the number of the ascending thresholds <= the grey value."""
    g = np.ascontiguousarray(grey, dtype=np.uint16)
    if g.ndim != 3:
        raise ValueError("grey must be a 3-D array")
    t = np.ascontiguousarray(thresholds, dtype=np.uint16)
    lb = np.ascontiguousarray(labels, dtype=np.int32)
    if lb.size != t.size + 1:
        raise ValueError("labels needs one entry more than thresholds")
    out = np.empty(g.shape, dtype=_LABEL_DTYPES[label_bytes])
    _geom_check(load().ls_geom_classify(*g.shape, _p(g), t.size, _p(t) if t.size else None, _p(lb),
                                        label_bytes, _p(out)), "ls_geom_classify")
    return out


# layer (name, cin, cout) of the learned pressure network, in parameter order
LPNET_LAYERS = [("W0a", 16, 16), ("W0b", 16, 16), ("W1", 16, 32), ("W2", 32, 64), ("W3", 64, 64),
                ("U2", 64, 32), ("U1", 32, 16), ("U0", 16, 16)]


def lpnet_flatten(params):
    """{name: (27, cout, cin) weights, name_b: (cout,) biases} -> flat float32 vector."""
    parts = []
    for name, cin, cout in LPNET_LAYERS:
        parts.append(np.asarray(params[name], np.float32).reshape(-1))
        parts.append(np.asarray(params[name + "_b"], np.float32).reshape(-1))
    return np.concatenate(parts)


def lpnet_unflatten(flat):
    out, o = {}, 0
    for name, cin, cout in LPNET_LAYERS:
        n = 27 * cout * cin
        out[name] = flat[o:o + n].reshape(27, cout, cin)
        o += n
        out[name + "_b"] = flat[o:o + cout].copy()
        o += cout
    return out


class PendingDownload:
    """Copies started by Context.download_async: wait() blocks until all have landed."""

    def __init__(self, ev, outs):
        self._ev = ev
        self.outs = outs  # keeps the buffers alive while the copies run

    def wait(self):
        if self._ev:
            st = load().ls_event_wait(self._ev)
            load().ls_event_release(self._ev)
            self._ev = None
            if st != 0:
                raise LsError(st, "ls_event_wait")
        return self.outs

    def __del__(self):
        try:
            self.wait()
        except Exception:
            pass


class LPNet:
    """The learned pressure network on the GPU (owns an ls_lpnet). Fields are torch CUDA
    float32 tensors of shape (D, H, W) or numpy arrays (copied to the device)."""

    def __init__(self, shape, seed=0):
        import torch  # noqa: F401  (device memory for the fields)
        self.shape = tuple(int(v) for v in shape)
        h = C.c_void_p()
        st = load().ls_lpnet_create(*self.shape, int(seed), C.byref(h))
        if st != 0:
            raise LsError(st, "ls_lpnet_create")
        self.h = h
        self.n = int(load().ls_lpnet_param_count(self.h))

    def close(self):
        if self.h:
            load().ls_lpnet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, allowed=(0,)):
        if st not in allowed:
            raise LsError(st, (load().ls_lpnet_last_error(self.h) or b"").decode())
        return st

    def _dev(self, a):
        import torch
        if isinstance(a, torch.Tensor):
            t = a.to(device="cuda", dtype=torch.float32).contiguous()
        else:
            t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
        if tuple(t.shape) != self.shape:
            raise ValueError(f"field shape {tuple(t.shape)} != {self.shape}")
        return t

    def get_params(self):
        out = np.empty(self.n, np.float32)
        self._check(load().ls_lpnet_get_params(self.h, _p(out), self.n))
        return out

    def set_params(self, flat):
        flat = np.ascontiguousarray(flat, np.float32)
        if flat.size != self.n:
            raise ValueError("wrong parameter count")
        self._check(load().ls_lpnet_set_params(self.h, _p(flat), self.n))

    def get_grads(self):
        out = np.empty(self.n, np.float32)
        self._check(load().ls_lpnet_get_grads(self.h, _p(out), self.n))
        return out

    def forward(self, c0, c1, c2):
        import torch
        t = [self._dev(c) for c in (c0, c1, c2)]
        out = torch.empty(self.shape, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        # status 2: a tensor-core wait gave up and the pass was recomputed with mma.sync
        self.last_status = self._check(load().ls_lpnet_forward(self.h, *[C.c_void_p(x.data_ptr()) for x in t],
                                                               C.c_void_p(out.data_ptr())), (0, 2))
        return out

    def train_step(self, c0, c1, c2, target, mask, lr=1e-3, update=True):
        import torch
        t = [self._dev(c) for c in (c0, c1, c2, target, mask)]
        count = int((t[4] > 0).sum().item())
        loss = C.c_double(0.0)
        torch.cuda.synchronize()
        self._check(load().ls_lpnet_train_step(self.h, *[C.c_void_p(x.data_ptr()) for x in t], max(count, 1),
                                               float(lr), 1 if update else 0, C.byref(loss)))
        return float(loss.value)


class Context:
    """One simulation domain on the GPU (owns an ls_ctx)."""

    def __init__(self, shape, label_bytes=1, params=None):
        L = load()
        self.shape = tuple(int(v) for v in shape)
        self.I, self.J, self.K = self.shape
        self.N = self.I * self.J * self.K
        self.NP = (self.I + 1) * self.J * self.K
        self.label_bytes = int(label_bytes)
        self.params = params if params is not None else _abi.default_params()
        h = C.c_void_p()
        st = L.ls_create(C.byref(h), self.I, self.J, self.K, self.label_bytes, C.byref(self.params))
        if st != 0:
            raise LsError(st, "ls_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().ls_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, allowed=(0,)):
        if st not in allowed:
            msg = load().ls_last_error(self.h)
            raise LsError(st, msg.decode() if msg else "")
        return st

    # parameters -----------------------------------------------------------
    def set_params(self, params):
        self.params = params
        self._check(load().ls_set_params(self.h, C.byref(params)))

    # transfers --------------------------------------------------------------
    def _dtype(self, fid):
        if fid == 0:
            return np.uint8 if self.label_bytes == 1 else np.uint16
        if fid in (1, 14):
            return np.float32
        return np.float64

    def upload(self, name, arr, padded=False):
        fid = FIELDS[name]
        a = np.ascontiguousarray(np.asarray(arr).reshape(-1), dtype=self._dtype(fid))
        self._check(load().ls_upload_field(self.h, fid, _p(a), a.size, int(padded)))

    def download_async(self, names, outs, padded=False):
        """Start copying the fields `names` into the host arrays `outs` (contiguous, of the
        fields' dtypes and sizes; page-locked for the copies to overlap) and return a
        PendingDownload; the context's later steps wait on the device only for the copies of
        the fields they overwrite."""
        fids = (C.c_int * len(names))(*[FIELDS[nm] for nm in names])
        n = self.NP if padded else self.N
        ptrs = (C.c_void_p * len(names))()
        for q, (nm, o) in enumerate(zip(names, outs)):
            if not (isinstance(o, np.ndarray) and o.flags.c_contiguous and o.size == n
                    and o.dtype == self._dtype(FIELDS[nm])):
                raise ValueError(f"buffer for {nm} must be a contiguous {self._dtype(FIELDS[nm])} array of {n}")
            ptrs[q] = o.ctypes.data
        ev = C.c_void_p()
        self._check(load().ls_download_fields_async(self.h, len(names), fids, ptrs, int(padded), C.byref(ev)))
        return PendingDownload(ev, list(outs))

    def count_nonfinite(self, name):
        c = C.c_longlong(0)
        self._check(load().ls_count_nonfinite(self.h, FIELDS[name], C.byref(c)))
        return int(c.value)

    def download(self, name, padded=False, out=None):
        fid = FIELDS[name]
        n = self.NP if padded else self.N
        if out is None:
            out = np.empty(n, dtype=self._dtype(fid))
        self._check(load().ls_download_field(self.h, fid, _p(out), n, int(padded)))
        return out.reshape((self.I + (1 if padded else 0), self.J, self.K))

    # initialisation ---------------------------------------------------------
    def init_all(self):
        """Fresh start of src/main.cpp:189-206; returns the initial sulphide count."""
        L = load()
        self._check(L.ls_init_fields(self.h))
        cnt = C.c_ulonglong(0)
        self._check(L.ls_init_frac(self.h, C.byref(cnt)))
        self._check(L.ls_init_saturation(self.h))
        self._check(L.ls_init_acid(self.h))
        self._check(L.ls_props(self.h))
        return int(cnt.value)

    def init_fields(self):
        self._check(load().ls_init_fields(self.h))

    def init_frac(self):
        cnt = C.c_ulonglong(0)
        self._check(load().ls_init_frac(self.h, C.byref(cnt)))
        return int(cnt.value)

    def init_saturation(self):
        self._check(load().ls_init_saturation(self.h))

    def init_acid(self):
        self._check(load().ls_init_acid(self.h))

    # hot path ---------------------------------------------------------------
    def props(self):
        self._check(load().ls_props(self.h))

    def pressure(self, t):
        info = LsSolveInfo()
        st = self._check(load().ls_pressure_step(self.h, float(t), C.byref(info)), (0, 1, 2, 3))
        return st in (0, 2), info.as_dict()

    def pressure_learned_inputs(self):
        """The learned start's input fields for the system assembled by pressure_setup(t):
        (Pore-row mask, (log10 K + 15) / 3, identity-row values / top pressure), torch CUDA
        float32 tensors of the grid's shape."""
        import torch
        out = [torch.empty(self.shape, dtype=torch.float32, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()
        self._check(load().ls_pressure_learned_inputs(self.h, *[C.c_void_p(t.data_ptr()) for t in out]))
        return tuple(out)

    def pressure_solve_start(self, start, scale=1.0):
        """Solve the assembled pressure system from x = scale * top pressure * start on the
        Pore rows (start: torch CUDA float32 tensor of the grid's shape)."""
        import torch
        if tuple(start.shape) != self.shape or start.dtype != torch.float32 or not start.is_cuda:
            raise ValueError("start must be a CUDA float32 tensor of the grid's shape")
        start = start.contiguous()
        info = LsSolveInfo()
        torch.cuda.synchronize()
        st = self._check(load().ls_pressure_solve_start(self.h, C.c_void_p(start.data_ptr()), float(scale),
                                                        C.byref(info)), (0, 1, 2, 3))
        return st in (0, 2), info.as_dict()

    def set_precond_weights(self, flat):
        """Weights of the learned coarse solver of the pressure multigrid (press_solver =
        PRESS_LEARNED): the flat float32 parameter vector of an ls_lpnet."""
        w = np.ascontiguousarray(flat, dtype=np.float32).ravel()
        self._check(load().ls_pressure_set_precond_weights(self.h, _p(w), w.size))

    def pressure_fallbacks(self):
        """Learned pressure solves on this context that fell back to the plain cycle."""
        return int(load().ls_pressure_fallbacks(self.h))

    def dissolve_fallbacks(self):
        """Dissolution calls on this context redone with the full wavefront schedule."""
        return int(load().ls_dissolve_fallbacks(self.h))

    def mg_level(self, level):
        """Multigrid level `level` of the last FP32-inner pressure solve: dict with its shape
        and host copies of comp (int32), e, f0, f1, f2 (float32)."""
        dims = np.zeros(3, dtype=np.int32)
        self._check(load().ls_pressure_mg_level(self.h, int(level), _p(dims), None, None, None, None, None))
        shape = tuple(int(v) for v in dims)
        out = {"shape": shape, "comp": np.empty(shape, np.int32)}
        for k in ("e", "f0", "f1", "f2"):
            out[k] = np.empty(shape, np.float32)
        self._check(load().ls_pressure_mg_level(self.h, int(level), _p(dims), _p(out["comp"]), _p(out["e"]),
                                                _p(out["f0"]), _p(out["f1"]), _p(out["f2"])))
        return out

    def flux(self):
        self._check(load().ls_flux(self.h))

    def saturation(self, dt):
        info = LsSubstepInfo()
        self._check(load().ls_saturation(self.h, float(dt), C.byref(info)))
        return info.as_dict()

    def saturation_implicit(self, dt):
        info = LsSolveInfo()
        st = self._check(load().ls_saturation_implicit(self.h, float(dt), C.byref(info)), (0, 1, 3, 8))
        return st == 0, st != 8, info.as_dict()

    def surface(self):
        self._check(load().ls_surface(self.h))

    def transport(self, dt, which=3):
        ci, ai = LsSolveInfo(), LsSolveInfo()
        st = self._check(load().ls_transport(self.h, float(dt), int(which), C.byref(ci), C.byref(ai)),
                         (0, 1, 3))
        return st == 0, ci.as_dict(), ai.as_dict()

    def precip(self):
        self._check(load().ls_precip(self.h))

    def dissolve(self, dt):
        n = C.c_int(0)
        info = LsSubstepInfo()
        self._check(load().ls_dissolve(self.h, float(dt), C.byref(n), C.byref(info)))
        return int(n.value), info.as_dict()

    def snapshot(self):
        self._check(load().ls_snapshot(self.h))

    def rollback(self):
        self._check(load().ls_rollback(self.h))

    def step(self, t, dt):
        info = LsStepInfo()
        self._check(load().ls_step(self.h, float(t), float(dt), C.byref(info)))
        d = info.as_dict()
        return bool(d["success"]), d

    def synchronize(self):
        self._check(load().ls_synchronize(self.h))

    def stream(self):
        return load().ls_stream(self.h)

    def device_bytes(self):
        return int(load().ls_device_bytes(self.h))

    def device_peak_bytes(self):
        """The most device bytes held at once (memory_mode MEM_LEAN: reserved by its pool)."""
        return int(load().ls_device_peak_bytes(self.h))

    def host_bytes(self):
        """Host bytes of the context (the snapshot of memory_mode MEM_LEAN)."""
        return int(load().ls_host_bytes(self.h))

    # test hooks -------------------------------------------------------------
    def pressure_setup(self, t):
        self._check(load().ls_pressure_setup(self.h, float(t)))

    def pressure_apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        y = np.empty_like(x)
        self._check(load().ls_pressure_apply(self.h, _p(x), _p(y)))
        return y

    def pressure_rhs(self):
        b = np.empty(self.N)
        self._check(load().ls_pressure_rhs(self.h, _p(b)))
        return b

    def transport_apply(self, dt, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        y = np.empty_like(x)
        self._check(load().ls_transport_apply(self.h, float(dt), _p(x), _p(y)))
        return y

    # timing -----------------------------------------------------------------
    def timing(self, enable=True):
        self._check(load().ls_timing_enable(self.h, int(bool(enable))))

    def timing_reset(self):
        self._check(load().ls_timing_reset(self.h))

    def timing_get(self, name):
        ms = C.c_double(0.0)
        cnt = C.c_longlong(0)
        self._check(load().ls_timing_get(self.h, TIMERS[name], C.byref(ms), C.byref(cnt)))
        return float(ms.value), int(cnt.value)

    def timing_bytes(self, name):
        b = C.c_double(0.0)
        self._check(load().ls_timing_bytes(self.h, TIMERS[name], C.byref(b)))
        return float(b.value)

    def launches(self):
        return int(load().ls_kernel_launches(self.h))

    # time loop --------------------------------------------------------------
    def run(self, tmax, dt, t0=0.0, n0=0, on_step=None, max_steps=None):
        """Time loop of src/main.cpp:293-558 (retry manager, dt ramp; no files)."""
        t, n = t0, n0
        dt_target = dt
        current_dt = min(60.0, dt_target) if n0 == 0 else dt_target
        log = []
        while True:
            while True:
                ok, info = self.step(t, current_dt)
                if ok:
                    break
                self.rollback()
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
            if not (t < tmax) or (max_steps is not None and len(log) >= max_steps):
                break
        return log
