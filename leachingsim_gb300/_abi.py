"""ctypes mirror of include/leachingsim.h (structs, enums and signatures).

The structs here must stay field-for-field identical to the C header; the
CPU test suite checks their sizes against the compiled library.
"""
import ctypes as C

AIR, PORE, ROCK, SULPHIDE, PRECIPITATE = 1, 2, 3, 4, 5

LS_OK = 0
LS_NOT_CONVERGED = 1
LS_STAGNATED_FALLBACK_USED = 2
LS_NONFINITE = 3
LS_BAD_ARG = 4
LS_CUDA_ERROR = 5
LS_TIMEOUT = 6
LS_NO_DEVICE = 7
LS_UNPHYSICAL = 8

STATUS_NAMES = {
    0: "LS_OK", 1: "LS_NOT_CONVERGED", 2: "LS_STAGNATED_FALLBACK_USED",
    3: "LS_NONFINITE", 4: "LS_BAD_ARG", 5: "LS_CUDA_ERROR", 6: "LS_TIMEOUT",
    7: "LS_NO_DEVICE", 8: "LS_UNPHYSICAL",
}

# ls_field
FIELDS = {
    "label": 0, "frac": 1, "permeability": 2, "viscosity": 3, "pressure": 4,
    "conc": 5, "acid": 6, "flux_x": 7, "flux_y": 8, "flux_z": 9,
    "saturation": 10, "cap_pressure": 11, "rel_perm": 12, "precipitate": 13,
    "kmult": 14,
}
# every other field is float64; labels per label_bytes
FIELD_DTYPES = {0: None, 1: "float32", 14: "float32"}

# ls_bc_mode
BC_REFERENCE, BC_FLOW_I = 0, 1

# ls_memory_mode
MEM_RESIDENT, MEM_LEAN = 0, 1

# ls_press_solver
PRESS_MIXED, PRESS_FP64, PRESS_JACOBI64, PRESS_LEARNED = 0, 1, 2, 3

# ls_timer
TIMERS = {
    "props": 0, "press_setup": 1, "press_inner": 2, "press_outer": 3, "flux": 4,
    "saturation": 5, "transport": 6, "precip": 7, "dissolve": 8, "snapshot": 9,
    "kry_apply": 10, "cg_apply": 11,
}


class LsParams(C.Structure):
    _fields_ = [
        ("D", C.c_double), ("dx", C.c_double), ("Dpore_fac", C.c_double),
        ("kext", C.c_double), ("kreac", C.c_double), ("theta", C.c_double),
        ("c_sat", C.c_double), ("evaporative_flux", C.c_double),
        ("top_pressure", C.c_double), ("max_cap_grad", C.c_double),
        ("vg_alpha", C.c_double), ("vg_n", C.c_double), ("s_res", C.c_double),
        ("porosity", C.c_double), ("time_scalar", C.c_double),
        ("rock_D_fac", C.c_double), ("alpha_transfer", C.c_double),
        ("solid_density", C.c_double),
        ("use_instant_precipitation", C.c_int), ("use_implicit_saturation", C.c_int),
        ("enable_microporosity", C.c_int), ("debug_mode", C.c_int),
        ("compat_shift", C.c_int),
        ("press_rtol", C.c_double), ("press_max_it", C.c_int), ("press_solver", C.c_int),
        ("conc_rtol", C.c_double), ("conc_max_it", C.c_int),
        ("sat_rtol", C.c_double), ("sat_max_it", C.c_int),
        ("bc_mode", C.c_int), ("p_inlet", C.c_double), ("p_outlet", C.c_double),
        ("conc_inlet", C.c_double), ("acid_inlet", C.c_double),
        ("pore_permeability", C.c_double), ("rock_permeability", C.c_double),
        ("memory_mode", C.c_int),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class LsSolveInfo(C.Structure):
    _fields_ = [
        ("iterations", C.c_int), ("outer_iterations", C.c_int), ("converged", C.c_int),
        ("reason", C.c_int), ("rel_residual", C.c_double), ("min_value", C.c_double),
        ("max_value", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class LsSubstepInfo(C.Structure):
    _fields_ = [("max_rate", C.c_double), ("num_steps", C.c_int), ("dt_sub", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class LsBudget(C.Structure):
    _fields_ = [
        ("conc", C.c_double), ("acid", C.c_double), ("mineral", C.c_double),
        ("precipitate", C.c_double), ("acid_consumed", C.c_double),
        ("mineral_dissolved", C.c_double), ("sulphide_voxels", C.c_longlong),
        ("precipitate_voxels", C.c_longlong),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class LsStepInfo(C.Structure):
    _fields_ = [
        ("pressure", LsSolveInfo), ("saturation", LsSubstepInfo),
        ("saturation_solve", LsSolveInfo), ("conc", LsSolveInfo), ("acid", LsSolveInfo),
        ("leaching", LsSubstepInfo), ("leached", C.c_int), ("picard_iterations", C.c_int),
        ("success", C.c_int), ("budget", LsBudget),
    ]

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = v.as_dict() if hasattr(v, "as_dict") else v
        return out


def default_params(**overrides):
    """CLI defaults of the reference (src/main.cpp:39, 89-91) plus this library's solver
    defaults; keyword overrides set fields by name."""
    p = LsParams()
    p.D = 1.0
    p.dx = 1.0
    p.Dpore_fac = 1.0
    p.kext = 1.0
    p.kreac = 1.0
    p.theta = 1.0
    p.c_sat = 0.95
    p.evaporative_flux = 0.0
    p.top_pressure = 10000.0
    p.max_cap_grad = 50000.0
    p.vg_alpha = 1.0
    p.vg_n = 2.0
    p.s_res = 0.05
    p.porosity = 0.1
    p.time_scalar = 1.0
    p.rock_D_fac = 1e-4
    p.alpha_transfer = 1e-5
    p.solid_density = 1.0
    p.use_instant_precipitation = 0
    p.use_implicit_saturation = 0
    p.enable_microporosity = 0
    p.debug_mode = 0
    p.compat_shift = 1
    p.press_rtol = 1e-8
    p.press_max_it = 10000
    p.press_solver = PRESS_MIXED
    p.conc_rtol = 1e-10
    p.conc_max_it = 10000
    p.sat_rtol = 1e-10
    p.sat_max_it = 10000
    p.bc_mode = BC_REFERENCE
    p.p_inlet = 1.0
    p.p_outlet = 0.0
    p.conc_inlet = 0.0
    p.acid_inlet = 0.0
    p.pore_permeability = 1.0e-12
    p.rock_permeability = 1.0e-18
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(f"ls_params has no field {k!r}")
        setattr(p, k, v)
    return p
