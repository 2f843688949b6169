"""The C-ABI library: loads without a GPU, exports every function include/leachingsim.h
declares, and its structs have the layout the ctypes mirror assumes. No compute calls."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from leachingsim_gb300 import _abi, runtime

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "leachingsim.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(ls_\w+)\s*\(", text)
    return sorted(set(names))


def test_library_loads_and_exports_all_declared_symbols():
    L = runtime.load()
    names = declared_functions()
    assert len(names) >= 38
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, f"not exported: {missing}"
    # every declared function is bound by the Python runtime with a signature
    unbound = [n for n in names if n not in runtime.SYMBOLS]
    assert not unbound, f"declared but not bound in runtime.py: {unbound}"


def test_abi_version():
    assert runtime.load().ls_abi_version() == 3


def test_struct_layout_matches_header():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "leachingsim.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(ls_params), sizeof(ls_solve_info),
         sizeof(ls_substep_info), sizeof(ls_step_info));
  printf("%zu %zu %zu\n", offsetof(ls_params, compat_shift), offsetof(ls_params, press_solver),
         offsetof(ls_params, sat_max_it));
  printf("%zu %zu\n", offsetof(ls_step_info, leached), offsetof(ls_step_info, success));
  printf("%zu %zu %zu %zu\n", offsetof(ls_params, bc_mode), offsetof(ls_params, rock_permeability),
         offsetof(ls_step_info, budget), sizeof(ls_budget));
  printf("%zu %d %d\n", offsetof(ls_params, memory_mode), (int)LS_MEM_RESIDENT, (int)LS_MEM_LEAN);
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    vals = [int(v) for v in out]
    assert vals[0] == C.sizeof(_abi.LsParams)
    assert vals[1] == C.sizeof(_abi.LsSolveInfo)
    assert vals[2] == C.sizeof(_abi.LsSubstepInfo)
    assert vals[3] == C.sizeof(_abi.LsStepInfo)
    assert vals[4] == _abi.LsParams.compat_shift.offset
    assert vals[5] == _abi.LsParams.press_solver.offset
    assert vals[6] == _abi.LsParams.sat_max_it.offset
    assert vals[7] == _abi.LsStepInfo.leached.offset
    assert vals[8] == _abi.LsStepInfo.success.offset
    assert vals[9] == _abi.LsParams.bc_mode.offset
    assert vals[10] == _abi.LsParams.rock_permeability.offset
    assert vals[11] == _abi.LsStepInfo.budget.offset
    assert vals[12] == C.sizeof(_abi.LsBudget)
    assert vals[13] == _abi.LsParams.memory_mode.offset
    assert (vals[14], vals[15]) == (_abi.MEM_RESIDENT, _abi.MEM_LEAN)


def test_defaults_match_between_c_and_python():
    L = runtime.load()
    p = _abi.LsParams()
    L.ls_params_default(C.byref(p))
    assert p.as_dict() == _abi.default_params().as_dict()


def test_create_rejects_bad_arguments_without_touching_a_gpu():
    L = runtime.load()
    h = C.c_void_p()
    # argument checks come before any device query
    assert L.ls_create(C.byref(h), 1, 8, 8, 1, None) == _abi.LS_BAD_ARG
    assert L.ls_create(C.byref(h), 8, 8, 8, 3, None) == _abi.LS_BAD_ARG
    assert L.ls_create(None, 8, 8, 8, 1, None) == _abi.LS_BAD_ARG
    assert L.ls_last_error(None) == b"null context"
    assert L.ls_destroy(None) == _abi.LS_OK


def test_create_rejects_grids_beyond_32_bit_indices():
    """Voxel ids and row indices are 32-bit: (I+1)*J*K plus a plane and a grid stride of
    headroom must stay below 2^31; larger grids are refused before any device work (the
    large single domain, 768 x 1024 x 1024, is inside the limit)."""
    L = runtime.load()
    h = C.c_void_p()
    p = _abi.default_params()
    assert L.ls_create(C.byref(h), 1300, 1300, 1300, 1, C.byref(p)) == _abi.LS_BAD_ARG
    assert not h.value
    assert L.ls_create(C.byref(h), 1, 8, 8, 1, C.byref(p)) == _abi.LS_BAD_ARG
    assert L.ls_create(C.byref(h), 8, 8, 8, 3, C.byref(p)) == _abi.LS_BAD_ARG
    assert (768 + 1) * 1024 * 1024 + 1024 * 1024 + (1 << 22) < (1 << 31)
