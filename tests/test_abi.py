"""The C-ABI library builds, loads and exports every entry point that
include/nekcem_gpu.h declares; argument errors come back as status codes
(no GPU is needed for any of this)."""
import ctypes as C
import os
import re

import pytest

from nekcem_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "nekcem_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nekgpu_\w+)\s*\(", src)))


def test_header_declares_the_boundary_entry_points():
    """The calls a Fortran driver makes in place of cem_maxwell_init,
    cem_maxwell_op_rk and cem_error, and the adjoint pair."""
    names = declared()
    for must in ("nekgpu_init", "nekgpu_set_state", "nekgpu_get_state", "nekgpu_stage",
                 "nekgpu_step", "nekgpu_norms", "nekgpu_finalize", "nekgpu_op_rk_host",
                 "nekgpu_adjoint_init", "nekgpu_adjoint_run"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = L.load()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    bound = {n for n, _, _ in L.SIGNATURES}
    assert set(declared()) <= bound, set(declared()) - bound


def test_error_strings():
    lib = L.load()
    for code in range(0, -10, -1):
        s = lib.nekgpu_error_string(code).decode()
        assert s and s != "unknown status"
    assert lib.nekgpu_error_string(-99).decode() == "unknown status"
    assert lib.nekgpu_version() >= 1


def test_null_arguments_are_rejected():
    lib = L.load()
    h = C.c_void_p()
    assert lib.nekgpu_init(None, None, 2) == -1
    assert lib.nekgpu_init(C.byref(h), None, 2) == -1
    assert lib.nekgpu_init_box(C.byref(h), None, 2) == -1
    assert lib.nekgpu_finalize(None) == -1
    assert lib.nekgpu_step(None, 1, None, 0.1) == -1
    assert lib.nekgpu_set_state(None, None, None, 0) == -1
    b = L.NekgpuBox()
    b.N = 3; b.nelx = b.nely = b.nelz = 2
    for d in range(3):
        b.lo[d] = 0.0; b.hi[d] = 1.0; b.bc[d] = 0
    assert lib.nekgpu_init_box(C.byref(h), C.byref(b), 7) == -1  # unknown form
    b.bc[2] = 5
    assert lib.nekgpu_init_box(C.byref(h), C.byref(b), 2) == -1  # bad boundary code


def test_device_check_without_gpu_is_a_status():
    lib = L.load()
    st = lib.nekgpu_device_check(0)
    assert st in (0, -3)
