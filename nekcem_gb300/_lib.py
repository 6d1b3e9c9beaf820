"""ctypes binding of the C ABI in ``include/nekcem_gpu.h``.

Loads the in-tree ``libnekcem_gb300.so`` (built by ``nekcem_gb300.build``).
There is no fallback: if the library is missing or the GPU is absent, calls
raise.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

OK = 0
ERR = {
    -1: "NEKGPU_ERR_ARG", -2: "NEKGPU_ERR_MESH", -3: "NEKGPU_ERR_CUDA", -4: "NEKGPU_ERR_NOMEM",
    -5: "NEKGPU_ERR_STATE", -6: "NEKGPU_ERR_BLOWUP", -7: "NEKGPU_ERR_TIMEOUT",
    -8: "NEKGPU_ERR_UNSUPPORTED", -9: "NEKGPU_ERR_TOO_LARGE",
}
PLAIN, FUSED64, MIXED, MIXED_NAIVE = 0, 1, 2, 3
FORMS = {"plain": PLAIN, "fused64": FUSED64, "mixed": MIXED, "mixed_naive": MIXED_NAIVE}
BC_PEC, BC_PERIODIC = 0, 1

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
lp = C.POINTER(C.c_longlong)


class NekgpuMesh(C.Structure):
    _fields_ = [
        ("nx1", C.c_int), ("nelt", C.c_int),
        ("dxm1", dp), ("w3mn", dp),
        ("rxmn", dp), ("rymn", dp), ("rzmn", dp), ("sxmn", dp), ("symn", dp), ("szmn", dp),
        ("txmn", dp), ("tymn", dp), ("tzmn", dp),
        ("bmn", dp), ("xmn", dp), ("ymn", dp), ("zmn", dp),
        ("unxm", dp), ("unym", dp), ("unzm", dp), ("aream", dp),
        ("cemface", ip), ("glo_face", lp), ("cempec", ip), ("ncempec", C.c_int),
        ("Z_0", dp), ("Z_1", dp), ("Y_0", dp), ("Y_1", dp),
        ("ebm1", dp), ("hbm1", dp), ("C0", C.c_double),
        ("pmlsigma", dp), ("pmlptr", ip), ("npml", C.c_int),
        ("permittivity", dp), ("permeability", dp),
    ]


class NekgpuBox(C.Structure):
    _fields_ = [
        ("N", C.c_int), ("nelx", C.c_int), ("nely", C.c_int), ("nelz", C.c_int),
        ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("bc", C.c_int * 3),
        ("permittivity", dp), ("permeability", dp), ("C0", C.c_double),
        ("pml_thick", C.c_int), ("pml_order", C.c_double), ("pml_referr", C.c_double),
    ]


class NekgpuError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: {ERR.get(status, status)} ({msg})")
        self.status = status


# (name, restype, argtypes) of every exported entry point
SIGNATURES = [
    ("nekgpu_error_string", C.c_char_p, [C.c_int]),
    ("nekgpu_version", C.c_int, []),
    ("nekgpu_device_check", C.c_int, [C.c_int]),
    ("nekgpu_init", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(NekgpuMesh), C.c_int]),
    ("nekgpu_init_box", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(NekgpuBox), C.c_int]),
    ("nekgpu_init2d", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(NekgpuMesh), C.c_int]),
    ("nekgpu_finalize", C.c_int, [C.c_void_p]),
    ("nekgpu_box_export_d", C.c_int, [C.POINTER(NekgpuBox), C.c_char_p, dp, C.POINTER(C.c_long)]),
    ("nekgpu_box_export_i", C.c_int, [C.POINTER(NekgpuBox), C.c_char_p, lp, C.POINTER(C.c_long)]),
    ("nekgpu_sizes", C.c_int, [C.c_void_p, C.POINTER(C.c_long), C.POINTER(C.c_long), ip, ip]),
    ("nekgpu_get_array", C.c_int, [C.c_void_p, C.c_char_p, dp]),
    ("nekgpu_volume", C.c_double, [C.c_void_p]),
    ("nekgpu_set_source_kind", C.c_int, [C.c_void_p, C.c_int]),
    ("nekgpu_set_source", C.c_int, [C.c_void_p, C.c_int, dp, C.c_double, C.c_double, C.c_double, C.c_double]),
    ("nekgpu_set_incident", C.c_int, [C.c_void_p, ip, C.c_long, dp, dp, C.c_double]),
    ("nekgpu_set_array", C.c_int, [C.c_void_p, C.c_char_p, dp]),
    ("nekgpu_set_graphene", C.c_int, [C.c_void_p, dp, ip, C.c_long, dp]),
    ("nekgpu_set_graphene_current", C.c_int, [C.c_void_p, dp, C.c_long]),
    ("nekgpu_get_graphene_current", C.c_int, [C.c_void_p, dp, C.c_long]),
    ("nekgpu_set_dealias", C.c_int, [C.c_void_p, C.c_int, dp, dp, dp, dp]),
    ("nekgpu_set_dispersive", C.c_int, [C.c_void_p, C.c_int, dp, C.c_long, ip, C.c_long]),
    ("nekgpu_set_current", C.c_int, [C.c_void_p, C.c_int, dp, C.c_long]),
    ("nekgpu_get_current", C.c_int, [C.c_void_p, C.c_int, dp, C.c_long]),
    ("nekgpu_set_state", C.c_int, [C.c_void_p, dp, dp, C.c_long]),
    ("nekgpu_get_state", C.c_int, [C.c_void_p, dp, dp, C.c_long]),
    ("nekgpu_set_rk_register", C.c_int, [C.c_void_p, dp, dp, C.c_long]),
    ("nekgpu_get_rk_register", C.c_int, [C.c_void_p, dp, dp, C.c_long]),
    ("nekgpu_register_host", C.c_int, [C.c_void_p, C.c_void_p, C.c_long]),
    ("nekgpu_unregister_host", C.c_int, [C.c_void_p, C.c_void_p]),
    ("nekgpu_stage", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double]),
    ("nekgpu_step", C.c_int, [C.c_void_p, C.c_int, dp, C.c_double]),
    ("nekgpu_op_rk_host", C.c_int, [C.c_void_p, dp, dp, C.c_long, C.c_double, C.c_double]),
    ("nekgpu_cem_maxwell", C.c_int, [C.c_void_p]),
    ("nekgpu_restrict_to_face", C.c_int, [C.c_void_p]),
    ("nekgpu_flux3d", C.c_int, [C.c_void_p]),
    ("nekgpu_add_flux_to_res", C.c_int, [C.c_void_p]),
    ("nekgpu_usersrc", C.c_int, [C.c_void_p, C.c_double]),
    ("nekgpu_invqmass", C.c_int, [C.c_void_p]),
    ("nekgpu_rk_maxwell_ab", C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    ("nekgpu_gs_op_fields", C.c_int, [C.c_void_p, dp, C.c_int]),
    ("nekgpu_get_work", C.c_int, [C.c_void_p, C.c_char_p, dp]),
    ("nekgpu_norms", C.c_int, [C.c_void_p, dp, dp, C.c_long, dp, dp]),
    ("nekgpu_norms_noalloc", C.c_int, [C.c_void_p, C.c_void_p, dp, dp]),
    ("nekgpu_energy", C.c_int, [C.c_void_p, dp]),
    ("nekgpu_check_blowup", C.c_int, [C.c_void_p]),
    ("nekgpu_selftest_wait", C.c_int, [C.c_void_p, C.c_int]),
    ("nekgpu_selftest_pair_join", C.c_int, [C.c_void_p, C.c_void_p, dp, C.c_long]),
    ("nekgpu_adjoint_gradient", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, dp, dp, dp,
                                         C.c_int, dp, dp]),
    ("nekgpu_adjoint_init", C.c_int, [C.c_void_p, dp, C.c_int]),
    ("nekgpu_adjoint_host_snapshots", C.c_int, [C.c_void_p, C.c_int]),
    ("nekgpu_adjoint_recompute_mixed", C.c_int, [C.c_void_p, C.c_int]),
    ("nekgpu_adjoint_run", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, dp, dp]),
    ("nekgpu_write_vtk", C.c_int, [C.c_void_p, C.c_char_p, dp, dp, C.c_long]),
    ("nekgpu_checkpoint_save", C.c_int, [C.c_void_p, C.c_char_p, C.c_double, C.c_long]),
    ("nekgpu_checkpoint_load", C.c_int, [C.c_void_p, C.c_char_p, dp, C.POINTER(C.c_long)]),
    ("nekgpu_time_steps", C.c_int, [C.c_void_p, C.c_int, dp, C.c_double, dp]),
    ("nekgpu_last_launches", C.c_long, [C.c_void_p]),
    ("nekgpu_device_bytes", C.c_long, [C.c_void_p]),
    ("nekgpu_sync", C.c_int, [C.c_void_p]),
]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the product library (building it in place if asked)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if build_if_missing:
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"CUDA library not built: {path}")
        L = C.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str):
    if status != OK:
        msg = load().nekgpu_error_string(status).decode()
        raise NekgpuError(status, where, msg)
