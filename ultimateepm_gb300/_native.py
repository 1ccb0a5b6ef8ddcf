"""ctypes binding of the C ABI in include/uepm_gb300.h (libuepm_gb300.so, built in-tree).

There is no fallback: if the native library is missing this module raises on first use, so nothing
ever silently computes band structures on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libuepm_gb300.so")

UEPM_OK = 0
UEPM_ERR_INVALID = -1
UEPM_ERR_RUNTIME = -2
UEPM_ERR_OUT_OF_RANGE = -3
UEPM_ERR_CUDA = -4
UEPM_ERR_NOMEM = -5
UEPM_ERR_NOT_CONVERGED = -6
UEPM_K_OK = 0
UEPM_K_NOCONVERGE = 1  # an iteration cap ended an iterative kernel before it converged
UEPM_K_NONFINITE = 2  # NaN / Inf reached H(k) or the reduction

UEPM_NONLOCAL = 1
UEPM_SOC = 2
UEPM_WANT_VALUES = 1
UEPM_WANT_VECTORS = 2
UEPM_WANT_GRADIENT = 4
UEPM_PREC_FP64 = 0
UEPM_PREC_MIXED = 1

# Symbols include/uepm_gb300.h declares; tests check every one is exported.
EXPORTED = [
    "uepm_version", "uepm_last_error", "uepm_material_size", "uepm_generate_basis", "uepm_generate_path",
    "uepm_materials_load", "uepm_ctx_create", "uepm_ctx_destroy", "uepm_ctx_set_precision", "uepm_ctx_order",
    "uepm_ctx_set_workspace_limit", "uepm_solve", "uepm_solve_device", "uepm_assemble_device",
    "uepm_adjust_values", "uepm_kernel_launches", "uepm_ctx_set_profiling", "uepm_ctx_read_profile",
    "uepm_kernel_name", "uepm_measure_peak", "uepm_ctx_force_complex", "uepm_assemble_device_noalloc",
    "uepm_ctx_get_tuning", "uepm_ctx_set_tuning", "uepm_ctx_autotune", "uepm_batch_create", "uepm_batch_destroy",
    "uepm_batch_add", "uepm_batch_clear", "uepm_batch_set_graph", "uepm_batch_run", "uepm_batch_kernels_per_run",
    "uepm_server_create", "uepm_server_destroy", "uepm_server_submit", "uepm_server_wait", "uepm_server_stats",
    "uepm_server_reset_stats", "uepm_star_expand_device", "uepm_star_operations", "uepm_dielectric_sums_device",
    "uepm_pivot_reciprocal_device", "uepm_ds_special_device",
]
UEPM_SERVE_VELOCITY = 1
NOALLOC_SCRATCH_BYTES = 16 << 20
KERNEL_KINDS = 10


class UepmMaterial(C.Structure):
    """struct uepm_material (include/uepm_gb300.h)."""

    _fields_ = [
        ("lattice_constant", C.c_double),
        ("V3S", C.c_double), ("V4S", C.c_double), ("V8S", C.c_double), ("V11S", C.c_double),
        ("V3A", C.c_double), ("V4A", C.c_double), ("V8A", C.c_double), ("V11A", C.c_double),
        ("nl_well", C.c_int32), ("has_nonlocal", C.c_int32),
        ("alpha0_cation", C.c_double), ("beta0_cation", C.c_double), ("A2_cation", C.c_double),
        ("alpha0_anion", C.c_double), ("beta0_anion", C.c_double), ("A2_anion", C.c_double),
        ("R0_cation", C.c_double), ("R2_cation", C.c_double), ("R0_anion", C.c_double), ("R2_anion", C.c_double),
        ("period_anion", C.c_uint32), ("period_cation", C.c_uint32),
        ("has_soc", C.c_int32), ("_pad", C.c_int32),
        ("radial_extent_anion", C.c_double), ("radial_extent_cation", C.c_double),
        ("alpha_soc", C.c_double), ("mu_soc", C.c_double),
    ]


class UepmTuning(C.Structure):
    """struct uepm_tuning (include/uepm_gb300.h); 0 in a field means automatic."""

    _fields_ = [("reduction", C.c_int32), ("ctas_per_sm", C.c_int32), ("vector_lanes", C.c_int32),
                ("chunk", C.c_int32), ("cluster", C.c_int32), ("max_iter", C.c_int32), ("tensor_cores", C.c_int32),
                ("streams", C.c_int32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class UepmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return LIB_PATH


def load():
    """Load libuepm_gb300.so (raises if it was not built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"ultimateepm_gb300 native library not found at {LIB_PATH}; build it with "
                "`python -m ultimateepm_gb300.build` (there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        vp, dp, ip, u32p = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint32)
        mp = C.POINTER(UepmMaterial)
        sig = {
            "uepm_version": (C.c_int, []),
            "uepm_last_error": (C.c_char_p, []),
            "uepm_material_size": (C.c_int, []),
            "uepm_generate_basis": (C.c_int, [C.c_uint, ip, C.c_int]),
            "uepm_generate_path": (C.c_int, [C.c_char_p, C.c_uint, dp, C.c_int, u32p]),
            "uepm_materials_load": (C.c_int, [C.c_char_p, mp, C.c_char_p, C.c_int, C.c_int]),
            "uepm_ctx_create": (C.c_int, [mp, ip, C.c_int, C.c_uint32, C.POINTER(vp)]),
            "uepm_ctx_destroy": (C.c_int, [vp]),
            "uepm_ctx_set_precision": (C.c_int, [vp, C.c_int]),
            "uepm_ctx_order": (C.c_int, [vp]),
            "uepm_ctx_set_workspace_limit": (C.c_int, [vp, C.c_size_t]),
            "uepm_solve": (C.c_int, [vp, dp, C.c_size_t, C.c_int, C.c_uint32, dp, dp, dp, ip]),
            "uepm_solve_device": (C.c_int, [vp, vp, C.c_size_t, C.c_int, C.c_uint32, vp, vp, vp, vp, vp]),
            "uepm_assemble_device": (C.c_int, [vp, vp, C.c_size_t, vp, vp]),
            "uepm_adjust_values": (C.c_int, [dp, C.c_size_t, C.c_int, C.c_int, C.c_int, dp, ip]),
            "uepm_kernel_launches": (C.c_uint64, []),
            "uepm_ctx_set_profiling": (C.c_int, [vp, C.c_int]),
            "uepm_ctx_read_profile": (C.c_int, [vp, dp, C.POINTER(C.c_uint64), C.c_int]),
            "uepm_kernel_name": (C.c_char_p, [C.c_int]),
            "uepm_measure_peak": (C.c_int, [C.c_int, dp]),
            "uepm_ctx_force_complex": (C.c_int, [vp, C.c_int]),
            "uepm_assemble_device_noalloc": (C.c_int, [vp, vp, C.c_size_t, vp, vp]),
            "uepm_ctx_get_tuning": (C.c_int, [vp, C.POINTER(UepmTuning)]),
            "uepm_ctx_set_tuning": (C.c_int, [vp, C.POINTER(UepmTuning)]),
            "uepm_ctx_autotune": (C.c_int, [vp, C.c_int, C.c_uint32, C.c_size_t, vp]),
            "uepm_batch_create": (C.c_int, [C.POINTER(vp)]),
            "uepm_batch_destroy": (None, [vp]),
            "uepm_batch_add": (C.c_int, [vp, vp, vp, C.c_size_t, C.c_int, C.c_uint32, vp, vp, vp, vp]),
            "uepm_batch_clear": (C.c_int, [vp]),
            "uepm_batch_set_graph": (C.c_int, [vp, C.c_int]),
            "uepm_batch_run": (C.c_int, [vp, vp]),
            "uepm_batch_kernels_per_run": (C.c_uint64, [vp]),
            "uepm_server_create": (C.c_int, [C.POINTER(vp), C.c_int, C.c_size_t, C.c_int, C.c_size_t, C.c_int,
                                             C.POINTER(vp)]),
            "uepm_server_destroy": (C.c_int, [vp]),
            "uepm_server_submit": (C.c_int64, [vp, C.c_int, dp, C.c_size_t, C.c_int, C.c_uint32, C.c_double, dp, dp,
                                               ip]),
            "uepm_server_wait": (C.c_int, [vp, C.c_int64, C.c_double]),
            "uepm_server_stats": (C.c_int, [vp, dp, dp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), dp]),
            "uepm_server_reset_stats": (C.c_int, [vp]),
            "uepm_star_expand_device": (C.c_int, [vp, vp, vp, vp, C.c_size_t, C.c_int, vp, vp, vp]),
            "uepm_star_operations": (C.c_int, [dp, dp, C.c_size_t, C.POINTER(C.c_uint16), ip]),
            "uepm_pivot_reciprocal_device": (C.c_int, [vp, C.c_double, C.c_size_t, vp, vp]),
            "uepm_ds_special_device": (C.c_int, [C.c_int, vp, C.c_size_t, vp, vp]),
            "uepm_dielectric_sums_device": (C.c_int, [vp, vp, vp, vp, C.c_size_t, C.c_int, C.c_int, C.c_int, vp, C.c_int,
                                                      C.c_double, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if L.uepm_material_size() != C.sizeof(UepmMaterial):
            raise RuntimeError("uepm_material layout mismatch between header and binding")
        _lib = L
        return L


def last_error() -> str:
    return load().uepm_last_error().decode(errors="replace")


def check(code: int) -> int:
    if code < 0:
        raise UepmError(code, last_error())
    return code
