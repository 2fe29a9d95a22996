"""ctypes binding of the C ABI declared in include/exafac_gb300.h.

Loading the library needs no GPU; calling anything that launches work does.
There is no CPU fallback: on a machine without the built library every entry
point raises."""
from __future__ import annotations

import ctypes
import os

from . import _build

MAX_MODES = 8
OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "device-side check failed", 4: "device wait timed out",
          5: "unsupported", 6: "workspace too small"}
SAMPLER = {"cp_arls_lev": 0, "sts_cp": 1}
PRECISION = {"fp64": 0, "tf32": 1, "bf16": 2}
PREPROCESSING = {"none": 0, "None": 0, "log_count": 1, "ones": 2}
DTYPE = {"float32": 0, "float64": 1}


class ExafacError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn}: {ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class AlsConfig(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int32), ("R", ctypes.c_int32), ("dims", ctypes.c_int64 * MAX_MODES),
                ("nnz", ctypes.c_int64), ("J_max", ctypes.c_int64), ("sampler", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("preprocessing", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Factors(ctypes.Structure):
    _fields_ = [("U", ctypes.c_void_p * MAX_MODES), ("sigma", ctypes.c_void_p)]


class StepInfo(ctypes.Structure):
    _fields_ = [("unique_samples", ctypes.c_int64), ("hits", ctypes.c_int64), ("touched_rows", ctypes.c_int64),
                ("hits_total", ctypes.c_int64), ("device_status", ctypes.c_int32), ("pad", ctypes.c_int32)]


# name -> (restype, argtypes)
_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_SZ = ctypes.c_size_t
SIGNATURES = {
    "exafac_last_error": (ctypes.c_char_p, []),
    "exafac_abi_version": (ctypes.c_int, []),
    "exafac_kernel_launches": (ctypes.c_longlong, []),
    "exafac_tree_node_count": (_I64, [_I64, _I32]),
    "exafac_tree_build": (ctypes.c_int, [_I64, _I32, _I32, _P, _P, _P]),
    "exafac_tree_sample": (ctypes.c_int, [_I64, _I32, _I32, _P, _P, _I64, _P, _P, _P, _P, _I64, _P]),
    "exafac_quad_forms_f32": (ctypes.c_int, [_I32, _I64, _P, _P, _P, _P, _I32, _P]),
    "exafac_tree_build_f32": (ctypes.c_int, [_I64, _I32, _I32, _P, _P, _P]),
    "exafac_syev": (ctypes.c_int, [_I32, _P, _P, _P, _P, _SZ, _P]),
    "exafac_pinv_square": (ctypes.c_int, [_I32, _P, _P, ctypes.c_double, _P, _SZ, _P]),
    "exafac_dense_workspace_bytes": (_SZ, [_I32]),
    "exafac_pinv_square_static": (ctypes.c_int, [_I32, _P, _P, ctypes.c_double, _P]),
    "exafac_als_workspace_size": (ctypes.c_int, [ctypes.POINTER(AlsConfig), ctypes.POINTER(_SZ), ctypes.POINTER(_SZ)]),
    "exafac_als_create": (ctypes.c_int, [ctypes.POINTER(AlsConfig), _P, _SZ, ctypes.POINTER(_P)]),
    "exafac_als_destroy": (ctypes.c_int, [_P]),
    "exafac_als_init": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(Factors), _P, _SZ, ctypes.POINTER(ctypes.c_double),
                                       _P]),
    "exafac_als_draw": (ctypes.c_int, [_P, _I32, _I64, _P, _P, _P, _P, _P]),
    "exafac_als_step": (ctypes.c_int, [_P, _I32, _I64, _P, _P, _P]),
    "exafac_als_exact_step": (ctypes.c_int, [_P, _I32, _P]),
    "exafac_als_sweeps": (ctypes.c_int, [_P, _I64, _I32, _P, _P]),
    "exafac_als_sampled_mttkrp": (ctypes.c_int, [_P, _I32, _I64, _P, _P, _P, _P]),
    "exafac_als_fit": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), _P]),
    "exafac_als_estimated_fit": (ctypes.c_int, [_P, _I64, _P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(_I64), _P]),
    "exafac_als_set_seed": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "exafac_als_enable_timing": (ctypes.c_int, [_P, _I32]),
    "exafac_als_region_times": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double)]),
    "exafac_als_step_info": (ctypes.c_int, [_P, ctypes.POINTER(StepInfo), _P]),
    "exafac_als_set_wait_limit": (ctypes.c_int, [_P, ctypes.c_uint32, _I64]),
    "exafac_als_last_dedup": (ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P),
                                             ctypes.POINTER(_P)]),
    "exafac_cp_sampled_model": (ctypes.c_int, [_I32, _I32, _P, _I64, _P, _P, _P, _I32, _P, _P]),
    "exafac_cp_sampled_adjoint": (ctypes.c_int, [_I32, _I32, _P, _I64, _P, _P, _P, _P, _I32, _P, _P]),
    "exafac_gcp_sample_entries": (ctypes.c_int, [_I32, _P, _I64, _P, _P, _I64, _I64, ctypes.c_uint64,
                                                 ctypes.c_uint64, _P, _P, _P, _I32, _P]),
    "exafac_adam_step": (ctypes.c_int, [_I32, _P, _P, _P, _P, _P, _I32, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, _I64, _I32, ctypes.c_double, _P]),
}

_lib = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads libexafac_gb300.so (building it first if needed and allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libexafac_gb300.so is not built ({path}); run __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(fn: str, code: int):
    if code != OK:
        msg = load().exafac_last_error()
        raise ExafacError(fn, code, msg.decode() if msg else "")


def call(name: str, *args):
    lib = load()
    rc = getattr(lib, name)(*args)
    check(name, rc)
    return rc
