"""ctypes declarations of the C ABI in include/bkma_gb300.h.

The library is loaded from the package root (in-tree build). There is no
fallback: if libbkma_gb300.so is missing, load() raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB

BKMA_OK = 0
BKMA_ERR_INVALID_ARG = 1
STATUS_NAMES = {0: "BKMA_OK", 1: "BKMA_ERR_INVALID_ARG", 2: "BKMA_ERR_UNSUPPORTED",
                3: "BKMA_ERR_CUDA", 4: "BKMA_ERR_TIMEOUT", 5: "BKMA_ERR_NO_DEVICE",
                6: "BKMA_ERR_HOST"}

BKMA_F32, BKMA_F64, BKMA_BF16 = 0, 1, 2
BKMA_ADV_AUTO, BKMA_ADV_STAGED, BKMA_ADV_PLAIN = 0, 1, 2
BKMA_W_REFERENCE, BKMA_W_LAGRANGE, BKMA_W_TABLE = 0, 1, 2
BKMA_CONV_TORCH, BKMA_CONV_REFERENCE = 0, 1
BKMA_CONV_AUTO, BKMA_CONV_TENSOR, BKMA_CONV_PLAIN = 0, 1, 2


class AdvDesc(C.Structure):
    _fields_ = [("n0", C.c_int64), ("n1", C.c_int64), ("n2", C.c_int64),
                ("i0_offset", C.c_int64), ("i0_count", C.c_int64),
                ("dtype", C.c_int32), ("degree", C.c_int32), ("weights", C.c_int32),
                ("impl", C.c_int32), ("inplace", C.c_int32), ("reserved", C.c_int32),
                ("dt", C.c_double), ("minX", C.c_double), ("maxX", C.c_double),
                ("minVx", C.c_double), ("maxVx", C.c_double),
                ("velocity", C.POINTER(C.c_double))]


class AdvPlanInfo(C.Structure):
    _fields_ = [("lines", C.c_int64), ("exception_lines", C.c_int64),
                ("tile_cols", C.c_int32), ("tile_slabs", C.c_int32), ("threads", C.c_int32),
                ("smem_bytes", C.c_int32), ("npts", C.c_int32), ("autotuned", C.c_int32),
                ("tiles", C.c_int64), ("path", C.c_int32), ("reserved", C.c_int32)]


class AdvField(C.Structure):
    _fields_ = [("data", C.c_void_p), ("n0", C.c_int64), ("n1", C.c_int64),
                ("n2", C.c_int64), ("degree", C.c_int32), ("weights", C.c_int32),
                ("dt", C.c_double), ("minX", C.c_double), ("maxX", C.c_double),
                ("minVx", C.c_double), ("maxVx", C.c_double),
                ("velocity", C.POINTER(C.c_double))]


class ConvDesc(C.Structure):
    _fields_ = [("batch", C.c_int64), ("cin", C.c_int64), ("cout", C.c_int64),
                ("length", C.c_int64), ("ksize", C.c_int64), ("n2", C.c_int64),
                ("dtype", C.c_int32), ("semantics", C.c_int32), ("impl", C.c_int32),
                ("inplace", C.c_int32)]


_vp = C.c_void_p
_st = C.c_int
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)

# name -> (restype, argtypes); every function declared in include/bkma_gb300.h
SIGNATURES = {
    "bkma_abi_version": (C.c_int32, []),
    "bkma_last_error": (C.c_char_p, []),
    "bkma_impl_from_name": (_st, [C.c_char_p, _i32p, _i32p]),
    "bkma_adv_plan_create": (_st, [C.POINTER(AdvDesc), C.POINTER(_vp)]),
    "bkma_adv_plan_info_get": (_st, [_vp, C.POINTER(AdvPlanInfo)]),
    "bkma_adv_plan_autotune": (_st, [_vp, _vp, _vp]),
    "bkma_adv_plan_set_tile": (_st, [_vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "bkma_adv_plan_set_fusion": (_st, [_vp, C.c_int32]),
    "bkma_adv_plan_set_fused_state": (_st, [_vp, C.c_int32]),
    "bkma_adv_plan_set_weights": (_st, [_vp, _vp, C.c_int32]),
    "bkma_adv_plan_line_table": (_st, [_vp, _i32p, _dp]),
    "bkma_adv_plan_status": (_st, [_vp, _vp]),
    "bkma_adv_plan_set_wait_limit": (_st, [_vp, C.c_uint32]),
    "bkma_adv_plan_destroy": (_st, [_vp]),
    "bkma_adv_step": (_st, [_vp, _vp, _vp, C.c_int32, _vp]),
    "bkma_adv_run_host": (_st, [_vp, _vp, C.c_int32, _vp]),
    "bkma_adv_fill": (_st, [_vp, _vp, C.c_int32, C.c_double, C.c_uint64, _vp]),
    "bkma_adv_error_norms": (_st, [_vp, _vp, C.c_int32, _vp, C.c_int32, _dp, _vp]),
    "bkma_adv_validate": (_st, [_vp, _vp, C.c_int64, _dp, _dp, _vp]),
    "bkma_adv_batch_create": (_st, [C.POINTER(AdvField), C.c_int32, C.c_int32, C.POINTER(_vp)]),
    "bkma_adv_batch_step": (_st, [_vp, C.c_int32, _vp]),
    "bkma_adv_batch_info": (_st, [_vp, _i64p, _i32p]),
    "bkma_adv_batch_autotune": (_st, [_vp, _vp]),
    "bkma_adv_batch_tiles": (_st, [_vp, _i32p, _i32p, _i64p, _i32p, _i64p]),
    "bkma_adv_batch_destroy": (_st, [_vp]),
    "bkma_conv_plan_create": (_st, [C.POINTER(ConvDesc), C.POINTER(_vp)]),
    "bkma_conv_plan_scratch_bytes": (_st, [_vp, _i64p]),
    "bkma_conv_run": (_st, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "bkma_conv_plan_status": (_st, [_vp, _vp]),
    "bkma_conv_plan_set_wait_limit": (_st, [_vp, C.c_uint32]),
    "bkma_conv_plan_destroy": (_st, [_vp]),
    "bkma_fill": (_st, [_vp, C.c_int64, C.c_int32, C.c_double, _vp]),
    "bkma_conv_check": (_st, [_vp, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int64, _dp,
                              _i32p, _vp]),
    "bkma_conv1d_bf16_inplace_noalloc": (_st, [_vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64,
                                               C.c_int64, _vp]),
    "bkma_conv1d_noalloc_status": (_st, [_vp]),
    "bkma_mlp_create": (_st, [C.c_uint64, C.POINTER(_vp)]),
    "bkma_mlp_create_stencil": (_st, [C.c_uint64, C.c_int32, C.POINTER(_vp)]),
    "bkma_mlp_info": (_st, [_vp, _i32p, _i32p]),
    "bkma_mlp_samples_grid": (_st, [C.c_int64, C.c_uint64, C.c_int64, C.c_int64, C.c_int32,
                                    C.c_int32, _vp, _vp, _vp, _vp]),
    "bkma_mlp_params": (_st, [_vp, _vp, C.c_int32]),
    "bkma_mlp_samples": (_st, [C.c_int64, C.c_uint64, C.c_int64, _vp, _vp, _vp, _vp]),
    "bkma_mlp_grad": (_st, [_vp, _vp, _vp, _vp, C.c_int64, _vp, _dp, _vp]),
    "bkma_mlp_train": (_st, [_vp, _vp, _vp, _vp, C.c_int64, C.c_int32, C.c_int32, C.c_float,
                             C.c_uint64, _dp, _vp]),
    "bkma_mlp_infer": (_st, [_vp, _vp, C.c_int64, _vp, _vp]),
    "bkma_mlp_destroy": (_st, [_vp]),
}

_LIB = None


class BkmaError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def load(path: str | None = None):
    """Load libbkma_gb300.so. Raises if it has not been built: the CUDA path is
    the only path."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with bkma_gb300.build.build_library() "
                           "(there is no CPU fallback)")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def check(status: int):
    if status != BKMA_OK:
        raise BkmaError(status, load().bkma_last_error().decode(errors="replace"))
