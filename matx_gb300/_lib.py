"""ctypes binding of libgbfir.so (include/gbfir.h).

The library is loaded from this package's directory only (it is built in-tree by
``matx_gb300.build``).  There is no fallback: if the shared object is missing or
cannot be loaded, every operator raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbfir.so")

GBFIR_F32, GBFIR_C64, GBFIR_F64, GBFIR_C128 = 0, 1, 2, 3
PREC = {"fp32": 0, "bf16": 1, "fp16": 2, "bf16x3": 3}

STATUS = {
    0: "success", 1: "invalid parameter", 2: "invalid dimension", 3: "invalid size",
    4: "invalid type", 5: "not supported", 6: "CUDA error", 7: "null pointer",
    8: "misaligned pointer", 9: "workspace missing or too small", 10: "device wait timed out",
}


class GbfirError(RuntimeError):
    """Raised for a non-zero gbfir_status; ``code`` mirrors matxError_t classes."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class Buf(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("batch", ctypes.c_int64), ("len", ctypes.c_int64),
                ("batch_stride", ctypes.c_int64), ("dtype", ctypes.c_int32)]


class Buf2d(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("batch", ctypes.c_int64), ("rows", ctypes.c_int64),
                ("cols", ctypes.c_int64), ("batch_stride", ctypes.c_int64), ("row_stride", ctypes.c_int64),
                ("dtype", ctypes.c_int32)]


class RaggedDesc(ctypes.Structure):
    _fields_ = [("inp", ctypes.c_void_p), ("out", ctypes.c_void_p), ("h", ctypes.c_void_p),
                ("in_len", ctypes.c_int64), ("out_len", ctypes.c_int64), ("h_len", ctypes.c_int32),
                ("up", ctypes.c_int32), ("down", ctypes.c_int32), ("pad_", ctypes.c_int32)]


class RaggedPlanInfo(ctypes.Structure):
    _fields_ = [("num_tiles", ctypes.c_int64), ("shared_bytes", ctypes.c_int64), ("table_bytes", ctypes.c_int64),
                ("window_elems", ctypes.c_int64), ("buffers", ctypes.c_int64), ("precision", ctypes.c_int64)]


# (name, restype, argtypes) of every symbol include/gbfir.h declares
_B = Buf
_i32, _i64, _p, _sz = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_size_t
SIGNATURES = [
    ("gbfir_conv1d", ctypes.c_int, [_B, _B, _B, _i32, _i32, _i32, _p]),
    ("gbfir_conv1d_axis", ctypes.c_int, [_B, _B, _B, _i64, _i64, _i64, _i32, _i32, _i32, _p]),
    ("gbfir_conv1d_fft", ctypes.c_int, [_B, _B, _B, _i32, _i32, _p]),
    ("gbfir_conv2d", ctypes.c_int, [Buf2d, Buf2d, Buf2d, _i32, _p]),
    ("gbfir_upsample", ctypes.c_int, [_B, _B, _i64, _p]),
    ("gbfir_downsample", ctypes.c_int, [_B, _B, _i64, _p]),
    ("gbfir_upfirdn", ctypes.c_int, [_B, _B, _B, _i64, _i64, _i32, _i32, _p]),
    ("gbfir_filter_workspace_size", _sz, [_i64, _i64, _i32]),
    ("gbfir_filter", ctypes.c_int, [_B, _B, _p, _i32, _p, _i32, _i32, _p, _sz, _p]),
    ("gbfir_resample_poly", ctypes.c_int, [_B, _B, _B, _i64, _i64, _i32, _p]),
    ("gbfir_channelize_poly", ctypes.c_int, [_B, _B, _B, _i64, _i64, _i32, _p]),
    ("gbfir_resample_poly_bwd_workspace_size", _sz, [_i64, _i64, _i64, _i64, _i64]),
    ("gbfir_resample_poly_bwd", ctypes.c_int, [_B, _B, _B, _B, _B, _i64, _i64, _p, _sz, _p]),
    ("gbfir_resample_poly_bwd_prec", ctypes.c_int, [_B, _B, _B, _B, _B, _i64, _i64, _i32, _p, _sz, _p]),
    ("gbfir_resample_poly_bwd_noalloc", ctypes.c_int, [_B, _B, _B, _B, _B, _i64, _i64, _p]),
    ("gbfir_conv1d_bwd_workspace_size", _sz, [_i64, _i64, _i64, _i32]),
    ("gbfir_conv1d_bwd", ctypes.c_int, [_B, _B, _B, _B, _B, _i32, _p, _sz, _p]),
    ("gbfir_conv1d_bwd_prec", ctypes.c_int, [_B, _B, _B, _B, _B, _i32, _i32, _p, _sz, _p]),
    ("gbfir_ragged_workspace_size", _sz, [_i64, _i64]),
    ("gbfir_ragged_plan", _i64, [_p, _i64, _p, _p]),
    ("gbfir_ragged_plan_prec", _i64, [_p, _i64, _i32, _p, _p]),
    ("gbfir_ragged_tile_register", ctypes.c_int, [_i64, _i64, _i64, _i32, _i32, _i32]),
    ("gbfir_ragged_tile_clear", ctypes.c_int, []),
    ("gbfir_ragged_resample", ctypes.c_int, [_p, _i64, _p, _p, _i32, _p, _sz, _p]),
    ("gbfir_set_resample_tile", ctypes.c_int, [_i32, _i32, _i32, _i32]),
    ("gbfir_resample_tile_register", ctypes.c_int, [_i64, _i64, _i64, _i32, _i32, _i32, _i32]),
    ("gbfir_resample_tile_clear", ctypes.c_int, []),
    ("gbfir_tc_status", ctypes.c_int, []),
    ("gbfir_launch_count", ctypes.c_uint64, []),
    ("gbfir_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("gbfir_last_error", ctypes.c_char_p, []),
    ("gbfir_version", ctypes.c_int, []),
]

_LIB = None


def load():
    """Load libgbfir.so (raises if it was not built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"matx_gb300: {LIB_PATH} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(rc: int):
    if rc != 0:
        msg = load().gbfir_last_error().decode(errors="replace")
        raise GbfirError(rc, msg)
