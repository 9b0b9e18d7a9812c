"""ctypes binding of ``libstride_gb300.so`` (declarations: include/stride_gb300.h).

Loading fails loudly when the library has not been built: the decoder has no
CPU fallback.
"""
from __future__ import annotations

import ctypes
import threading

from . import _build

STRIDE_OK = 0
STRIDE_ERR_ARG = -1
STRIDE_ERR_MAGIC = -2
STRIDE_ERR_VERSION = -3
STRIDE_ERR_TRUNCATED = -4
STRIDE_ERR_OFFSET = -5
STRIDE_ERR_CORRUPT = -6
STRIDE_ERR_UNSUPPORTED = -7
STRIDE_ERR_CUDA = -8
STRIDE_ERR_TIMEOUT = -9
STRIDE_ERR_NOMEM = -10
STRIDE_ERR_BUSY = -11

# Errors about the bytes themselves surface as ValueError, like the
# reference's "bad magic" / "expected v5" checks (utils/paradelta_v5_cuda.py:520-523).
FORMAT_ERRORS = {STRIDE_ERR_ARG, STRIDE_ERR_MAGIC, STRIDE_ERR_VERSION, STRIDE_ERR_TRUNCATED,
                 STRIDE_ERR_OFFSET, STRIDE_ERR_CORRUPT, STRIDE_ERR_UNSUPPORTED}


class StrideFormatError(ValueError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class StrideDeviceError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class StrideInfo(ctypes.Structure):
    _fields_ = [("n_meshlets", ctypes.c_uint32), ("g_bits", ctypes.c_uint32 * 3),
                ("n_v", ctypes.c_uint64), ("n_t", ctypes.c_uint64), ("nbytes", ctypes.c_uint64),
                ("center", ctypes.c_float * 3), ("scale", ctypes.c_float),
                ("pred_n", ctypes.c_int32 * 9), ("pred_k", ctypes.c_int32 * 3), ("kernels", ctypes.c_uint32),
                ("g_min", ctypes.c_float * 3), ("g_range", ctypes.c_float * 3),
                ("shared_bytes", ctypes.c_uint32), ("persistent_blocks", ctypes.c_uint32)]


class LaunchCfg(ctypes.Structure):
    _fields_ = [("warps_per_cta", ctypes.c_int32), ("persistent", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("stage_bytes", ctypes.c_uint32),
                ("code_bytes", ctypes.c_uint32)]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class ServerOpts(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_batch", ctypes.c_uint32),
                ("n_streams", ctypes.c_uint32), ("max_queue", ctypes.c_uint32),
                ("copy_to_host", ctypes.c_uint32), ("pad0", ctypes.c_uint32),
                ("pinned_budget_bytes", ctypes.c_uint64)]


class ServerResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("pad", ctypes.c_uint32),
                ("n_v", ctypes.c_uint64), ("n_t", ctypes.c_uint64),
                ("d_idx", ctypes.c_void_p), ("d_pos", ctypes.c_void_p),
                ("h_idx", ctypes.c_void_p), ("h_pos", ctypes.c_void_p),
                ("t_submit_us", ctypes.c_double), ("t_admit_us", ctypes.c_double),
                ("t_done_us", ctypes.c_double)]


# (name, restype, argtypes) of every entry point in include/stride_gb300.h
_P = ctypes.c_void_p
_I = ctypes.c_int
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_SZ = ctypes.c_size_t


class Pldt5Info(ctypes.Structure):
    _fields_ = [("n_meshlets", ctypes.c_uint32), ("n_boundary", ctypes.c_uint32),
                ("g_bits", ctypes.c_uint32 * 3), ("n_v", ctypes.c_uint64), ("n_t", ctypes.c_uint64),
                ("nbytes", ctypes.c_uint64), ("center", ctypes.c_float * 3), ("scale", ctypes.c_float),
                ("lin3_w", ctypes.c_float * 3)]


SIGNATURES = [
    ("stride_last_error_message", ctypes.c_char_p, []),
    ("stride_error_string", ctypes.c_char_p, [_I]),
    ("stride_device_info", _I, [ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("stride_inspect", _I, [_P, _SZ, ctypes.POINTER(StrideInfo)]),
    ("stride_open", _I, [_P, _SZ, ctypes.POINTER(_P)]),
    ("stride_reload", _I, [_P, _P, _SZ, _P]),
    ("stride_info", _I, [_P, ctypes.POINTER(StrideInfo)]),
    ("stride_decode", _I, [_P, _P, _P, _P, _P]),
    ("stride_decode_host", _I, [_P, _P, _P, _P]),
    ("stride_status", _I, [_P, _I, ctypes.POINTER(_U32)]),
    ("stride_decode_timed", _I, [_P, _P, _P, _P, _P]),
    ("stride_side_table", _I, [_P, _P, _P, _P]),
    ("stride_meshlet_ranges", _I, [_P, _P, _P, _P]),
    ("stride_meshlet_bounds", _I, [_P, _P, _P, _P]),
    ("stride_cull_meshlets", _I, [_P, ctypes.c_uint32, _P, _P, _P, _P]),
    ("stride_set_config", _I, [_P, ctypes.POINTER(LaunchCfg)]),
    ("stride_set_wait_limit", _I, [_P, _U64]),
    ("stride_close", None, [_P]),
    ("stride_decode_static", _I, [_P, _SZ, _P, _P, _P]),
    ("stride_batch_create", _I, [_P, _P, _U32, ctypes.POINTER(_P)]),
    ("stride_batch_info", _I, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    ("stride_batch_offsets", _I, [_P, _P, _P]),
    ("stride_batch_set_config", _I, [_P, ctypes.POINTER(LaunchCfg)]),
    ("stride_batch_get_config", _I, [_P, ctypes.POINTER(LaunchCfg)]),
    ("stride_batch_decode", _I, [_P, _P, _P, _P]),
    ("stride_batch_decode_timed", _I, [_P, _P, _P, _P, _P]),
    ("stride_batch_image", _I, [_P, _P, ctypes.POINTER(_U64)]),
    ("stride_batch_upload", _I, [_P, _P, _P, _SZ]),
    ("stride_batch_decode_to_host", _I, [_P, _P, _P, _P, _P, _P]),
    ("stride_batch_capture_graph", _I, [_P, _P, _P, _P]),
    ("stride_batch_launch_graph", _I, [_P, _P]),
    ("stride_batch_autotune", _I, [_P, _P, _P, _P, _I, ctypes.POINTER(LaunchCfg),
                                   ctypes.POINTER(ctypes.c_float)]),
    ("stride_batch_status", _I, [_P, _I, ctypes.POINTER(_U32), ctypes.POINTER(_U32)]),
    ("stride_batch_destroy", None, [_P]),
    ("stride_server_create", _I, [ctypes.POINTER(ServerOpts), ctypes.POINTER(_P)]),
    ("stride_server_submit", _I, [_P, _P, _SZ, ctypes.POINTER(_U64)]),
    ("stride_server_wait", _I, [_P, _U64, _I, ctypes.POINTER(ServerResult)]),
    ("stride_server_release", _I, [_P, _U64]),
    ("stride_server_hold", _I, [_P, _I]),
    ("stride_server_stats", _I, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    ("stride_server_destroy", None, [_P]),
    ("pldt5_open", _I, [_P, _SZ, ctypes.POINTER(_P)]),
    ("pldt5_inspect", _I, [_P, _SZ, ctypes.POINTER(Pldt5Info)]),
    ("pldt5_info", _I, [_P, ctypes.POINTER(Pldt5Info)]),
    ("pldt5_decode", _I, [_P, _P, _P, _P]),
    ("pldt5_status", _I, [_P, _I]),
    ("pldt5_close", None, [_P]),
]

_lib = None
_lock = threading.Lock()


def load():
    """Load the decoder library (raises if it is missing or incomplete)."""
    global _lib
    with _lock:
        if _lib is None:
            lib = ctypes.CDLL(_build.decoder_library())
            for name, res, args in SIGNATURES:
                fn = getattr(lib, name)  # AttributeError: the build is incomplete
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def last_error() -> str:
    return load().stride_last_error_message().decode(errors="replace")


def check(rc: int, what: str = "stride"):
    if rc == STRIDE_OK:
        return
    msg = f"{what}: {load().stride_error_string(rc).decode()} ({last_error()})"
    if rc in FORMAT_ERRORS:
        raise StrideFormatError(rc, msg)
    raise StrideDeviceError(rc, msg)


def inspect_pldt5(data: bytes) -> Pldt5Info:
    """Host-only parse/validation of a PLDT v5 stream (no GPU needed)."""
    info = Pldt5Info()
    data = bytes(data)
    check(load().pldt5_inspect(data, len(data), ctypes.byref(info)), "pldt5_inspect")
    return info


def inspect(data: bytes) -> StrideInfo:
    """Host-only header parse/validation (no GPU needed)."""
    info = StrideInfo()
    data = bytes(data)
    check(load().stride_inspect(data, len(data), ctypes.byref(info)), "stride_inspect")
    return info
