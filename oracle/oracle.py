"""ctypes binding of the C oracles (``stride_oracle.c``, ``pldt5_oracle.c``).

TEST INFRASTRUCTURE ONLY.  The C files restate the reference CPU decoders
``decode_dup`` (STRIDE DPR4 v3, encoder/paradelta_v5_dup.py:471-618) and
``decode_paradelta_v5`` (PLDT v5, encoder/paradelta_v5.py:286-462); this
module builds them with gcc (no FMA contraction, so the float64 arithmetic
rounds exactly like numpy) and exposes them as numpy functions.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "stride_oracle.c")
SOURCES = [SRC, os.path.join(HERE, "pldt5_oracle.c")]
HEADERS = [os.path.join(HERE, "so_bits.h")]
LIB = os.path.join(HERE, "libstride_oracle.so")

_lib = None


class OracleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"oracle error {code}: {msg}")
        self.code = code


def build(force: bool = False) -> str:
    """Compile the oracles with gcc (-O2, no FMA contraction)."""
    stale = not os.path.exists(LIB) or any(os.path.getmtime(LIB) < os.path.getmtime(f) for f in SOURCES + HEADERS)
    if force or stale:
        cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math",
               "-fPIC", "-shared", "-pthread", *SOURCES, "-o", LIB + ".tmp", "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def library_path() -> str:
    return LIB


class _Header(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_uint32), ("version", ctypes.c_uint32),
                ("code_width", ctypes.c_uint32),
                ("center", ctypes.c_float * 3), ("scale", ctypes.c_float),
                ("per_coord_err", ctypes.c_float), ("g_min", ctypes.c_float * 3),
                ("g_range", ctypes.c_float * 3), ("g_bits", ctypes.c_uint32 * 3),
                ("pred_n", ctypes.c_int32 * 9), ("pred_k", ctypes.c_uint32 * 3),
                ("n_v_total", ctypes.c_uint32), ("n_t", ctypes.c_uint32),
                ("n_meshlets", ctypes.c_uint32), ("body_bit", ctypes.c_uint64)]


class _P5Header(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_uint32), ("version", ctypes.c_uint32),
                ("code_width", ctypes.c_uint32),
                ("center", ctypes.c_float * 3), ("scale", ctypes.c_float),
                ("per_coord_err", ctypes.c_float), ("g_min", ctypes.c_float * 3),
                ("g_range", ctypes.c_float * 3), ("g_bits", ctypes.c_uint32 * 3),
                ("n_v", ctypes.c_uint32), ("n_t", ctypes.c_uint32),
                ("n_boundary", ctypes.c_uint32), ("n_meshlets", ctypes.c_uint32),
                ("lin3_w", ctypes.c_float * 3), ("boundary_bit", ctypes.c_uint64)]


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        lib.so_error.restype = ctypes.c_char_p
        lib.so_error.argtypes = [ctypes.c_int]
        lib.so_parse_header.argtypes = [u8p, ctypes.c_uint64, ctypes.POINTER(_Header)]
        lib.so_decode.argtypes = [u8p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                                  ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        lib.so_decode_mt.argtypes = [u8p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        lib.so_bitcodec_read.argtypes = [u8p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_int32, ctypes.c_void_p]
        lib.so_side_table.argtypes = [u8p, ctypes.c_uint64] + [ctypes.c_void_p] * 7
        lib.p5_parse_header.argtypes = [u8p, ctypes.c_uint64, ctypes.POINTER(_P5Header)]
        lib.p5_decode.argtypes = [u8p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                  ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        lib.p5_tables.argtypes = [u8p, ctypes.c_uint64] + [ctypes.c_void_p] * 6
        _lib = lib
    return _lib


def _buf(data: bytes):
    arr = np.frombuffer(data, dtype=np.uint8)
    return arr, arr.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def _check(rc: int):
    if rc != 0:
        raise OracleError(rc, _load().so_error(rc).decode())


@dataclass
class Header:
    code_width: int
    center: np.ndarray
    scale: float
    per_coord_err: float
    g_min: np.ndarray
    g_range: np.ndarray
    g_bits: np.ndarray
    pred_n: np.ndarray
    pred_k: np.ndarray
    n_v_total: int
    n_t: int
    n_meshlets: int


def parse_header(data: bytes) -> Header:
    lib = _load()
    arr, p = _buf(data)
    h = _Header()
    _check(lib.so_parse_header(p, len(arr), ctypes.byref(h)))
    return Header(int(h.code_width), np.array(h.center[:], np.float32), float(h.scale),
                  float(h.per_coord_err), np.array(h.g_min[:], np.float32),
                  np.array(h.g_range[:], np.float32), np.array(h.g_bits[:], np.int64),
                  np.array(h.pred_n[:], np.int64).reshape(3, 3), np.array(h.pred_k[:], np.int64),
                  int(h.n_v_total), int(h.n_t), int(h.n_meshlets))


def decode(data: bytes, *, with_codes: bool = False, slack: int = 1 << 16):
    """Sequential decode -> (pos float32 (n_v, 3), idx int64 (n_t, 3)[, codes int64])."""
    lib = _load()
    h = parse_header(data)
    arr, p = _buf(data)
    cap_v = h.n_v_total + slack
    cap_t = h.n_t + slack
    pos = np.empty((cap_v, 3), np.float32)
    idx = np.empty((cap_t, 3), np.int64)
    codes = np.empty((cap_v, 3), np.int64) if with_codes else None
    nv = ctypes.c_uint64()
    nt = ctypes.c_uint64()
    _check(lib.so_decode(p, len(arr), pos.ctypes.data, idx.ctypes.data,
                         codes.ctypes.data if codes is not None else None,
                         cap_v, cap_t, ctypes.byref(nv), ctypes.byref(nt)))
    out = (pos[:nv.value], idx[:nt.value])
    if with_codes:
        out = out + (codes[:nv.value],)
    return out


def decode_mt(data: bytes, n_threads: int = 0, *, out=None):
    """Meshlet-parallel decode on ``n_threads`` host threads (0 = all cores)."""
    lib = _load()
    h = parse_header(data)
    arr, p = _buf(data)
    if n_threads <= 0:
        n_threads = os.cpu_count() or 1
    if out is None:
        pos = np.empty((h.n_v_total, 3), np.float32)
        idx = np.empty((h.n_t, 3), np.int64)
    else:
        pos, idx = out
    nv = ctypes.c_uint64()
    nt = ctypes.c_uint64()
    _check(lib.so_decode_mt(p, len(arr), pos.ctypes.data, idx.ctypes.data,
                            pos.shape[0], idx.shape[0], n_threads,
                            ctypes.byref(nv), ctypes.byref(nt)))
    return pos[:nv.value], idx[:nt.value]


def bitcodec_read(data: bytes, ops):
    """Read fields: ops = [(kind, k), ...], kind 'fixed' | 'rice' | 'eg'."""
    lib = _load()
    arr, p = _buf(data)
    kinds = np.array([{"fixed": 0, "rice": 1, "eg": 2}[o[0]] for o in ops], np.int32)
    ks = np.array([o[1] for o in ops], np.int32)
    out = np.zeros(len(ops), np.uint64)
    _check(lib.so_bitcodec_read(p, len(arr), kinds.ctypes.data, ks.ctypes.data,
                                len(ops), out.ctypes.data))
    return [int(x) for x in out]


def side_table(data: bytes):
    """Per-meshlet side table of the reference GPU harness's blob, from the
    DPR4 bytes: start_bit, n_local, n_tris, n_strips, resid_bit (the anchor),
    n_kind0 and sub_offs (M, 5) -- starts of dy, dz, px, py, pz relative to
    the anchor.  Bit positions are absolute in ``data``."""
    lib = _load()
    h = parse_header(data)
    arr, p = _buf(data)
    M = h.n_meshlets
    out = {"start_bit": np.zeros(M, np.uint64), "n_local": np.zeros(M, np.uint32),
           "n_tris": np.zeros(M, np.uint32), "n_strips": np.zeros(M, np.uint32),
           "resid_bit": np.zeros(M, np.uint64), "n_kind0": np.zeros(M, np.uint32),
           "sub_offs": np.zeros((M, 5), np.uint16)}
    _check(lib.so_side_table(p, len(arr), *[out[k].ctypes.data for k in
                                            ("start_bit", "n_local", "n_tris", "n_strips", "resid_bit",
                                             "n_kind0", "sub_offs")]))
    return out


# ---------------------------------------------------------------- PLDT v5 --
def parse_header_v5(data: bytes) -> _P5Header:
    """Global header of a PLDT v5 stream (encoder/paradelta_v5.py:290-306)."""
    lib = _load()
    arr, p = _buf(data)
    h = _P5Header()
    _check(lib.p5_parse_header(p, len(arr), ctypes.byref(h)))
    return h


def decode_v5(data: bytes):
    """Decode a PLDT v5 stream like ``decode_paradelta_v5``: returns
    (positions float32 (n_v, 3), triangles int64 (n_t, 3)); the rows are the
    boundary vertices, then every meshlet's interior vertices."""
    lib = _load()
    arr, p = _buf(data)
    nv, nt = ctypes.c_uint64(), ctypes.c_uint64()
    _check(lib.p5_decode(p, len(arr), None, None, 0, 0, ctypes.byref(nv), ctypes.byref(nt)))
    pos = np.empty((nv.value, 3), np.float32)
    idx = np.empty((nt.value, 3), np.int64)
    _check(lib.p5_decode(p, len(arr), pos.ctypes.data, idx.ctypes.data, nv.value, nt.value,
                         ctypes.byref(nv), ctypes.byref(nt)))
    return pos, idx


def tables_v5(data: bytes):
    """Per-meshlet tables of a PLDT v5 stream as the reference GPU decoder
    derives them (utils/paradelta_v5_cuda.py:515-660): absolute start bits,
    n_bnd, n_int, n_tris, n_strips (int32) and the float64 boundary rows."""
    lib = _load()
    arr, p = _buf(data)
    h = parse_header_v5(data)
    M, nb = h.n_meshlets, h.n_boundary
    out = {"off_bits": np.zeros(M, np.uint64), "n_bnd": np.zeros(M, np.int32), "n_int": np.zeros(M, np.int32),
           "n_tris": np.zeros(M, np.int32), "n_strips": np.zeros(M, np.int32),
           "bnd_rows": np.zeros((nb, 3), np.float64)}
    _check(lib.p5_tables(p, len(arr), *[out[k].ctypes.data for k in
                                        ("off_bits", "n_bnd", "n_int", "n_tris", "n_strips", "bnd_rows")]))
    return out
