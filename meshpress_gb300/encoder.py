"""Python binding of the project STRIDE (DPR4 v3) encoder.

The encoder is the caller-side producer of decoder inputs (C++, host only,
``csrc/encoder/stride_encode.cpp``).  It writes the byte layout of the
reference ``encode_dup`` (encoder/paradelta_v5_dup.py:316-464) with its own
meshlet partition, strips and predictor fit, so the GPU decoder can be fed
meshes of millions of triangles in seconds.

``STRIDEEncoder`` mirrors the constructor of the reference class
(encoder/implementation/stride.py:18-53): ``max_verts``, ``max_tris``,
``precision_error``, ``precision_mode`` ("world" | "bbox_frac") and
``predictor`` ("generalized" -> the fitted integer-rational predictor,
"canonical" -> (1, 1, -1), K = 0).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import _build

_lib = None


class _Opts(ctypes.Structure):
    _fields_ = [("max_verts", ctypes.c_int32), ("max_tris", ctypes.c_int32),
                ("precision_error", ctypes.c_double), ("precision_mode", ctypes.c_int32),
                ("predictor", ctypes.c_int32)]


def _load():
    global _lib
    if _lib is None:
        path = _build.encoder_library()
        lib = ctypes.CDLL(path)
        lib.stride_encode.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                      ctypes.c_uint64, ctypes.POINTER(_Opts),
                                      ctypes.POINTER(ctypes.c_void_p)]
        lib.stride_encode.restype = ctypes.c_int
        lib.stride_encode_last_error.restype = ctypes.c_char_p
        for name, rt in (("stride_encode_nbytes", ctypes.c_uint64),
                         ("stride_encode_bytes", ctypes.c_void_p),
                         ("stride_encode_n_dup", ctypes.c_uint64),
                         ("stride_encode_l2g", ctypes.c_void_p),
                         ("stride_encode_codes", ctypes.c_void_p),
                         ("stride_encode_n_meshlets", ctypes.c_uint32)):
            fn = getattr(lib, name)
            fn.argtypes = [ctypes.c_void_p]
            fn.restype = rt
        lib.stride_encode_free.argtypes = [ctypes.c_void_p]
        lib.pldt5_encode.argtypes = lib.stride_encode.argtypes
        lib.pldt5_encode.restype = ctypes.c_int
        for name, rt in (("pldt5_encode_nbytes", ctypes.c_uint64), ("pldt5_encode_bytes", ctypes.c_void_p),
                         ("pldt5_encode_n_rows", ctypes.c_uint64), ("pldt5_encode_rows", ctypes.c_void_p),
                         ("pldt5_encode_n_meshlets", ctypes.c_uint32),
                         ("pldt5_encode_n_boundary", ctypes.c_uint32)):
            fn = getattr(lib, name)
            fn.argtypes = [ctypes.c_void_p]
            fn.restype = rt
        lib.pldt5_encode_free.argtypes = [ctypes.c_void_p]
        _lib = lib
    return _lib


@dataclass
class EncodedMesh:
    """Encoder output: the DPR4 bytes plus, per decoded (duplicated) vertex,
    the source vertex id and its integer quantisation code."""
    data: bytes
    l2g: np.ndarray      # uint32 (n_v_dup,)
    codes: np.ndarray    # int32 (n_v_dup, 3)
    n_meshlets: int

    @property
    def n_v_dup(self) -> int:
        return int(self.l2g.shape[0])


def encode(verts, tris, *, max_verts: int = 256, max_tris: int = 256,
           precision_error: float = 0.0005, precision_mode: str = "world",
           predictor: str = "generalized") -> EncodedMesh:
    lib = _load()
    V = np.ascontiguousarray(verts, dtype=np.float64)
    T = np.ascontiguousarray(tris, dtype=np.int64)
    if V.ndim != 2 or V.shape[1] != 3 or T.ndim != 2 or T.shape[1] != 3:
        raise ValueError("verts and tris must be (n, 3) arrays")
    if precision_mode not in ("world", "bbox_frac"):
        raise ValueError(f"unknown precision_mode={precision_mode!r}")
    if predictor not in ("generalized", "canonical"):
        raise ValueError(f"predictor must be 'generalized' or 'canonical', got {predictor!r}")
    opts = _Opts(int(max_verts), int(max_tris), float(precision_error),
                 0 if precision_mode == "world" else 1,
                 1 if predictor == "generalized" else 0)
    h = ctypes.c_void_p()
    rc = lib.stride_encode(V.ctypes.data, V.shape[0], T.ctypes.data, T.shape[0],
                           ctypes.byref(opts), ctypes.byref(h))
    if rc != 0:
        raise ValueError(f"stride_encode failed: {lib.stride_encode_last_error().decode()}")
    try:
        n = lib.stride_encode_nbytes(h)
        data = ctypes.string_at(lib.stride_encode_bytes(h), n)
        nd = lib.stride_encode_n_dup(h)
        l2g = np.ctypeslib.as_array(ctypes.cast(lib.stride_encode_l2g(h), ctypes.POINTER(ctypes.c_uint32)),
                                    shape=(nd,)).copy() if nd else np.zeros(0, np.uint32)
        codes = np.ctypeslib.as_array(ctypes.cast(lib.stride_encode_codes(h), ctypes.POINTER(ctypes.c_int32)),
                                      shape=(nd, 3)).copy() if nd else np.zeros((0, 3), np.int32)
        nm = int(lib.stride_encode_n_meshlets(h))
    finally:
        lib.stride_encode_free(h)
    return EncodedMesh(data, l2g, codes, nm)


@dataclass
class EncodedPldt5:
    """A PLDT v5 stream and, per decoded row (the boundary vertices, then
    every meshlet's interior vertices), its source vertex id."""
    data: bytes
    rows: np.ndarray     # uint32 (n_rows,)
    n_meshlets: int
    n_boundary: int


def encode_pldt5(verts, tris, *, max_verts: int = 256, max_tris: int = 256,
                 precision_error: float = 0.0005, precision_mode: str = "world") -> EncodedPldt5:
    """Encode a mesh as PLDT v5, the format of the reference's CuPy decoder
    (encoder/paradelta_v5.py:144-279), for decoder inputs at scale: this
    project's partition, strips and quantisation, canonical lin3 weights."""
    lib = _load()
    V = np.ascontiguousarray(verts, dtype=np.float64)
    T = np.ascontiguousarray(tris, dtype=np.int64)
    if V.ndim != 2 or V.shape[1] != 3 or T.ndim != 2 or T.shape[1] != 3:
        raise ValueError("verts and tris must be (n, 3) arrays")
    if precision_mode not in ("world", "bbox_frac"):
        raise ValueError(f"unknown precision_mode={precision_mode!r}")
    opts = _Opts(int(max_verts), int(max_tris), float(precision_error), 0 if precision_mode == "world" else 1, 0)
    h = ctypes.c_void_p()
    rc = lib.pldt5_encode(V.ctypes.data, V.shape[0], T.ctypes.data, T.shape[0], ctypes.byref(opts), ctypes.byref(h))
    if rc != 0:
        raise ValueError(f"pldt5_encode failed: {lib.stride_encode_last_error().decode()}")
    try:
        data = ctypes.string_at(lib.pldt5_encode_bytes(h), lib.pldt5_encode_nbytes(h))
        nr = lib.pldt5_encode_n_rows(h)
        rows = np.ctypeslib.as_array(ctypes.cast(lib.pldt5_encode_rows(h), ctypes.POINTER(ctypes.c_uint32)),
                                     shape=(nr,)).copy() if nr else np.zeros(0, np.uint32)
        out = EncodedPldt5(data, rows, int(lib.pldt5_encode_n_meshlets(h)), int(lib.pldt5_encode_n_boundary(h)))
    finally:
        lib.pldt5_encode_free(h)
    return out


@dataclass
class CompressedModel:
    """Same fields as the reference ``CompressedModel`` (utils/types.py:231-235)."""
    data: bytes
    bits_per_vertex: float
    bits_per_triangle: float


class STRIDEEncoder:
    """Encoder with the reference STRIDEEncoder's constructor arguments."""

    def __init__(self, *, max_verts: int = 256, max_tris: int = 256,
                 precision_error: float = 0.0005, precision_mode: str = "world",
                 predictor: str = "generalized"):
        self.max_verts = max_verts
        self.max_tris = max_tris
        self.precision_error = precision_error
        self.precision_mode = precision_mode
        self.predictor = predictor

    def encode_arrays(self, verts, tris) -> EncodedMesh:
        return encode(verts, tris, max_verts=self.max_verts, max_tris=self.max_tris,
                      precision_error=self.precision_error,
                      precision_mode=self.precision_mode, predictor=self.predictor)

    def encode(self, verts, tris) -> CompressedModel:
        e = self.encode_arrays(verts, tris)
        n_v = len(verts)
        n_t = len(tris)
        return CompressedModel(e.data, len(e.data) * 8 / n_v, len(e.data) * 8 / n_t)
