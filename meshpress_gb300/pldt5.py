"""GPU decoder for PLDT v5 streams, the format the reference's CuPy
``ParaDeltaV5GpuDecoder`` reads (utils/paradelta_v5_cuda.py:515-718).

``ParaDeltaV5GpuDecoder(data)`` returns a ``PldtV5Decoder`` when ``data`` is a
PLDT v5 stream (magic 0x504C4454, version 5), so code written against the
reference's class keeps working on its old bytes.  Decoding runs in
``libstride_gb300.so`` (``pldt5_*`` in include/stride_gb300.h) and matches the
reference CPU decoder ``decode_paradelta_v5`` (encoder/paradelta_v5.py:286-462)
bit for bit; rows are the boundary vertices, then every meshlet's interior
vertices.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _torch():
    import torch
    return torch


def _stream_handle(stream=None) -> int:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def is_pldt5(data) -> bool:
    """True for a PLDT v5 stream (magic and version bytes)."""
    b = bytes(data[:5])
    return len(b) == 5 and b[:4] == b"PLDT" and b[4] == 5


class PldtV5Decoder:
    """One PLDT v5 stream on the GPU.  Attributes as the reference's class:
    ``n_meshlets``, ``n_boundary``, ``n_v_total``, ``n_t_total``,
    ``meshlets_per_block`` (accepted, in [1, 16])."""

    def __init__(self, data: bytes, meshlets_per_block: int = 1):
        if meshlets_per_block < 1 or meshlets_per_block > 16:
            raise ValueError("meshlets_per_block must be in [1, 16]")
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("CUDA device not available: the PLDT v5 decoder runs on the GPU only")
        self.meshlets_per_block = int(meshlets_per_block)
        self._lib = _lib.load()
        self._data = bytes(data)
        torch.cuda.init()
        h = ctypes.c_void_p()
        _lib.check(self._lib.pldt5_open(self._data, len(self._data), ctypes.byref(h)), "pldt5_open")
        self._h = h
        info = _lib.Pldt5Info()
        _lib.check(self._lib.pldt5_info(self._h, ctypes.byref(info)), "pldt5_info")
        self.info = info
        self.n_meshlets = int(info.n_meshlets)
        self.n_boundary = int(info.n_boundary)
        self.n_v_total = int(info.n_v)
        self.n_t_total = int(info.n_t)
        self.d_verts = None
        self.d_tris = None
        self._device = torch.cuda.current_device()

    def _outputs(self):
        torch = _torch()
        if self.d_tris is None:
            self.d_tris = torch.empty((self.n_t_total, 3), dtype=torch.uint32, device=f"cuda:{self._device}")
            self.d_verts = torch.empty((self.n_v_total, 3), dtype=torch.float32, device=f"cuda:{self._device}")
        return self.d_tris, self.d_verts

    def decode_into(self, d_idx, d_pos, *, stream=None, check: bool = True):
        """Decode into caller-provided CUDA tensors (32-bit (n_t, 3) indices,
        float32 (n_v, 3) world positions)."""
        assert d_idx.is_cuda and d_pos.is_cuda and d_idx.is_contiguous() and d_pos.is_contiguous()
        assert d_idx.numel() >= 3 * self.n_t_total and d_pos.numel() >= 3 * self.n_v_total
        rc = self._lib.pldt5_decode(self._h, ctypes.c_void_p(_stream_handle(stream)),
                                    ctypes.c_void_p(d_idx.data_ptr()), ctypes.c_void_p(d_pos.data_ptr()))
        _lib.check(rc, "pldt5_decode")
        if check:
            self.check()

    def check(self):
        """Wait for the last decode and raise if the stream was invalid."""
        _lib.check(self._lib.pldt5_status(self._h, 1), "pldt5 decode")

    def decode_to_device(self, *, stream=None, check: bool = True):
        """-> (triangles torch.uint32 (n_t, 3), positions torch.float32 (n_v, 3))
        in world space, resident on the GPU (reused by later calls)."""
        tris, verts = self._outputs()
        self.decode_into(tris, verts, stream=stream, check=check)
        return tris, verts

    def decode(self, *, stream=None, check: bool = True):
        """Reference order: -> (positions, triangles) as CUDA tensors (the
        reference returns normalised positions and int32 triangles, :712)."""
        tris, verts = self.decode_to_device(stream=stream, check=check)
        return verts, tris

    def decode_to_host(self, out=None, *, stream=None):
        """-> (positions np.float32 (n_v, 3), triangles np.uint32 (n_t, 3))
        (reference :714-718)."""
        tris, verts = self.decode_to_device(stream=stream)
        if out is None:
            return verts.cpu().numpy(), tris.view(_torch().int32).cpu().numpy().view(np.uint32)
        pos, idx = out
        pos[...] = verts.cpu().numpy()
        idx[...] = tris.view(_torch().int32).cpu().numpy().view(np.uint32)
        return pos, idx

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pldt5_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
