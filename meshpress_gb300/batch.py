"""Many STRIDE streams decoded by one launch (C ABI ``stride_batch_*``).

The reference decodes one mesh per ``ParaDeltaV5GpuDecoder``
(utils/paradelta_v5_cuda.py:580-718); this adds a batch: every stream is
copied into one device arena, one device meshlet queue spans all of them,
and the same parse + decode kernels run once over the whole batch (with a
persistent, work-stealing grid when the autotuner picks it), optionally
replayed from a captured CUDA graph.  Outputs are concatenated: mesh ``i``
owns triangles ``[t_offset[i], t_offset[i+1])`` (indices local to the mesh)
and positions ``[v_offset[i], v_offset[i+1])``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


class BatchDecoder:
    def __init__(self, blobs):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("CUDA device not available: the STRIDE decoder runs on the GPU only")
        self._lib = _lib.load()
        self._blobs = [bytes(b) for b in blobs]
        n = len(self._blobs)
        if n == 0:
            raise ValueError("empty batch")
        ptrs = (ctypes.c_char_p * n)(*self._blobs)
        lens = (ctypes.c_size_t * n)(*[len(b) for b in self._blobs])
        h = ctypes.c_void_p()
        _lib.check(self._lib.stride_batch_create(ctypes.cast(ptrs, ctypes.c_void_p), ctypes.cast(lens, ctypes.c_void_p),
                                                 n, ctypes.byref(h)), "stride_batch_create")
        self._h = h
        nm, nv, nt = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(self._lib.stride_batch_info(h, ctypes.byref(nm), ctypes.byref(nv), ctypes.byref(nt)))
        self.n_meshes = n
        self.n_meshlets, self.n_v_total, self.n_t_total = int(nm.value), int(nv.value), int(nt.value)
        vo = np.zeros(n, np.uint64)
        to = np.zeros(n, np.uint64)
        _lib.check(self._lib.stride_batch_offsets(h, ctypes.c_void_p(vo.ctypes.data), ctypes.c_void_p(to.ctypes.data)))
        self.v_offset = np.append(vo, np.uint64(self.n_v_total)).astype(np.int64)
        self.t_offset = np.append(to, np.uint64(self.n_t_total)).astype(np.int64)
        self._device = torch.cuda.current_device()
        self.d_tris = torch.empty((self.n_t_total, 3), dtype=torch.uint32, device=f"cuda:{self._device}")
        self.d_verts = torch.empty((self.n_v_total, 3), dtype=torch.float32, device=f"cuda:{self._device}")

    @staticmethod
    def _stream(stream=None) -> ctypes.c_void_p:
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        return ctypes.c_void_p(int(s.cuda_stream))

    def _ptrs(self):
        return ctypes.c_void_p(self.d_tris.data_ptr()), ctypes.c_void_p(self.d_verts.data_ptr())

    def config(self) -> _lib.LaunchCfg:
        c = _lib.LaunchCfg()
        _lib.check(self._lib.stride_batch_get_config(self._h, ctypes.byref(c)))
        return c

    def set_config(self, cfg: _lib.LaunchCfg):
        _lib.check(self._lib.stride_batch_set_config(self._h, ctypes.byref(cfg)), "stride_batch_set_config")

    def decode(self, *, stream=None, check: bool = True):
        """-> (triangles uint32 (n_t, 3), positions float32 (n_v, 3)), device."""
        i, p = self._ptrs()
        _lib.check(self._lib.stride_batch_decode(self._h, self._stream(stream), i, p), "stride_batch_decode")
        if check:
            self.check()
        return self.d_tris, self.d_verts

    def decode_timed(self, *, stream=None):
        """Synchronous decode; -> device milliseconds of (scan, connectivity,
        vertex) kernels."""
        i, p = self._ptrs()
        ms = (ctypes.c_float * 3)()
        _lib.check(self._lib.stride_batch_decode_timed(self._h, self._stream(stream), i, p, ms), "decode_timed")
        self.check()
        return tuple(float(x) for x in ms)

    def decode_to_host(self, out=None, *, stream=None):
        """Decode and copy the outputs to host memory, the copies overlapping
        the decode; -> (positions float32 (n_v, 3), triangles uint32 (n_t,
        3)), numpy.  ``out`` = (positions, triangles) host arrays of those
        shapes (pinned memory makes the copies asynchronous); by default
        new arrays."""
        if out is None:
            pos = np.empty((self.n_v_total, 3), np.float32)
            idx = np.empty((self.n_t_total, 3), np.uint32)
        else:
            pos, idx = out
            if pos.shape != (self.n_v_total, 3) or pos.dtype != np.float32 or not pos.flags.c_contiguous:
                raise ValueError("positions: a C-contiguous float32 array of shape (n_v, 3)")
            if idx.shape != (self.n_t_total, 3) or idx.dtype != np.uint32 or not idx.flags.c_contiguous:
                raise ValueError("triangles: a C-contiguous uint32 array of shape (n_t, 3)")
        i, p = self._ptrs()
        _lib.check(self._lib.stride_batch_decode_to_host(self._h, self._stream(stream), i, p,
                                                         ctypes.c_void_p(idx.ctypes.data),
                                                         ctypes.c_void_p(pos.ctypes.data)), "batch decode to host")
        return pos, idx

    def image(self):
        """-> (blob offsets (n_meshes,), image bytes): layout of the arena
        image that ``upload`` takes."""
        off = np.zeros(self.n_meshes, np.uint64)
        nb = ctypes.c_uint64()
        _lib.check(self._lib.stride_batch_image(self._h, ctypes.c_void_p(off.ctypes.data), ctypes.byref(nb)))
        return off.astype(np.int64), int(nb.value)

    def make_image(self, blobs=None) -> np.ndarray:
        """Host arena image of ``blobs`` (default: the batch's own streams)."""
        blobs = self._blobs if blobs is None else [bytes(b) for b in blobs]
        off, nb = self.image()
        img = np.zeros(nb, np.uint8)
        for o, b in zip(off, blobs):
            img[o:o + len(b)] = np.frombuffer(b, np.uint8)
        return img

    def upload(self, image_ptr: int, nbytes: int, *, stream=None):
        """Replace every stream from a host image (one asynchronous copy
        when the image is in pinned memory)."""
        _lib.check(self._lib.stride_batch_upload(self._h, self._stream(stream), ctypes.c_void_p(image_ptr),
                                                 int(nbytes)), "stride_batch_upload")

    def check(self):
        bm, bl = ctypes.c_uint32(), ctypes.c_uint32()
        _lib.check(self._lib.stride_batch_status(self._h, 1, ctypes.byref(bm), ctypes.byref(bl)), "batch decode")

    def capture_graph(self, stream):
        i, p = self._ptrs()
        _lib.check(self._lib.stride_batch_capture_graph(self._h, self._stream(stream), i, p), "graph capture")

    def launch_graph(self, stream, *, check: bool = False):
        _lib.check(self._lib.stride_batch_launch_graph(self._h, self._stream(stream)), "graph launch")
        if check:
            self.check()

    def autotune(self, iters: int = 3, *, stream=None):
        """Time every launch shape on this batch, keep the fastest."""
        i, p = self._ptrs()
        best = _lib.LaunchCfg()
        ms = ctypes.c_float()
        _lib.check(self._lib.stride_batch_autotune(self._h, self._stream(stream), i, p, int(iters),
                                                   ctypes.byref(best), ctypes.byref(ms)), "autotune")
        return best, float(ms.value)

    def mesh(self, i: int):
        """(triangles, positions) views of mesh i in the concatenated outputs."""
        return (self.d_tris[self.t_offset[i]:self.t_offset[i + 1]],
                self.d_verts[self.v_offset[i]:self.v_offset[i + 1]])

    def close(self):
        if getattr(self, "_h", None):
            self._lib.stride_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
