"""Drop-in replacement for the reference ``ParaDeltaV5GpuDecoder``.

Reference: utils/paradelta_v5_cuda.py:580-718.  Same class name, constructor
(``data``, ``meshlets_per_block`` in [1, 16]) and ``decode()`` /
``decode_to_host()`` methods, plus ``decode_to_device()``.  The input is the
DPR4 v3 bitstream that ``STRIDEEncoder`` writes
(encoder/paradelta_v5_dup.py:316-464), or a PLDT v5 stream (the reference
class's own format), for which the constructor returns a
``pldt5.PldtV5Decoder``; any other stream (PLDT v4 included) is rejected
with ``ValueError`` like any other bad magic (utils/paradelta_v5_cuda.py:520).

Everything runs in ``libstride_gb300.so`` through its C ABI; PyTorch only
provides device memory and the current stream.  There is no CPU fallback:
without a CUDA device the constructor raises ``RuntimeError`` (the reference
raises ``RuntimeError("cupy not installed")`` in the same place, :598-599).
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


class ParaDeltaV5GpuDecoder:
    """GPU decoder for one STRIDE (DPR4 v3) stream.

    Attributes kept from the reference (utils/paradelta_v5_cuda.py:597-684,
    read by scripts/bench_stride_decode_sweep.py:53-79): ``n_meshlets``,
    ``n_v_total``, ``n_t_total``, ``meshlets_per_block`` (accepted for
    compatibility; the reference kernel ignores it too, :259-260), ``d_buf``
    (the stream on the device, uint8), ``d_verts_norm`` (normalised
    positions of the last ``decode(normalised=True)``), ``d_tris``,
    ``_shared_bytes`` and ``_persistent_blocks`` (shared memory per CTA and
    CTAs of the last decode's main kernel).
    """

    def __new__(cls, data: bytes = b"", meshlets_per_block: int = 1):
        from .pldt5 import PldtV5Decoder, is_pldt5
        if cls is ParaDeltaV5GpuDecoder and is_pldt5(data):
            return PldtV5Decoder(data, meshlets_per_block)  # __init__ below is not run for it
        return super().__new__(cls)

    def __init__(self, data: bytes, meshlets_per_block: int = 1):
        if meshlets_per_block < 1 or meshlets_per_block > 16:
            raise ValueError("meshlets_per_block must be in [1, 16]")
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError("CUDA device not available: the STRIDE decoder runs on the GPU only")
        self.meshlets_per_block = int(meshlets_per_block)
        self._lib = _lib.load()
        self._data = bytes(data)
        torch.cuda.init()
        h = ctypes.c_void_p()
        _lib.check(self._lib.stride_open(self._data, len(self._data), ctypes.byref(h)), "stride_open")
        self._h = h
        info = _lib.StrideInfo()
        _lib.check(self._lib.stride_info(self._h, ctypes.byref(info)), "stride_info")
        self.info = info
        self.n_meshlets = int(info.n_meshlets)
        self.n_v_total = int(info.n_v)
        self.n_t_total = int(info.n_t)
        self.g_bits = tuple(int(b) for b in info.g_bits)
        self.d_verts = None
        self.d_tris = None
        self.d_verts_norm = None
        self._d_buf = None
        self._device = torch.cuda.current_device()

    # -- reference attributes --------------------------------------------------
    @property
    def d_buf(self):
        """The encoded stream on the device (torch.uint8), made on first use."""
        if self._d_buf is None:
            torch = _torch()
            self._d_buf = torch.frombuffer(bytearray(self._data), dtype=torch.uint8).to(f"cuda:{self._device}")
        return self._d_buf

    def _launch_info(self):
        info = _lib.StrideInfo()
        _lib.check(self._lib.stride_info(self._h, ctypes.byref(info)), "stride_info")
        return info

    @property
    def _shared_bytes(self) -> int:
        """Dynamic shared memory per CTA of the last decode's main kernel
        (0 before the first decode)."""
        return int(self._launch_info().shared_bytes)

    @property
    def _persistent_blocks(self) -> int:
        """CTAs of the last decode's main kernel (0 before the first decode)."""
        return int(self._launch_info().persistent_blocks)

    # -- launch configuration ------------------------------------------------
    def set_launch_config(self, cfg: _lib.LaunchCfg):
        _lib.check(self._lib.stride_set_config(self._h, ctypes.byref(cfg)), "stride_set_config")
        _lib.check(self._lib.stride_info(self._h, ctypes.byref(self.info)), "stride_info")  # kernels per decode

    # -- decoding --------------------------------------------------------------
    def _outputs(self):
        torch = _torch()
        if self.d_tris is None:
            self.d_tris = torch.empty((self.n_t_total, 3), dtype=torch.uint32, device=f"cuda:{self._device}")
            self.d_verts = torch.empty((self.n_v_total, 3), dtype=torch.float32, device=f"cuda:{self._device}")
        return self.d_tris, self.d_verts

    def decode_into(self, d_idx, d_pos, *, codes=None, stream=None, check: bool = True):
        """Decode into caller-provided CUDA tensors (uint32 (n_t, 3), float32
        (n_v, 3)); ``codes`` optionally receives the int32 (n_v, 3) codes."""
        torch = _torch()
        assert d_idx.is_cuda and d_pos.is_cuda and d_idx.is_contiguous() and d_pos.is_contiguous()
        assert d_idx.numel() >= 3 * self.n_t_total and d_pos.numel() >= 3 * self.n_v_total
        cptr = None
        if codes is not None:
            assert codes.dtype == torch.int32 and codes.is_cuda and codes.numel() >= 3 * self.n_v_total
            cptr = ctypes.c_void_p(codes.data_ptr())
        rc = self._lib.stride_decode(self._h, ctypes.c_void_p(_stream_handle(stream)),
                                     ctypes.c_void_p(d_idx.data_ptr()), ctypes.c_void_p(d_pos.data_ptr()), cptr)
        _lib.check(rc, "stride_decode")
        if check:
            self.check()

    def check(self):
        """Wait for the last decode and raise if the stream was invalid."""
        bad = ctypes.c_uint32()
        _lib.check(self._lib.stride_status(self._h, 1, ctypes.byref(bad)), "stride decode")

    def meshlet_ranges(self, *, stream=None):
        """Where each meshlet's rows lie in the last decode's outputs ->
        (v_first, t_first) torch.int64 (n_meshlets + 1,) exclusive prefix
        sums; meshlet m owns vertex rows v_first[m]:v_first[m+1]."""
        torch = _torch()
        dev = torch.device("cuda", torch.cuda.current_device())
        v = torch.empty(self.n_meshlets + 1, dtype=torch.int64, device=dev)
        t = torch.empty(self.n_meshlets + 1, dtype=torch.int64, device=dev)
        _lib.check(self._lib.stride_meshlet_ranges(self._h, ctypes.c_void_p(_stream_handle(stream)),
                                                   ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(t.data_ptr())),
                   "stride_meshlet_ranges")
        return v, t

    def meshlet_bounds(self, verts, *, stream=None):
        """Axis-aligned bounds of each meshlet's rows of ``verts`` (the last
        decode's positions, CUDA float32 (n_v, 3)) -> torch.float32
        (n_meshlets, 6): min x y z, max x y z."""
        torch = _torch()
        assert verts.is_cuda and verts.dtype == torch.float32 and verts.is_contiguous()
        assert verts.numel() >= 3 * self.n_v_total
        out = torch.empty((self.n_meshlets, 6), dtype=torch.float32, device=verts.device)
        _lib.check(self._lib.stride_meshlet_bounds(self._h, ctypes.c_void_p(_stream_handle(stream)),
                                                   ctypes.c_void_p(verts.data_ptr()), ctypes.c_void_p(out.data_ptr())),
                   "stride_meshlet_bounds")
        return out

    def side_table(self, *, stream=None):
        """The last decode's side table, derived on the device -> (resid_bit
        torch.int64 (n_meshlets,): the stream bit of each meshlet's anchor,
        sub_offs torch.int16 (n_meshlets, 5): dy dz px py pz starts after
        it, as uint16 bit patterns).  The reference GPU harness reads this
        table from encoder-written files instead."""
        torch = _torch()
        dev = torch.device("cuda", torch.cuda.current_device())
        resid = torch.empty(self.n_meshlets, dtype=torch.int64, device=dev)
        subs = torch.empty((self.n_meshlets, 5), dtype=torch.int16, device=dev)
        _lib.check(self._lib.stride_side_table(self._h, ctypes.c_void_p(_stream_handle(stream)),
                                               ctypes.c_void_p(resid.data_ptr()), ctypes.c_void_p(subs.data_ptr())),
                   "stride_side_table")
        return resid, subs

    def decode_to_device(self, *, stream=None, check: bool = True):
        """-> (triangles torch.uint32 (n_t, 3), positions torch.float32 (n_v, 3))
        in world space, resident on the GPU.  The tensors are reused by later
        calls, like the reference's output arrays (:686-690)."""
        tris, verts = self._outputs()
        self.decode_into(tris, verts, stream=stream, check=check)
        return tris, verts

    def decode(self, *, stream=None, check: bool = True, normalised: bool = False):
        """Reference order: -> (positions (n_v, 3) float32, triangles (n_t, 3))
        as CUDA tensors.  By default world-space positions and uint32
        triangles; ``normalised=True`` returns what the reference's decode()
        returns (:686-712): positions before ``* scale + center`` --
        float32(g_min + q / (2^g_bits - 1) * g_range), the float64 expression
        of decode_dup (encoder/paradelta_v5_dup.py:607-616) -- kept in
        ``d_verts_norm``, and the triangles as int32."""
        if not normalised:
            tris, verts = self.decode_to_device(stream=stream, check=check)
            return verts, tris
        torch = _torch()
        tris, verts = self._outputs()
        codes = torch.empty((self.n_v_total, 3), dtype=torch.int32, device=verts.device)
        self.decode_into(tris, verts, codes=codes, stream=stream, check=check)
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            vn = torch.empty((self.n_v_total, 3), dtype=torch.float64, device=verts.device)
            for d in range(3):
                gmin, grange, bits = float(self.info.g_min[d]), float(self.info.g_range[d]), int(self.g_bits[d])
                if bits == 0:
                    vn[:, d] = gmin
                else:
                    # one operation per step, in decode_dup's order, each rounded in float64
                    vn[:, d] = (codes[:, d].double() / float((1 << bits) - 1)) * grange + gmin
            self.d_verts_norm = vn.float()
        return self.d_verts_norm, tris.view(torch.int32)

    def decode_to_host(self, out=None, *, stream=None):
        """-> (positions np.float32 (n_v, 3), triangles np.uint32 (n_t, 3)),
        copied to host memory (reference :714-718).  ``out`` may supply the two
        host arrays (pinned memory makes the copies asynchronous)."""
        if out is None:
            pos = np.empty((self.n_v_total, 3), np.float32)
            idx = np.empty((self.n_t_total, 3), np.uint32)
        else:
            pos, idx = out
        rc = self._lib.stride_decode_host(self._h, ctypes.c_void_p(_stream_handle(stream)),
                                          ctypes.c_void_p(idx.ctypes.data), ctypes.c_void_p(pos.ctypes.data))
        _lib.check(rc, "stride_decode_host")
        return pos, idx

    def reload(self, data: bytes, *, stream=None):
        """Swap in a new stream (device buffers are reused when large enough)."""
        self._data = bytes(data)
        rc = self._lib.stride_reload(self._h, self._data, len(self._data), ctypes.c_void_p(_stream_handle(stream)))
        _lib.check(rc, "stride_reload")
        info = _lib.StrideInfo()
        _lib.check(self._lib.stride_info(self._h, ctypes.byref(info)), "stride_info")
        self.info = info
        self.n_meshlets = int(info.n_meshlets)
        if int(info.n_v) != self.n_v_total or int(info.n_t) != self.n_t_total:
            self.d_verts = self.d_tris = None
        self.n_v_total = int(info.n_v)
        self.n_t_total = int(info.n_t)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.stride_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def decode_to_device(data: bytes):
    """One-shot helper: -> (triangles torch.uint32, positions torch.float32)."""
    dec = ParaDeltaV5GpuDecoder(data)
    tris, verts = dec.decode_to_device()
    return tris.clone(), verts.clone()


def cull_meshlets(bounds, planes, *, stream=None):
    """Frustum culling of meshlet bounds (CUDA float32 (n, 6), as
    meshlet_bounds returns) against six planes (24 numbers: a b c d per
    plane, inside where a x + b y + c z + d >= 0) -> (visible bits
    torch.int32 (ceil(n / 32),), visible count torch.int32 (1,)), on the
    device.  A meshlet is culled when its box lies wholly outside a plane."""
    torch = _torch()
    assert bounds.is_cuda and bounds.dtype == torch.float32 and bounds.is_contiguous() and bounds.shape[-1] == 6
    n = bounds.shape[0]
    pl = np.ascontiguousarray(np.asarray(planes, np.float32).reshape(24))
    vis = torch.empty(max(1, (n + 31) // 32), dtype=torch.int32, device=bounds.device)
    cnt = torch.empty(1, dtype=torch.int32, device=bounds.device)
    lib = _lib.load()
    _lib.check(lib.stride_cull_meshlets(ctypes.c_void_p(bounds.data_ptr()), n, ctypes.c_void_p(pl.ctypes.data),
                                        ctypes.c_void_p(_stream_handle(stream)), ctypes.c_void_p(vis.data_ptr()),
                                        ctypes.c_void_p(cnt.data_ptr())), "stride_cull_meshlets")
    return vis, cnt
