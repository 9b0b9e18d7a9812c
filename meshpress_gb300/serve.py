"""Continuous-batching decode server (C ABI ``stride_server_*``).

The reference has no serving path: every ``ParaDeltaV5GpuDecoder`` decodes
one stream when called (utils/paradelta_v5_cuda.py:686-712).  This server
accepts encoded blobs from any thread, keeps their payloads and results in
one device arena of a fixed HBM budget, and a native scheduler thread packs
whatever is queued into batched launches on several streams, so requests
arriving while others decode are admitted as memory and streams free up.

Results stay on the device until released; ``wait`` returns views of them
as torch tensors (no copy) plus the request's timestamps.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib


class _DeviceArray:
    """Borrowed device memory exposed through the CUDA array interface."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2, "strides": None}


@dataclass
class ServedResult:
    req_id: int
    status: int
    n_v: int
    n_t: int
    tris: object        # torch.uint32 (n_t, 3) view into the arena, or None on error
    verts: object       # torch.float32 (n_v, 3) view into the arena, or None on error
    host_tris: object   # np.uint32 (n_t, 3) view of pinned memory (copy_to_host), else None
    host_verts: object
    t_submit_us: float
    t_admit_us: float
    t_done_us: float

    @property
    def latency_ms(self) -> float:
        return (self.t_done_us - self.t_submit_us) / 1e3

    @property
    def ok(self) -> bool:
        return self.status == _lib.STRIDE_OK


class DecodeServer:
    def __init__(self, hbm_budget_bytes: int, *, max_batch: int = 256, n_streams: int = 2, max_queue: int = 0,
                 copy_to_host: bool = False, pinned_budget_bytes: int = 0):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("CUDA device not available: the STRIDE decoder runs on the GPU only")
        torch.cuda.init()
        self._lib = _lib.load()
        self._device = torch.cuda.current_device()
        opts = _lib.ServerOpts(int(hbm_budget_bytes), int(max_batch), int(n_streams), int(max_queue),
                               int(bool(copy_to_host)), 0, int(pinned_budget_bytes))
        h = ctypes.c_void_p()
        _lib.check(self._lib.stride_server_create(ctypes.byref(opts), ctypes.byref(h)), "stride_server_create")
        self._h = h
        self.copy_to_host = bool(copy_to_host)

    def submit(self, data: bytes) -> int:
        rid = ctypes.c_uint64()
        data = bytes(data)
        _lib.check(self._lib.stride_server_submit(self._h, data, len(data), ctypes.byref(rid)), "submit")
        return int(rid.value)

    def wait(self, req_id: int, timeout_ms: int = -1) -> ServedResult:
        import torch
        r = _lib.ServerResult()
        _lib.check(self._lib.stride_server_wait(self._h, int(req_id), int(timeout_ms), ctypes.byref(r)), "wait")
        n_v, n_t = int(r.n_v), int(r.n_t)
        tris = verts = htris = hverts = None
        if r.status == _lib.STRIDE_OK:
            dev = f"cuda:{self._device}"
            if n_t and r.d_idx:
                tris = torch.as_tensor(_DeviceArray(r.d_idx, (n_t, 3), "<i4"), device=dev).view(torch.uint32)
            else:
                tris = torch.empty((0, 3), dtype=torch.uint32, device=dev)
            if n_v and r.d_pos:
                verts = torch.as_tensor(_DeviceArray(r.d_pos, (n_v, 3), "<f4"), device=dev)
            else:
                verts = torch.empty((0, 3), dtype=torch.float32, device=dev)
            if r.h_idx and n_t:
                htris = np.ctypeslib.as_array(ctypes.cast(r.h_idx, ctypes.POINTER(ctypes.c_uint32)),
                                              shape=(n_t, 3))
            if r.h_pos and n_v:
                hverts = np.ctypeslib.as_array(ctypes.cast(r.h_pos, ctypes.POINTER(ctypes.c_float)),
                                               shape=(n_v, 3))
        return ServedResult(int(req_id), int(r.status), n_v, n_t, tris, verts, htris, hverts,
                            float(r.t_submit_us), float(r.t_admit_us), float(r.t_done_us))

    def release(self, req_id: int):
        """Free the request's results (views from ``wait`` become invalid)."""
        _lib.check(self._lib.stride_server_release(self._h, int(req_id)), "release")

    def hold(self, on: bool = True):
        """Queue submissions without launching them until ``hold(False)``."""
        _lib.check(self._lib.stride_server_hold(self._h, int(bool(on))), "hold")

    def stats(self) -> dict:
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(self._lib.stride_server_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"launches": int(a.value), "completed": int(b.value), "arena_peak_bytes": int(c.value)}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.stride_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
