"""The reference's own CUDA decoder, run on this GPU as a baseline.

TEST INFRASTRUCTURE ONLY (used by tests/test_gpu_reference_kernel.py).
The reference ships a STRIDE decode-throughput harness,
bench_cpp/stride_dup_decode_bench.cu: one warp per meshlet, lane 0 parses
the connectivity, lanes 0-2 the three axes, lane 0 predicts, the warp
writes fp32 positions and uint32 indices.  Its kernel is not bit-exact by
design (fp32 dequantisation, int16 code storage) and it reads a side table
that is not in the DPR4 bytes (per-meshlet residual offsets and substream
sub-offsets, written by the reference's scripts/dump_stride_dup_blob.py
from encoder metadata).

build() compiles that kernel, unmodified, from the reference source into a
cubin (oracle/_ref/, git-ignored; it travels with the tree to machines
without the reference sources).  RefKernel loads the
cubin with the CUDA driver API, derives the side table from the DPR4 bytes
with the C oracle (so_side_table), and launches the kernel the way the
reference harness does (stride_dup_decode_bench.cu:662-685): a persistent
grid of min(n_meshlets, 16 x SMs) blocks of 128 threads, its work counter
zeroed before every launch.

The reference's PLDT v5 GPU harness, bench_cpp/stride_decode_bench.cu
(kernel paradelta_v5_fused_decode, :171; a verbatim copy of the CuPy
decoder's kernel in utils/paradelta_v5_cuda.py), is built the same way and
run by RefPldt5Kernel from the SBLB tables (sblb_blob) as the harness's
launch() does (:553-579): one 32-thread block per meshlet slot, a grid of
min(n_meshlets, 16 x SMs), per_warp_bytes of dynamic shared memory.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
CUBIN = os.path.join(REF_DIR, "stride_dup_decode.cubin")
ENTRY = os.path.join(REF_DIR, "stride_dup_decode.entry")
REFERENCE = os.environ.get("MESHPRESS_REFERENCE", "/root/reference")  # the reference checkout
REF_SRC = os.path.join(REFERENCE, "bench_cpp", "stride_dup_decode_bench.cu")
P5_CUBIN = os.path.join(REF_DIR, "stride_decode_v5.cubin")
P5_ENTRY = os.path.join(REF_DIR, "stride_decode_v5.entry")
P5_SRC = os.path.join(REFERENCE, "bench_cpp", "stride_decode_bench.cu")


def _compile(src: str, cubin: str, entry: str, pattern: str) -> None:
    """nvcc -cubin of one reference source, unmodified; the mangled names of
    the kernel entries matching `pattern` (from the ptxas report) go to `entry`."""
    os.makedirs(REF_DIR, exist_ok=True)
    r = subprocess.run(["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                        "-std=c++17", "-Xptxas", "-v", src, "-o", cubin + ".tmp"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference kernel build failed:\n{r.stderr}")
    names = sorted(set(re.findall(r"Compiling entry function '([^']*%s[^']*)'" % pattern, r.stdout + r.stderr)))
    if not names:
        raise RuntimeError("reference kernel entry name not found in the ptxas report")
    os.replace(cubin + ".tmp", cubin)
    with open(entry, "w") as f:
        f.write("\n".join(names) + "\n")


def _stale(src: str, cubin: str, entry: str) -> bool:
    return not os.path.exists(cubin) or not os.path.exists(entry) or os.path.getmtime(cubin) < os.path.getmtime(src)


def build(force: bool = False) -> bool:
    """Compile the reference kernels (DPR4 #5 and PLDT v5 #8) to sm_103a
    cubins when the reference tree is present; True when the DPR4 cubin
    exists."""
    if os.path.exists(REF_SRC) and (force or _stale(REF_SRC, CUBIN, ENTRY)):
        _compile(REF_SRC, CUBIN, ENTRY, "stride_dup_decode_kernel")
    if os.path.exists(P5_SRC) and (force or _stale(P5_SRC, P5_CUBIN, P5_ENTRY)):
        _compile(P5_SRC, P5_CUBIN, P5_ENTRY, "paradelta_v5_fused_decode")
    return os.path.exists(CUBIN) and os.path.exists(ENTRY)


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(ENTRY)


def available_v5() -> bool:
    return os.path.exists(P5_CUBIN) and os.path.exists(P5_ENTRY)


def dprb_blob(data: bytes) -> bytes:
    """The DPR4 stream as the reference GPU harness's input file (DPRB v4:
    a 112-byte little-endian header, the meshlet bits, then the per-meshlet
    tables; layout of scripts/dump_stride_dup_blob.py:121-156, read by
    bench_cpp/stride_dup_decode_bench.cu:527-596).  The side tables come
    from the bytes (so_side_table) instead of encoder metadata, so the file
    can be written for any stream."""
    import struct

    from . import oracle as orc
    h = orc.parse_header(data)
    st = orc.side_table(data)
    M = h.n_meshlets
    body_bit = (86 + 4 * M) * 8
    body = data[body_bit // 8:]
    n_local, n_tris = st["n_local"], st["n_tris"]
    v_off = np.concatenate([[0], np.cumsum(n_local[:-1], dtype=np.int64)]).astype(np.uint32)
    t_off = np.concatenate([[0], np.cumsum(n_tris[:-1], dtype=np.int64)]).astype(np.uint32)
    head = struct.pack("<II", 0x42525044, 4)
    head += struct.pack("<III", M, int(n_local.sum()), int(n_tris.sum()))
    head += struct.pack("<I", len(body)) + struct.pack("<II", 0, 0)
    head += struct.pack("<fff", *[float(x) for x in h.center]) + struct.pack("<f", h.scale)
    head += struct.pack("<f", h.per_coord_err)
    head += struct.pack("<fff", *[float(x) for x in h.g_min]) + struct.pack("<fff", *[float(x) for x in h.g_range])
    head += struct.pack("<III", *[int(x) for x in h.g_bits])
    head += struct.pack("<9h", *[int(x) for x in h.pred_n.reshape(9)]) + struct.pack("<3B", *[int(x) for x in h.pred_k])
    head += b"\x00\x00\x00"
    assert len(head) == 112
    parts = [head, body, (st["start_bit"] - body_bit).astype("<u8").tobytes(), n_local.astype("<u4").tobytes(),
             n_tris.astype("<u4").tobytes(), st["n_strips"].astype("<u4").tobytes(), v_off.astype("<u4").tobytes(),
             t_off.astype("<u4").tobytes(), (st["resid_bit"] - body_bit).astype("<u8").tobytes(),
             st["n_kind0"].astype("<u4").tobytes(), st["sub_offs"].astype("<u2").tobytes()]
    return b"".join(parts)


def sblb_blob(data: bytes, meshlets_per_block: int = 1) -> bytes:
    """A PLDT v5 stream as the reference PLDT v5 GPU harness's input file
    (SBLB v1: a 64-byte little-endian header, the stream, the per-meshlet
    tables, the float32 boundary rows; layout of scripts/dump_stride_blob.py:
    7-31 and 82-108, read by bench_cpp/stride_decode_bench.cu).  The
    reference takes the tables from its CuPy decoder
    (utils/paradelta_v5_cuda.py:515-684); here they come from the bytes
    (tables_v5), with the same per-warp shared-memory size (:662-678)."""
    import struct

    from . import oracle as orc
    h = orc.parse_header_v5(data)
    t = orc.tables_v5(data)
    M, nb = int(h.n_meshlets), int(h.n_boundary)
    n_bnd, n_int, n_tris, n_strips = t["n_bnd"], t["n_int"], t["n_tris"], t["n_strips"]
    tris_off = np.concatenate([[0], np.cumsum(n_tris, dtype=np.int64)]).astype(np.int32)
    int_cur = np.concatenate([[0], np.cumsum(n_int[:-1], dtype=np.int64)]).astype(np.int32)[:M]
    n_v_total = nb + int(n_int.sum())
    n_t_total = int(tris_off[-1])
    # parse_globals_v5 keeps the float64 boundary expression as float32 (:553-562)
    bnd_pos = t["bnd_rows"].astype(np.float32)
    code_bytes = 4 if h.code_width else 2
    mx = (lambda a: int(a.max()) if len(a) else 0)  # noqa: E731
    shared = (mx(n_bnd + n_int) * 16 + mx(n_bnd) * 4 + 32 + mx(n_int) * 3 * code_bytes + mx(n_int) * 8
              + mx(n_tris) * 3)
    per_warp = (shared + 15) & ~15
    delta = float(np.float32(2.0 * float(h.per_coord_err)))
    head = struct.pack("<IIIIIIIIffffIIII", 0x424C4253, 1, int(h.code_width), M, nb, n_v_total, n_t_total,
                       len(data), float(h.lin3_w[0]), float(h.lin3_w[1]), float(h.lin3_w[2]), delta, per_warp,
                       int(meshlets_per_block), 0, 0)
    assert len(head) == 64
    parts = [head, bytes(data), t["off_bits"].astype("<u8").tobytes(), n_bnd.astype("<i4").tobytes(),
             n_int.astype("<i4").tobytes(), n_tris.astype("<i4").tobytes(), n_strips.astype("<i4").tobytes(),
             tris_off.astype("<i4").tobytes(), int_cur.astype("<i4").tobytes(), bnd_pos.astype("<f4").tobytes()]
    return b"".join(parts)


_cuda = None


def _driver():
    global _cuda
    if _cuda is None:
        lib = ctypes.CDLL("libcuda.so.1")
        vp, u = ctypes.c_void_p, ctypes.c_uint
        lib.cuModuleLoadData.argtypes = [ctypes.POINTER(vp), vp]
        lib.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        lib.cuModuleUnload.argtypes = [vp]
        lib.cuLaunchKernel.argtypes = [vp, u, u, u, u, u, u, u, vp, vp, vp]
        _cuda = lib
    return _cuda


def _ck(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"{what}: CUDA driver error {rc}")


class RefKernel:
    """The reference kernel prepared for one DPR4 stream on the current
    torch device (torch owns the device memory and the stream)."""

    WARPS_PER_BLOCK = 4  # stride_dup_decode_bench.cu:190

    def __init__(self, data: bytes):
        import torch

        from . import oracle as orc
        if not available():
            raise RuntimeError("reference kernel not built (oracle/_ref)")
        h = orc.parse_header(data)
        st = orc.side_table(data)
        M = h.n_meshlets
        body_bit = (86 + 4 * M) * 8  # the offset table ends byte-aligned
        dev = torch.device("cuda", torch.cuda.current_device())
        body = np.frombuffer(data, np.uint8)[body_bit // 8:]
        # the reference's buffered reader prefetches up to 32 bytes past a
        # meshlet (stride_dup_decode_bench.cu:636-637): pad with zeros
        buf = np.zeros(len(body) + 32, np.uint8)
        buf[:len(body)] = body
        v_off = np.concatenate([[0], np.cumsum(st["n_local"][:-1], dtype=np.int64)]).astype(np.uint32)
        t_off = np.concatenate([[0], np.cumsum(st["n_tris"][:-1], dtype=np.int64)]).astype(np.uint32)

        def dput(a):
            return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).to(dev)

        self.d = {
            "buf": dput(buf),
            "off": dput((st["start_bit"] - body_bit).astype(np.uint64)),
            "n_local": dput(st["n_local"]), "n_tris": dput(st["n_tris"]), "n_strips": dput(st["n_strips"]),
            "v_off": dput(v_off), "t_off": dput(t_off),
            "resid": dput((st["resid_bit"] - body_bit).astype(np.uint64)),
            "n_kind0": dput(st["n_kind0"]), "axis": dput(st["sub_offs"]),
            "counter": torch.zeros(4, dtype=torch.uint8, device=dev),
        }
        self.n_v, self.n_t, self.n_meshlets = int(st["n_local"].sum()), int(st["n_tris"].sum()), M
        self.verts = torch.empty((self.n_v, 3), dtype=torch.float32, device=dev)
        self.tris = torch.empty((self.n_t, 3), dtype=torch.int32, device=dev)
        self.h = h
        drv = _driver()
        self._mod = ctypes.c_void_p()
        self._fn = ctypes.c_void_p()
        with open(CUBIN, "rb") as f:
            image = f.read()
        self._image = ctypes.create_string_buffer(image, len(image))
        _ck(drv.cuModuleLoadData(ctypes.byref(self._mod), ctypes.cast(self._image, ctypes.c_void_p)),
            "cuModuleLoadData")
        name = open(ENTRY).read().strip().encode()
        _ck(drv.cuModuleGetFunction(ctypes.byref(self._fn), self._mod, name), "cuModuleGetFunction")
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        self.grid = min(M, 16 * sms)
        self._params = self._pack()

    def _pack(self):
        h = self.h
        P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        vals = [P(self.d["buf"]), P(self.d["off"]), P(self.d["n_local"]), P(self.d["n_tris"]),
                P(self.d["n_strips"]), P(self.d["v_off"]), P(self.d["t_off"]), P(self.d["resid"]),
                P(self.d["n_kind0"]), P(self.d["axis"]), ctypes.c_int(self.n_meshlets)]
        vals += [ctypes.c_float(float(x)) for x in h.g_min]
        vals += [ctypes.c_float(float(x)) for x in h.g_range]
        vals += [ctypes.c_int(int(x)) for x in h.g_bits]
        vals += [ctypes.c_float(float(x)) for x in h.center] + [ctypes.c_float(float(h.scale))]
        for d in range(3):
            vals += [ctypes.c_int(int(h.pred_n[d, 0])), ctypes.c_int(int(h.pred_n[d, 1])),
                     ctypes.c_int(int(h.pred_n[d, 2])), ctypes.c_int(int(h.pred_k[d]))]
        vals += [P(self.verts), P(self.tris), P(self.d["counter"])]
        self._vals = vals
        arr = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        return arr

    def launch(self, stream) -> None:
        """One decode on `stream` (a torch.cuda.Stream), as the reference
        harness's launch(): zero the work counter, launch."""
        self.d["counter"].zero_()
        _ck(_driver().cuLaunchKernel(self._fn, self.grid, 1, 1, 32 * self.WARPS_PER_BLOCK, 1, 1, 0,
                                     ctypes.c_void_p(int(stream.cuda_stream)),
                                     ctypes.cast(self._params, ctypes.c_void_p), None),
            "cuLaunchKernel")

    def close(self):
        if self._mod:
            _driver().cuModuleUnload(self._mod)
            self._mod = ctypes.c_void_p()


def parse_sblb(blob: bytes) -> dict:
    """The SBLB v1 file back into the harness's buffers (read_blob,
    bench_cpp/stride_decode_bench.cu:455-486)."""
    import struct
    f = struct.unpack_from("<IIIIIIIIffffIIII", blob, 0)
    if f[0] != 0x424C4253 or f[1] != 1:
        raise ValueError("not an SBLB v1 file")
    keys = ("magic", "version", "code_width", "n_meshlets", "n_boundary", "n_v_total", "n_t_total", "buf_size",
            "lin3_w0", "lin3_w1", "lin3_w2", "delta", "per_warp_bytes", "meshlets_per_block")
    h = dict(zip(keys, f))
    M, nb, o = h["n_meshlets"], h["n_boundary"], 64
    out = {"hdr": h}

    def take(name, dtype, count):
        nonlocal o
        a = np.frombuffer(blob, dtype, count, o)
        o += a.nbytes
        out[name] = a

    take("buf", np.uint8, h["buf_size"])
    take("off_bits", "<u8", M)
    for k in ("n_bnd", "n_int", "n_tris", "n_strips"):
        take(k, "<i4", M)
    take("tris_off", "<i4", M + 1)
    take("int_cursor", "<i4", M)
    take("bnd_pos", "<f4", 3 * nb)
    if o != len(blob):
        raise ValueError("SBLB file size does not match its header")
    return out


def v5_kernel_smem(n_bnd, n_int, n_tris, code_bytes: int) -> int:
    """Bytes of dynamic shared memory the PLDT v5 kernel's per-meshlet layout
    (stride_decode_bench.cu:212-222) reaches for the largest meshlet: float4
    rows and an int l2g entry for every local vertex, the 256-bit seen map,
    the interior codes, four short emit arrays, the byte triangles."""
    n_local = np.asarray(n_bnd, np.int64) + np.asarray(n_int, np.int64)
    end = n_local * 20 + 32 + np.asarray(n_int, np.int64) * (3 * code_bytes + 8) + np.asarray(n_tris, np.int64) * 3
    return int(end.max()) if len(end) else 0


class RefPldt5Kernel:
    """The reference PLDT v5 kernel prepared from an SBLB file on the current
    torch device, launched as the harness's launch() does.  Two guards the
    harness does not have, so that the launch stays in bounds:
    the stream gets 64 zero bytes of padding (the kernel's bit reader loads
    five bytes from its position), and the dynamic shared memory is raised to
    the kernel's real per-meshlet layout when the SBLB header's
    per_warp_bytes -- the CuPy decoder's sizing, which counts l2g for the
    boundary vertices only (utils/paradelta_v5_cuda.py:658-665) while the
    kernel reserves it for every local vertex (:292-293) -- is smaller.
    Meshlets of more than 256 local vertices are refused (the seen map has
    256 bits)."""

    def __init__(self, blob: bytes):
        import torch
        if not available_v5():
            raise RuntimeError("reference PLDT v5 kernel not built (oracle/_ref)")
        B = parse_sblb(blob)
        h = B["hdr"]
        self.hdr = h
        n_local = B["n_bnd"].astype(np.int64) + B["n_int"]
        if len(n_local) and int(n_local.max()) > 256:
            raise ValueError("a meshlet has more than 256 local vertices")
        code_bytes = 4 if h["code_width"] else 2
        need = (v5_kernel_smem(B["n_bnd"], B["n_int"], B["n_tris"], code_bytes) + 15) & ~15
        self.smem_header = int(h["per_warp_bytes"])
        self.smem = max(self.smem_header, need)
        if self.smem > 227 * 1024:
            raise ValueError("per-meshlet shared memory above the 227 KB limit")
        dev = torch.device("cuda", torch.cuda.current_device())
        buf = np.zeros(len(B["buf"]) + 64, np.uint8)
        buf[:len(B["buf"])] = B["buf"]

        def dput(a):
            return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).to(dev)

        self.d = {"buf": dput(buf), "off": dput(B["off_bits"]), "n_bnd": dput(B["n_bnd"]),
                  "n_int": dput(B["n_int"]), "n_tris": dput(B["n_tris"]), "n_strips": dput(B["n_strips"]),
                  "tris_off": dput(B["tris_off"]), "int_cur": dput(B["int_cursor"]),
                  "bnd_pos": dput(B["bnd_pos"] if len(B["bnd_pos"]) else np.zeros(3, np.float32)),
                  "counter": torch.zeros(4, dtype=torch.uint8, device=dev)}
        self.n_v, self.n_t, self.n_meshlets = int(h["n_v_total"]), int(h["n_t_total"]), int(h["n_meshlets"])
        self.verts = torch.zeros((max(1, self.n_v), 3), dtype=torch.float32, device=dev)
        self.tris = torch.zeros((max(1, self.n_t), 3), dtype=torch.int32, device=dev)
        drv = _driver()
        self._mod = ctypes.c_void_p()
        self._fn = ctypes.c_void_p()
        with open(P5_CUBIN, "rb") as f:
            image = f.read()
        self._image = ctypes.create_string_buffer(image, len(image))
        _ck(drv.cuModuleLoadData(ctypes.byref(self._mod), ctypes.cast(self._image, ctypes.c_void_p)),
            "cuModuleLoadData")
        names = open(P5_ENTRY).read().split()
        # the <short> instantiation for 16-bit codes, <int> for 32-bit (:566, :575)
        want = "IiE" if h["code_width"] else "IsE"
        name = next((n for n in names if want in n), None)
        if name is None:
            raise RuntimeError("PLDT v5 kernel instantiation not found in the cubin's entries")
        _ck(drv.cuModuleGetFunction(ctypes.byref(self._fn), self._mod, name.encode()), "cuModuleGetFunction")
        if self.smem > 48 * 1024:
            drv.cuFuncSetAttribute.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
            _ck(drv.cuFuncSetAttribute(self._fn, 8, self.smem), "cuFuncSetAttribute")  # max dynamic smem
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        self.grid = min(self.n_meshlets, 16 * sms)
        P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        I, F = ctypes.c_int, ctypes.c_float  # noqa: E741
        self._vals = [P(self.d["buf"]), P(self.d["off"]), P(self.d["n_bnd"]), P(self.d["n_int"]),
                      P(self.d["n_tris"]), P(self.d["n_strips"]), P(self.d["tris_off"]), I(h["n_boundary"]),
                      P(self.d["int_cur"]), P(self.d["bnd_pos"]), I(h["n_boundary"]),
                      F(h["lin3_w0"]), F(h["lin3_w1"]), F(h["lin3_w2"]), F(h["delta"]),
                      P(self.verts), P(self.tris), I(self.n_meshlets), I(h["per_warp_bytes"]),
                      I(h["meshlets_per_block"]), P(self.d["counter"])]
        self._params = (ctypes.c_void_p * len(self._vals))(
            *[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in self._vals])

    def launch(self, stream) -> None:
        """One decode on `stream`: zero the work counter, launch (:553-579)."""
        if self.n_meshlets == 0:
            return
        with __import__("torch").cuda.stream(stream):
            self.d["counter"].zero_()
        _ck(_driver().cuLaunchKernel(self._fn, self.grid, 1, 1, 32, 1, 1, self.smem,
                                     ctypes.c_void_p(int(stream.cuda_stream)),
                                     ctypes.cast(self._params, ctypes.c_void_p), None),
            "cuLaunchKernel")

    def close(self):
        if self._mod:
            _driver().cuModuleUnload(self._mod)
            self._mod = ctypes.c_void_p()


def world_rows_v5(v_norm: np.ndarray, data: bytes) -> np.ndarray:
    """Normalised rows as world coordinates in float32, as the CuPy decoder's
    decode_to_host does (utils/paradelta_v5_cuda.py:714-718)."""
    from . import oracle as orc
    h = orc.parse_header_v5(data)
    return v_norm.astype(np.float32) * np.float32(h.scale) + np.asarray(list(h.center), np.float32)
