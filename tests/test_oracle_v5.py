"""PLDT v5 oracle (oracle/pldt5_oracle.c) against golden vectors produced by
the reference itself (tests/golden/make_golden_v5.py: the reference encoder
``encode_from_prepared_v5`` and decoder ``decode_paradelta_v5``,
encoder/paradelta_v5.py:144-462)."""
import glob
import json
import os

import numpy as np
import pytest

import oracle
from tests import _golden

HERE = os.path.dirname(os.path.abspath(__file__))
# encoded meshes (v5_*) and crafted corner cases (v5x_*)
V5_CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "golden", "v5*_*.npz")))


def _load(name):
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    return z["blob"].tobytes(), z["pos"], z["idx"], json.loads(str(z["meta"]))


def test_fixtures_present():
    assert sum(c.startswith("v5_") for c in V5_CASES) >= 10 and sum(c.startswith("v5x_") for c in V5_CASES) >= 4


@pytest.mark.parametrize("name", V5_CASES)
def test_oracle_matches_reference_decoder(name):
    data, pos, idx, meta = _load(name)
    opos, oidx = oracle.decode_v5(data)
    assert opos.shape == pos.shape and oidx.shape == idx.shape
    assert np.array_equal(opos.view(np.uint32), pos.view(np.uint32))  # bit-exact float32
    assert np.array_equal(oidx, idx)
    h = oracle.parse_header_v5(data)
    assert h.n_meshlets == meta["n_meshlets"] and h.n_boundary == meta["n_boundary"]
    assert list(h.g_bits) == meta["g_bits"]
    if meta["kind"] == "pldt_v5":  # rows: the boundary vertices, then every meshlet's interior vertices
        assert len(opos) == meta["n_src_v"] and len(oidx) == meta["n_src_t"]


def test_rejects_other_formats_and_truncation():
    data, _, _, _ = _load("v5_grid33_b12")
    with pytest.raises(oracle.OracleError):
        oracle.decode_v5(_golden.load("grid33_b12")["data"])  # a DPR4 stream: bad magic
    bad = bytearray(data)
    bad[4] = 4  # version 4
    with pytest.raises(oracle.OracleError):
        oracle.decode_v5(bytes(bad))
    for cut in (3, 40, len(data) // 2, len(data) - 2):
        with pytest.raises(oracle.OracleError):
            oracle.decode_v5(data[:cut])


def test_sblb_blob_layout():
    """The reference PLDT v5 harness's input file written from the bytes
    (oracle.ref_gpu.sblb_blob; layout of scripts/dump_stride_blob.py)."""
    import struct

    from oracle import ref_gpu
    data, pos, idx, meta = _load("v5_noise129_mv128")
    blob = ref_gpu.sblb_blob(data)
    f = struct.unpack("<IIIIIIIIffffIIII", blob[:64])
    magic, version, code_width, M, nb, n_v, n_t, size = f[:8]
    assert (magic, version) == (0x424C4253, 1)
    assert M == meta["n_meshlets"] and nb == meta["n_boundary"]
    assert n_v == len(pos) and n_t == len(idx) and size == len(data)
    assert blob[64:64 + size] == data
    o = 64 + size
    off = np.frombuffer(blob, "<u8", M, o)
    o += 8 * M
    n_bnd, n_int, n_tris, n_strips = (np.frombuffer(blob, "<i4", M, o + 4 * M * i) for i in range(4))
    o += 16 * M
    tris_off = np.frombuffer(blob, "<i4", M + 1, o)
    o += 4 * (M + 1)
    int_cur = np.frombuffer(blob, "<i4", M, o)
    o += 4 * M
    bnd = np.frombuffer(blob, "<f4", 3 * nb, o).reshape(nb, 3)
    assert o + 12 * nb == len(blob)
    assert np.all(np.diff(off.astype(np.int64)) > 0) and tris_off[-1] == n_t
    assert nb + n_int.sum() == n_v and int_cur[-1] + n_int[-1] == n_v - nb
    # the boundary rows in world space are the decoder's first rows
    h = oracle.parse_header_v5(data)
    world = (bnd.astype(np.float64) * np.float32(h.scale) + np.array(h.center, np.float32)).astype(np.float32)
    assert np.abs(world - pos[:nb]).max() < 1e-5 * max(1.0, float(np.abs(pos).max()))


@pytest.mark.parametrize("name", V5_CASES)
def test_sblb_read_back_and_kernel_shared_memory(name):
    """The SBLB file parsed back the way the reference harness reads it
    (read_blob), and the shared memory the reference PLDT v5 kernel's
    per-meshlet layout reaches, which the launcher grants when the header's
    size (the CuPy decoder's formula) is smaller."""
    from oracle import ref_gpu
    data, pos, idx, meta = _load(name)
    B = ref_gpu.parse_sblb(ref_gpu.sblb_blob(data))
    h = B["hdr"]
    t = oracle.tables_v5(data)
    assert h["n_meshlets"] == meta["n_meshlets"] and h["n_boundary"] == meta["n_boundary"]
    assert h["n_v_total"] == len(pos) and h["n_t_total"] == len(idx)
    assert bytes(B["buf"]) == data
    for k in ("n_bnd", "n_int", "n_tris", "n_strips"):
        assert np.array_equal(B[k], t[k])
    cb = 4 if h["code_width"] else 2
    need = ref_gpu.v5_kernel_smem(B["n_bnd"], B["n_int"], B["n_tris"], cb)
    n_local = B["n_bnd"].astype(np.int64) + B["n_int"]
    # the kernel's layout: float4 rows and an l2g entry per local vertex,
    # the 256-bit seen map, interior codes, four short emit arrays, triangles
    want = int((n_local * 20 + 32 + B["n_int"].astype(np.int64) * (3 * cb + 8)
                + B["n_tris"].astype(np.int64) * 3).max()) if len(n_local) else 0
    assert need == want
    formula = ((int(n_local.max()) * 16 + int(B["n_bnd"].max()) * 4 + 32 + int(B["n_int"].max()) * 3 * cb
                + int(B["n_int"].max()) * 8 + int(B["n_tris"].max()) * 3 + 15) & ~15) if len(n_local) else 32
    assert h["per_warp_bytes"] == formula


@pytest.mark.parametrize("name", V5_CASES)
def test_host_inspect_matches_oracle(name):
    """pldt5_inspect (the library's host parse, no GPU): header fields and
    output sizes as the oracle decodes them."""
    from meshpress_gb300 import _lib
    data, pos, idx, meta = _load(name)
    info = _lib.inspect_pldt5(data)
    h = oracle.parse_header_v5(data)
    assert (info.n_meshlets, info.n_boundary) == (h.n_meshlets, h.n_boundary)
    assert list(info.g_bits) == list(h.g_bits) and info.nbytes == len(data)
    assert (info.n_v, info.n_t) == (len(pos), len(idx))
    assert info.scale == h.scale and list(info.lin3_w) == list(h.lin3_w)


def test_host_inspect_rejects():
    from meshpress_gb300 import _lib
    data, _, _, _ = _load("v5_grid33_mv64")
    with pytest.raises(_lib.StrideFormatError):
        _lib.inspect_pldt5(_golden.load("grid33_b12")["data"])  # DPR4 bytes
    bad = bytearray(data)
    bad[4] = 4
    with pytest.raises(_lib.StrideFormatError):
        _lib.inspect_pldt5(bytes(bad))
    for cut in (10, 60, 200):
        with pytest.raises(_lib.StrideFormatError):
            _lib.inspect_pldt5(data[:cut])
    # meshlet 1's offset equal to meshlet 0's: the table must increase
    h = oracle.parse_header_v5(data)
    t = oracle.tables_v5(data)
    table = int(t["off_bits"][0]) // 8 - 4 * h.n_meshlets  # the table ends where meshlet 0 starts
    bad = bytearray(data)
    bad[table + 4:table + 8] = bad[table:table + 4]
    with pytest.raises(_lib.StrideFormatError):
        _lib.inspect_pldt5(bytes(bad))


def test_host_inspect_rejects_a_boundary_count_the_bytes_cannot_hold():
    """A header claiming 2^31 boundary rows in a short stream is rejected
    before the host parse sizes any table from it (each row after the first
    takes at least three bits)."""
    from meshpress_gb300 import _lib
    data, _, _, _ = _load("v5_grid33_mv64")
    bad = bytearray(data)
    bad[61:65] = (0x7FFFFFFF).to_bytes(4, "big")  # n_boundary, after magic .. n_t (488 bits)
    with pytest.raises(_lib.StrideFormatError) as err:
        _lib.inspect_pldt5(bytes(bad))
    assert err.value.code == _lib.STRIDE_ERR_TRUNCATED
    h = oracle.parse_header_v5(data)
    assert int.from_bytes(data[61:65], "big") == h.n_boundary  # the field the test overwrote
