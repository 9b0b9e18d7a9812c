"""The CPU oracle (a C restatement of the reference decode_dup) against the
golden vectors produced by the reference itself."""
import json

import numpy as np
import pytest

import oracle
from tests import _golden


@pytest.mark.parametrize("name", _golden.names())
def test_oracle_matches_reference_decode(name):
    g = _golden.load(name)
    pos, idx, codes = oracle.decode(g["data"], with_codes=True)
    _golden.check_against(g, pos, idx, codes)


@pytest.mark.parametrize("name", _golden.names())
def test_oracle_meshlet_parallel_equals_sequential(name):
    g = _golden.load(name)
    pos, idx = oracle.decode(g["data"])
    p2, i2 = oracle.decode_mt(g["data"], 3)
    assert np.array_equal(p2.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(i2, idx)


def test_bitcodec_known_answers():
    z = np.load(_golden.GOLDEN + "/bitcodec.npz")
    ops = json.loads(str(z["ops"]))
    vals = oracle.bitcodec_read(z["blob"].tobytes(), [(o[0], o[1]) for o in ops])
    assert vals == [o[2] for o in ops]


def test_oracle_errors():
    g = _golden.load("grid33_b12")
    data = bytearray(g["data"])
    bad = bytes(data[:2]) + b"\x00\x00" + bytes(data[4:])
    with pytest.raises(oracle.OracleError):
        oracle.decode(bad)
    v = bytearray(data)
    v[4] = 5
    with pytest.raises(oracle.OracleError):
        oracle.decode(bytes(v))
    with pytest.raises(oracle.OracleError):
        oracle.decode(bytes(data[: len(data) // 2]))


@pytest.mark.parametrize("name", ["grid129_b12", "ico3_b12", "torus_b10"])
def test_side_table_layout(name):
    """The reference GPU harness's side table, derived from the bytes: every
    substream starts after the anchor and the six (tag, k) bytes, in the
    order dy dz px py pz, and the residual part ends before the next meshlet."""
    g = _golden.load(name)
    st = oracle.side_table(g["data"])
    h = oracle.parse_header(g["data"])
    assert st["n_local"].sum() == h.n_v_total and st["n_tris"].sum() == h.n_t
    assert (st["resid_bit"] >= st["start_bit"] + 48).all()
    sub = st["sub_offs"].astype(np.int64)
    assert (sub[:, 0] >= int(h.g_bits.sum()) + 96).all()
    assert (np.diff(sub, axis=1) >= 0).all()
    assert (st["start_bit"][1:].astype(np.int64) >= st["resid_bit"][:-1].astype(np.int64) + sub[:-1, 4]).all()
    assert ((st["n_kind0"] >= 1) & (st["n_kind0"] <= st["n_local"])).all()


def test_dprb_blob_layout():
    """The reference GPU harness's input file written from DPR4 bytes: header
    fields, section sizes and tables where its loader reads them."""
    import struct

    from oracle import ref_gpu
    g = _golden.load("grid129_b12")
    blob = ref_gpu.dprb_blob(g["data"])
    h = oracle.parse_header(g["data"])
    st = oracle.side_table(g["data"])
    M = h.n_meshlets
    magic, ver, m, nv, nt, buf_size = struct.unpack_from("<IIIIII", blob, 0)
    assert (magic, ver, m, nv, nt) == (0x42525044, 4, M, h.n_v_total, h.n_t)
    assert buf_size == len(g["data"]) - (86 + 4 * M)
    assert struct.unpack_from("<3I", blob, 76) == tuple(int(x) for x in h.g_bits)
    assert len(blob) == 112 + buf_size + M * (8 + 4 * 5 + 8 + 4 + 10)
    at = 112 + buf_size
    off = np.frombuffer(blob, "<u8", M, at)
    assert np.array_equal(off + (86 + 4 * M) * 8, st["start_bit"])
    at += 8 * M + 4 * 5 * M
    resid = np.frombuffer(blob, "<u8", M, at)
    assert np.array_equal(resid + (86 + 4 * M) * 8, st["resid_bit"])
    subs = np.frombuffer(blob, "<u2", 5 * M, at + 8 * M + 4 * M).reshape(M, 5)
    assert np.array_equal(subs, st["sub_offs"])
