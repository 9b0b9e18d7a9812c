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
