"""Project encoder: its streams decode (through the oracle) to its own integer
codes, to the source triangles, crack-free across meshlets."""
import os

import numpy as np
import pytest

import oracle
from meshpress_gb300 import encoder, synth
from tests import _meshes

B12 = synth.bbox_bits_error(12)

CASES = {
    "grid33_b12": (lambda: synth.heightfield_grid(33, seed=12), dict(precision_error=B12, precision_mode="bbox_frac")),
    "grid65_world": (lambda: synth.heightfield_grid(65, seed=2), dict(precision_error=0.0005)),
    "ico3_b12": (lambda: synth.icosphere(3, seed=3), dict(precision_error=B12, precision_mode="bbox_frac")),
    "ico4_b16_canon": (lambda: synth.icosphere(4, seed=4), dict(precision_error=synth.bbox_bits_error(16),
                                                               precision_mode="bbox_frac", predictor="canonical")),
    "torus_b10": (lambda: synth.torus(40, 17), dict(precision_error=synth.bbox_bits_error(10),
                                                    precision_mode="bbox_frac")),
    "grid129_b14": (lambda: synth.heightfield_grid(129, seed=1), dict(precision_error=synth.bbox_bits_error(14),
                                                                      precision_mode="bbox_frac")),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_encoder_roundtrip_through_oracle(name):
    make, kw = CASES[name]
    V, T = make()
    e = encoder.encode(V, T, **kw)
    pos, idx, codes = oracle.decode(e.data, with_codes=True)
    h = oracle.parse_header(e.data)
    assert h.n_v_total == e.n_v_dup == len(pos)
    assert h.n_t == len(T) == len(idx)
    assert np.array_equal(codes, e.codes.astype(np.int64))
    assert _meshes.same_triangle_set(T, idx, e.l2g)
    assert _meshes.crack_free(pos, e.l2g)
    if name.startswith(("ico", "torus")):
        assert _meshes.welded_is_closed_manifold(pos, idx)


def test_bbox_bits_give_requested_width():
    V, T = synth.heightfield_grid(65, seed=5)
    for b in (10, 12, 14, 16):
        e = encoder.encode(V, T, precision_error=synth.bbox_bits_error(b), precision_mode="bbox_frac")
        h = oracle.parse_header(e.data)
        assert int(h.g_bits.max()) == b


def test_encoder_rejects_bad_input():
    V, T = synth.heightfield_grid(9, seed=1)
    with pytest.raises(ValueError):
        encoder.encode(V, T + 1000)
    with pytest.raises(ValueError):
        encoder.encode(V, T, predictor="nope")


@pytest.mark.skipif(not os.path.isdir(os.path.join(os.environ.get("MESHPRESS_REFERENCE", "/root/reference"), "encoder")),
                    reason="reference checkout not present")
def test_reference_decoder_accepts_project_encoder_output():
    """The reference's own decode_dup reads the project encoder's bytes and
    returns what the oracle returns."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden
    _, _, decode_dup, _ = make_golden._import_reference()
    V, T = synth.icosphere(3, seed=9)
    e = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac")
    Vr, Tr = decode_dup(e.data)
    pos, idx = oracle.decode(e.data)
    assert np.array_equal(Vr.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(Tr, idx)
