"""Project PLDT v5 encoder (csrc/encoder/stride_encode.cpp, pldt5_encode):
its streams decode with the oracle of the reference decoder (which the
golden vectors pin) to every source vertex exactly once, within the
quantisation bound, with the source triangles."""
import numpy as np
import pytest

import oracle
from meshpress_gb300 import encoder, synth

CASES = {
    "grid65_b12": (lambda: synth.heightfield_grid(65, seed=1), dict(precision_error=synth.bbox_bits_error(12),
                                                                     precision_mode="bbox_frac")),
    "ico5_b14": (lambda: synth.icosphere(5, seed=2), dict(precision_error=synth.bbox_bits_error(14),
                                                          precision_mode="bbox_frac")),
    "torus_world": (lambda: synth.torus(40, 20), dict(precision_error=0.0005, precision_mode="world")),
    "noise129_mv64": (lambda: synth.noise_heightfield(129, seed=3), dict(precision_error=synth.bbox_bits_error(16),
                                                                         precision_mode="bbox_frac", max_verts=64,
                                                                         max_tris=64)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_round_trip_through_the_oracle(name):
    make, kw = CASES[name]
    V, T = make()
    e = encoder.encode_pldt5(V, T, **kw)
    pos, idx = oracle.decode_v5(e.data)
    h = oracle.parse_header_v5(e.data)
    assert h.n_meshlets == e.n_meshlets and h.n_boundary == e.n_boundary
    # rows: every source vertex exactly once (boundary rows first)
    assert np.array_equal(np.sort(e.rows), np.arange(len(V)))
    # within half a quantisation step (per_coord_err, normalised) plus the f32 output rounding
    bound = float(h.per_coord_err) * float(h.scale) * (1 + 1e-6) + 4 * np.finfo(np.float32).eps * np.abs(V).max()
    assert np.abs(pos.astype(np.float64) - V[e.rows]).max() <= bound
    # the source triangles (as vertex sets; strips may reverse a triangle's winding)
    src = np.unique(np.sort(np.asarray(T, np.int64), axis=1), axis=0)
    dec = np.unique(np.sort(e.rows[idx].astype(np.int64), axis=1), axis=0)
    assert len(idx) == len(T) and np.array_equal(src, dec)


def test_deterministic():
    V, T = synth.icosphere(4, seed=5)
    a = encoder.encode_pldt5(V, T, precision_error=synth.bbox_bits_error(12), precision_mode="bbox_frac")
    b = encoder.encode_pldt5(V, T, precision_error=synth.bbox_bits_error(12), precision_mode="bbox_frac")
    assert a.data == b.data and np.array_equal(a.rows, b.rows)
