"""PLDT v5 streams on the GPU (``ParaDeltaV5GpuDecoder`` with the reference
class's own format, csrc/pldt5.cu) against the golden vectors of the
reference decoder ``decode_paradelta_v5`` (encoder/paradelta_v5.py:286-462)
and the C oracle."""
import glob
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
# encoded meshes (v5_*) and crafted corner cases (v5x_*)
V5_CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, "golden", "v5*_*.npz")))


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshpress_gb300 import _build
    _build.build_decoder()
    oracle.build()
    return torch


def _load(name):
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    return z["blob"].tobytes(), z["pos"], z["idx"]


def _gpu(data):
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    dec = ParaDeltaV5GpuDecoder(data)
    try:
        pos, idx = dec.decode_to_host()
    finally:
        dec.close()
    return pos, idx


@pytest.mark.parametrize("name", V5_CASES)
def test_matches_reference_decoder(torch_cuda, name):
    from meshpress_gb300 import ParaDeltaV5GpuDecoder, PldtV5Decoder
    data, pos, idx = _load(name)
    dec = ParaDeltaV5GpuDecoder(data)
    assert isinstance(dec, PldtV5Decoder)
    assert dec.n_v_total == len(pos) and dec.n_t_total == len(idx)
    gpos, gidx = dec.decode_to_host()
    assert np.array_equal(gpos.view(np.uint32), pos.view(np.uint32))  # bit-exact float32
    assert np.array_equal(gidx.astype(np.int64), idx)
    # a second decode into the same outputs gives the same rows
    tris, verts = dec.decode_to_device()
    assert np.array_equal(verts.cpu().numpy().view(np.uint32), pos.view(np.uint32))
    dec.close()


def test_dpr4_streams_still_take_the_stride_decoder(torch_cuda):
    from meshpress_gb300 import ParaDeltaV5GpuDecoder, PldtV5Decoder
    from tests import _golden
    dec = ParaDeltaV5GpuDecoder(_golden.load("grid33_b12")["data"])
    assert not isinstance(dec, PldtV5Decoder)
    dec.close()


def test_corrupt_streams_rejected_or_exact(torch_cuda):
    """Bit flips in the meshlet payloads and truncations: the GPU rejects every
    stream the oracle rejects, and otherwise matches it exactly (it may also
    reject streams the reference would decode, as documented)."""
    from meshpress_gb300._lib import StrideFormatError
    data, _, _ = _load("v5_grid33_mv64")
    h = oracle.parse_header_v5(data)
    body = (h.boundary_bit + 7) // 8 + 4 * h.n_meshlets + 64
    rng = np.random.default_rng(12)
    agree = rejected = 0
    cases = [data[:n] for n in (len(data) - 1, len(data) // 2, body)]
    for _ in range(40):
        b = bytearray(data)
        at = int(rng.integers(body, len(b)))
        b[at] ^= 1 << int(rng.integers(0, 8))
        cases.append(bytes(b))
    for c in cases:
        try:
            opos, oidx = oracle.decode_v5(c)
            ok = True
        except oracle.OracleError:
            ok = False
        try:
            gpos, gidx = _gpu(c)
        except StrideFormatError:
            rejected += 1
            continue
        assert ok, "the GPU accepted a stream the reference decoder rejects"
        assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32))
        assert np.array_equal(gidx.astype(np.int64), oidx)
        agree += 1
    assert rejected > 0


def test_project_encoder_stream_at_scale(torch_cuda):
    """A 131,072-triangle heightfield (1,348 meshlets of at most 128
    vertices) written by the project PLDT v5 encoder: the GPU decode equals
    the oracle's bit for bit."""
    from meshpress_gb300 import encoder, synth
    V, T = synth.noise_heightfield(257, seed=3)
    e = encoder.encode_pldt5(V, T, precision_error=synth.bbox_bits_error(12), precision_mode="bbox_frac",
                             max_verts=128, max_tris=128)
    opos, oidx = oracle.decode_v5(e.data)
    gpos, gidx = _gpu(e.data)
    assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(gidx.astype(np.int64), oidx)
