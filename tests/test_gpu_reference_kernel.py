"""The reference's own CUDA decoders on this GPU, next to this repository's.

DPR4: bench_cpp/stride_dup_decode_bench.cu on the same DPR4 streams, its
side table derived from the bytes; its triangles must equal decode_dup's,
its positions are not bit-exact by design (fp32 dequantisation).  PLDT v5:
bench_cpp/stride_decode_bench.cu:171 fed from the SBLB file, against
decode_paradelta_v5.  The timing record of both kernels on the 2049 x 2049
heightfield is written by oracle/time_reference_gpu.py; here it runs on a
small grid."""
import json

import numpy as np
import pytest

import oracle
from oracle import ref_gpu
from meshpress_gb300 import encoder, synth
from tests import _golden

pytestmark = pytest.mark.gpu

B12 = synth.bbox_bits_error(12)


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not ref_gpu.available():
        pytest.skip("reference kernel not built (needs the reference tree at build time)")
    from meshpress_gb300 import _build
    _build.build_decoder()
    oracle.build()
    return torch


def _run_ref(torch, data):
    k = ref_gpu.RefKernel(data)
    s = torch.cuda.Stream()
    k.launch(s)
    s.synchronize()
    return k


@pytest.mark.parametrize("name", ["grid129_b12", "ico3_b12", "grid65_world"])
def test_reference_kernel_on_reference_encoded_streams(torch_cuda, name):
    """Streams written by the reference encoder (golden fixtures)."""
    torch = torch_cuda
    g = _golden.load(name)
    k = _run_ref(torch, g["data"])
    opos, oidx = oracle.decode(g["data"])
    tris = k.tris.cpu().numpy().view(np.uint32).astype(np.int64)
    assert np.array_equal(tris, oidx)
    pos = k.verts.cpu().numpy()
    assert np.max(np.abs(pos - opos)) < 1e-3  # fp32 dequantisation: close, not exact
    k.close()


def test_reference_timing_record_on_a_small_grid(torch_cuda):
    """The timing script that writes the committed record of both reference
    GPU kernels beside this repository's decoders, on a 257 x 257 grid."""
    if not ref_gpu.available_v5():
        pytest.skip("reference PLDT v5 kernel not built")
    from oracle import time_reference_gpu
    rec = time_reference_gpu.run(grid=257, reps=3, sample_clocks=False)
    json.dumps(rec)
    assert rec["triangles"] == 2 * 256 * 256
    for fmt in ("dpr4", "pldt5"):
        ref, ours = rec[fmt]["reference_kernel"], rec[fmt]["this_decoder"]
        assert ref["triangles_exact"] and ours["triangles_exact"]
        assert ours["positions_bit_exact_frac"] == 1.0
        assert ref["ms_mean"] > 0 and ours["ms_mean"] > 0
        assert ref["positions_max_abs_err"] < 1e-2


V5_FIXTURES = ["v5_grid33_b12", "v5_grid65_world", "v5_ico5_b14", "v5_noise129_mv128", "v5_torus_b10",
               "v5_tri1_b12", "v5_noise33_b16"]


@pytest.mark.parametrize("name", V5_FIXTURES)
def test_reference_pldt5_kernel_on_reference_encoded_streams(torch_cuda, name):
    """The reference PLDT v5 kernel (bench_cpp/stride_decode_bench.cu:171)
    run from the SBLB file of a reference-encoded stream: its triangles equal
    decode_paradelta_v5's; its positions (float32 prediction) come close."""
    if not ref_gpu.available_v5():
        pytest.skip("reference PLDT v5 kernel not built")
    torch = torch_cuda
    data = _golden.load(name)["data"]
    k = ref_gpu.RefPldt5Kernel(ref_gpu.sblb_blob(data))
    s = torch.cuda.Stream()
    k.launch(s)
    s.synchronize()
    opos, oidx = oracle.decode_v5(data)
    tris = k.tris.cpu().numpy()[:k.n_t].view(np.uint32).astype(np.int64)
    assert np.array_equal(tris, oidx)
    pos = ref_gpu.world_rows_v5(k.verts.cpu().numpy()[:k.n_v], data)
    ext = float(np.max(np.ptp(opos, axis=0))) if len(opos) else 1.0
    assert np.max(np.abs(pos - opos)) <= 1e-3 * max(ext, 1.0)  # float32 prediction: close, not exact
    k.close()
