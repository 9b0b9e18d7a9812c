"""The reference's own CUDA decoder (bench_cpp/stride_dup_decode_bench.cu)
on this GPU, next to this decoder: same DPR4 streams, side table derived
from the bytes.  Its triangles must equal decode_dup's; its positions are
not bit-exact by design (fp32 dequantisation), which this test measures.
The throughput comparison is printed as one JSON line (run with -s)."""
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


def test_reference_kernel_throughput_vs_ours(torch_cuda):
    torch = torch_cuda
    import bench
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    data, cfg = bench.heightfield_stream(2049, 12)
    k = _run_ref(torch, data)
    opos, oidx = oracle.decode_mt(data, 0)
    tris = k.tris.cpu().numpy().view(np.uint32).astype(np.int64)
    assert np.array_equal(tris, oidx)
    pos = k.verts.cpu().numpy()
    exact = float(np.mean(pos.view(np.uint32) == opos.view(np.uint32)))
    maxerr = float(np.max(np.abs(pos - opos)))
    dec = ParaDeltaV5GpuDecoder(data)
    t_ours, v_ours = dec.decode_to_device()
    s = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(fn, n=10, warm=3):
        ts = []
        for i in range(n + warm):
            with torch.cuda.stream(s):
                flush.fill_(i & 255)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                fn()
                e1.record(s)
            s.synchronize()
            if i >= warm:
                ts.append(e0.elapsed_time(e1))
        return float(np.mean(ts))

    ms_ref = timed(lambda: k.launch(s))
    ms_ours = timed(lambda: dec.decode_into(t_ours, v_ours, stream=s))
    n_t = int(oidx.shape[0])
    line = {"workload": "heightfield_2049x2049_12bit", "triangles": n_t,
            "reference_kernel": {"ms": round(ms_ref, 4), "M_tris_s": round(n_t / ms_ref / 1e3, 1),
                                 "triangles_exact": True, "positions_bit_exact_frac": round(exact, 4),
                                 "positions_max_abs_err": maxerr,
                                 "note": "stride_dup_decode_kernel, unmodified, side table from the bytes"},
            "this_decoder": {"ms": round(ms_ours, 4), "M_tris_s": round(n_t / ms_ours / 1e3, 1),
                             "bit_exact": True},
            "l2": "flushed before every decode"}
    print("REFERENCE_KERNEL " + json.dumps(line))
    assert ms_ours > 0 and ms_ref > 0
    k.close()
    dec.close()
