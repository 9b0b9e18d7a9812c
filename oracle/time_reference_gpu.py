"""Times the reference's own GPU decoders beside this repository's, on one GPU.

TEST INFRASTRUCTURE (run by hand on a GPU machine, and on a small grid by
tests/test_gpu_reference_kernel.py).  Two reference kernels, each compiled
unmodified from the reference sources into oracle/_ref (ref_gpu.build()):

- DPR4: bench_cpp/stride_dup_decode_bench.cu, stride_dup_decode_kernel (one
  warp per meshlet), on the DPR4 stream of the seeded heightfield, beside
  ParaDeltaV5GpuDecoder on the same stream;
- PLDT v5: bench_cpp/stride_decode_bench.cu:171, paradelta_v5_fused_decode
  (the kernel of the reference's CuPy decoder, utils/paradelta_v5_cuda.py),
  fed from the SBLB file that ref_gpu.sblb_blob writes for the PLDT v5
  stream of the same heightfield, beside PldtV5Decoder on that stream.

Every decode runs on one non-default stream after a 256 MiB write that
flushes L2, timed with CUDA events on that stream; SM clocks are sampled
with nvidia-smi while the timed loops run.  Exactness is measured against
the oracle: triangles equal or not, and the fraction of position words that
are bit-identical (the reference kernels dequantise in float32 by design).

    python oracle/time_reference_gpu.py [out.json] [--grid N] [--bits B] [--reps R]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _timed(torch, stream, fn, reps: int, warm: int = 3):
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ts = []
    for i in range(reps + warm):
        with torch.cuda.stream(stream):
            flush.fill_(i & 255)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
        stream.synchronize()
        if i >= warm:
            ts.append(e0.elapsed_time(e1))
    return {"ms_mean": round(float(np.mean(ts)), 4), "ms_min": round(float(np.min(ts)), 4), "reps": reps}


def _exactness(pos, tris, opos, oidx):
    pos = np.asarray(pos, np.float32).reshape(-1, 3)
    same_tris = bool(tris.shape == oidx.shape and np.array_equal(tris.astype(np.int64), oidx))
    if pos.shape != opos.shape:
        return {"triangles_exact": same_tris, "positions_bit_exact_frac": 0.0, "positions_max_abs_err": None}
    return {"triangles_exact": same_tris,
            "positions_bit_exact_frac": round(float(np.mean(pos.view(np.uint32) == opos.view(np.uint32))), 6),
            "positions_max_abs_err": float(np.max(np.abs(pos - opos))) if len(pos) else 0.0}


def run(grid: int = 2049, bits: int = 12, reps: int = 20, sample_clocks: bool = True) -> dict:
    sys.path.insert(0, REPO)
    import torch

    import bench
    import oracle
    from meshpress_gb300 import ParaDeltaV5GpuDecoder, encoder, synth
    from meshpress_gb300.pldt5 import PldtV5Decoder
    from oracle import ref_gpu

    if not (ref_gpu.available() and ref_gpu.available_v5()):
        raise RuntimeError("reference kernels not built (oracle/_ref)")
    oracle.build()
    stream = torch.cuda.Stream()
    V, T = synth.noise_heightfield(grid, seed=3)
    err = synth.bbox_bits_error(bits)
    dpr4 = encoder.encode(V, T, precision_error=err, precision_mode="bbox_frac").data
    v5 = encoder.encode_pldt5(V, T, precision_error=err, precision_mode="bbox_frac").data
    clocks = bench.ClockSampler(torch.cuda.current_device()) if sample_clocks else None
    rec = {"workload": f"heightfield_{grid}x{grid}_{bits}bit", "triangles": int(len(T)),
           "source_vertices": int(len(V)), "l2": "256 MiB write before every decode (untimed)",
           "timing": "CUDA events on the launching stream, mean over the timed decodes"}

    # DPR4: reference kernel (#5) and this decoder
    opos, oidx = oracle.decode_mt(dpr4, 0)
    k5 = ref_gpu.RefKernel(dpr4)
    dec = ParaDeltaV5GpuDecoder(dpr4)
    t_ours, v_ours = dec.decode_to_device()
    k5.launch(stream)
    stream.synchronize()
    if clocks:
        clocks.start()
    t5 = _timed(torch, stream, lambda: k5.launch(stream), reps)
    tours = _timed(torch, stream, lambda: dec.decode_into(t_ours, v_ours, stream=stream, check=False), reps)
    dec.check()
    ex5 = _exactness(k5.verts.cpu().numpy(), k5.tris.cpu().numpy().view(np.uint32), opos, oidx)
    exo = _exactness(v_ours.cpu().numpy(), t_ours.view(torch.int32).cpu().numpy().view(np.uint32), opos, oidx)
    rec["dpr4"] = {
        "stream_bytes": len(dpr4), "meshlets": int(k5.n_meshlets),
        "reference_kernel": {**t5, **ex5, "M_tris_s": round(len(T) / t5["ms_mean"] / 1e3, 1),
                             "what": "bench_cpp/stride_dup_decode_bench.cu stride_dup_decode_kernel, unmodified; "
                                     "grid min(meshlets, 16 x SMs) x 128 threads; side table from the bytes"},
        "this_decoder": {**tours, **exo, "M_tris_s": round(len(T) / tours["ms_mean"] / 1e3, 1),
                         "what": "ParaDeltaV5GpuDecoder.decode_into (scan + fused kernel)"}}
    k5.close()
    dec.close()
    del t_ours, v_ours

    # PLDT v5: reference kernel (#8) from the SBLB file, and this decoder
    opos5, oidx5 = oracle.decode_v5(v5)
    blob = ref_gpu.sblb_blob(v5)
    k8 = ref_gpu.RefPldt5Kernel(blob)
    p5 = PldtV5Decoder(v5)
    t5o, v5o = p5.decode_to_device()
    k8.launch(stream)
    stream.synchronize()
    t8 = _timed(torch, stream, lambda: k8.launch(stream), reps)
    t5ours = _timed(torch, stream, lambda: p5.decode_into(t5o, v5o, stream=stream, check=False), reps)
    if clocks:
        rec["clocks"] = clocks.stop()
    p5.check()
    world = ref_gpu.world_rows_v5(k8.verts.cpu().numpy()[:k8.n_v], v5)
    ex8 = _exactness(world, k8.tris.cpu().numpy()[:k8.n_t].view(np.uint32), opos5, oidx5)
    ex5o = _exactness(v5o.cpu().numpy(), t5o.view(torch.int32).cpu().numpy().view(np.uint32), opos5, oidx5)
    rec["pldt5"] = {
        "stream_bytes": len(v5), "meshlets": int(k8.n_meshlets), "boundary_vertices": int(k8.hdr["n_boundary"]),
        "vertices": int(k8.n_v),
        "reference_kernel": {**t8, **ex8, "M_tris_s": round(len(T) / t8["ms_mean"] / 1e3, 1),
                             "shared_bytes_header": k8.smem_header, "shared_bytes_launched": k8.smem,
                             "what": "bench_cpp/stride_decode_bench.cu:171 paradelta_v5_fused_decode<short>, "
                                     "unmodified, from the SBLB file; grid min(meshlets, 16 x SMs) x 32 threads; "
                                     "positions compared after the CuPy decoder's float32 v * scale + center"},
        "this_decoder": {**t5ours, **ex5o, "M_tris_s": round(len(T) / t5ours["ms_mean"] / 1e3, 1),
                         "what": "PldtV5Decoder.decode_into (csrc/pldt5.cu)"}}
    k8.close()
    p5.close()
    rec["gpu"] = torch.cuda.get_device_name()
    rec["command"] = "python oracle/time_reference_gpu.py" + (f" --grid {grid}" if grid != 2049 else "") + \
        (f" --bits {bits}" if bits != 12 else "")
    return rec


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("out", nargs="?", default=os.path.join(REPO, "profiles",
                                                           "reference_gpu_kernels_heightfield_2049_12bit.json"))
    ap.add_argument("--grid", type=int, default=2049)
    ap.add_argument("--bits", type=int, default=12)
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args(argv)
    rec = run(a.grid, a.bits, a.reps)
    with open(a.out, "w") as f:
        json.dump(rec, f, indent=1)
        f.write("\n")
    print(json.dumps(rec))
    return 0


if __name__ == "__main__":
    sys.exit(main())
