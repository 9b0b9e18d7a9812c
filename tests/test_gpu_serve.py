"""Continuous-batching server (stride_server_*): every response equals the
same stream decoded alone (bit-exact, no tolerance), whatever else was in
flight; admission respects the HBM budget; a bad request fails alone."""
import threading
import time

import numpy as np
import pytest

import oracle
from meshpress_gb300 import _lib, encoder, synth

pytestmark = pytest.mark.gpu

B12 = synth.bbox_bits_error(12)


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshpress_gb300 import _build
    _build.build_decoder()
    oracle.build()
    return torch


@pytest.fixture(scope="module")
def pool(torch_cuda):
    """Eighteen streams (200 .. 60 K triangles) with their alone-decodes."""
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    specs = synth.mixed_batch_specs(18, seed=17, t_min=200, t_max=6e4)
    out = []
    for kind, params in specs:
        V, T = synth.build_spec(kind, params)
        data = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data
        dec = ParaDeltaV5GpuDecoder(data)
        t, v = dec.decode_to_device()
        out.append((data, t.clone(), v.clone()))
        dec.close()
    return out


def _same(torch, res, t, v):
    assert res.ok, res.status
    assert torch.equal(res.tris.view(torch.int32), t.view(torch.int32))
    assert torch.equal(res.verts.view(torch.int32), v.view(torch.int32))


@pytest.mark.parametrize("pinned_budget", [0, 3 << 20], ids=["payloads_pinned", "pinned_and_staged"])
def test_alone_equals_mix(torch_cuda, pool, pinned_budget):
    """Every response equals the alone-decode, whether its payload was
    pinned at submit or staged by the scheduler (a 3 MiB pinned budget holds
    about three payloads at a time, so launches mix both kinds)."""
    torch = torch_cuda
    from meshpress_gb300.serve import DecodeServer
    # alone: one request in the server at a time
    with DecodeServer(256 << 20, n_streams=1, max_batch=1) as srv:
        for data, t, v in pool[:4]:
            rid = srv.submit(data)
            r = srv.wait(rid)
            _same(torch, r, t, v)
            srv.release(rid)
    # mix: three threads submit the pool twice over, interleaved; the first
    # half is queued behind a hold so that launches certainly share requests
    with DecodeServer(512 << 20, n_streams=3, max_batch=6, pinned_budget_bytes=pinned_budget) as srv:
        srv.hold(True)
        ids = {}
        lock = threading.Lock()

        def feed(k):
            for j in range(k, 2 * len(pool), 3):
                rid = srv.submit(pool[j % len(pool)][0])
                with lock:
                    ids[rid] = j % len(pool)
                time.sleep(0.0005 * (j % 4))
                if k == 0 and j >= len(pool):
                    srv.hold(False)

        th = [threading.Thread(target=feed, args=(k,)) for k in range(3)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        srv.hold(False)
        for rid, j in sorted(ids.items()):
            r = srv.wait(rid, timeout_ms=60000)
            _same(torch, r, pool[j][1], pool[j][2])
            assert r.t_submit_us <= r.t_admit_us <= r.t_done_us
            srv.release(rid)
        st = srv.stats()
        assert st["completed"] == 2 * len(pool)
        assert st["launches"] < 2 * len(pool)  # requests were batched together


def test_responses_match_oracle(torch_cuda, pool):
    from meshpress_gb300.serve import DecodeServer
    with DecodeServer(256 << 20, copy_to_host=True) as srv:
        ids = [(srv.submit(pool[j][0]), j) for j in (0, 5, 11)]
        for rid, j in ids:
            r = srv.wait(rid)
            assert r.ok
            opos, oidx = oracle.decode(pool[j][0])
            assert np.array_equal(r.host_tris.astype(np.int64), oidx)
            assert np.array_equal(r.host_verts.view(np.uint32), opos.view(np.uint32))
            srv.release(rid)


def test_budget_admission_and_peak(torch_cuda, pool):
    torch = torch_cuda
    from meshpress_gb300.serve import DecodeServer
    budget = 24 << 20
    with DecodeServer(budget, n_streams=2, max_batch=8) as srv:
        ids = [(srv.submit(data), j) for j, (data, _, _) in enumerate(pool)]
        for rid, j in ids:
            r = srv.wait(rid, timeout_ms=60000)
            _same(torch, r, pool[j][1], pool[j][2])
            srv.release(rid)  # frees arena space for the requests behind it
        assert srv.stats()["arena_peak_bytes"] <= budget
    # a request that cannot fit even alone is refused at submit
    V, T = synth.heightfield_grid(257, seed=8)  # 131,072 triangles: ~3 MB of outputs
    big = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data
    with DecodeServer(1 << 20) as srv:
        with pytest.raises(_lib.StrideDeviceError) as ei:
            srv.submit(big)
        assert ei.value.code == _lib.STRIDE_ERR_NOMEM


def test_bad_request_fails_alone(torch_cuda, pool):
    torch = torch_cuda
    from meshpress_gb300.serve import DecodeServer
    bad = pool[2][0][: len(pool[2][0]) - 64]  # truncated: offsets point past the end
    with DecodeServer(256 << 20, n_streams=1, max_batch=16) as srv:
        # hold the stream busy so the next requests queue up and share a launch
        first = srv.submit(pool[0][0])
        ids = [(srv.submit(pool[j][0]), j) for j in (1, 3, 4)]
        rb = srv.submit(bad)
        ids += [(srv.submit(pool[j][0]), j) for j in (5, 6)]
        r = srv.wait(rb, timeout_ms=60000)
        assert r.status in (_lib.STRIDE_ERR_OFFSET, _lib.STRIDE_ERR_CORRUPT, _lib.STRIDE_ERR_UNSUPPORTED)
        srv.release(rb)
        for rid, j in [(first, 0)] + ids:
            _same(torch, srv.wait(rid, timeout_ms=60000), pool[j][1], pool[j][2])
            srv.release(rid)


def test_queue_limit_and_errors(torch_cuda, pool):
    from meshpress_gb300.serve import DecodeServer
    with DecodeServer(64 << 20, max_queue=1, n_streams=1) as srv:
        with pytest.raises(_lib.StrideFormatError):
            srv.submit(b"\x00" * 200)  # bad magic, refused on the host
        rids = []
        busy = 0
        for _ in range(50):
            try:
                rids.append(srv.submit(pool[1][0]))
            except _lib.StrideDeviceError as e:
                assert e.code == _lib.STRIDE_ERR_BUSY
                busy += 1
        for rid in rids:
            assert srv.wait(rid, timeout_ms=60000).ok
            srv.release(rid)
        assert len(rids) >= 1
        with pytest.raises(_lib.StrideFormatError):
            srv.release(10 ** 9)  # unknown request


def test_bench_serve_passes(torch_cuda):
    """The bench's serve workload on a small pool: one Poisson pass and one
    burst pass, every response exact, the burst batching more than one
    request per launch."""
    import json
    import os
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    out = subprocess.run([sys.executable, os.path.join(repo, "bench.py"), "--workload", "serve", "--rates", "200",
                          "--serve-seconds", "0.5", "--serve-pool", "6", "--serve-burst", "64",
                          "--serve-host-rate", "0", "--serve-budget-gb", "4"],
                         env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(x) for x in out.stdout.splitlines() if x.startswith("{")]
    assert [x["config"]["workload"] for x in lines] == ["serve_poisson_200rps", "serve_burst64"]
    for x in lines:
        assert x["mismatched_responses"] == 0 and x["failed_responses"] == {}
        assert x["exact_responses"] == x["config"]["requests"]
        assert x["pool_bit_exact_vs_oracle"]
    assert lines[1]["mean_requests_per_launch"] > 2.0
