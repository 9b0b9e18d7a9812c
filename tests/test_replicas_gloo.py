"""Multi-process host logic of bench.py on CPU (gloo, world size 2).

The single-mesh workloads run one replica per rank; the batch workload
gives each rank its own share of the meshes (no exchange).  The job's step
time is the slowest rank's.  These tests run that host logic as two gloo
ranks.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import bench
    try:
        r, local, w = bench.dist_init("gloo")
        # each rank's mean step time; the job takes the slowest
        mine = 1.0 + rank  # ms
        worst = bench.reduce_max(mine)
        bench.barrier()
        value = bench.replica_value(1000, w, worst / 1e3)
        # the batch workload's path: each rank decodes its share of the meshes
        shard = bench.shard_batch(list(range(10)), r, w)
        got = [None] * w
        dist.all_gather_object(got, list(shard))
        q.put((rank, r, w, worst, value, got, bench.sharded_value(10, worst / 1e3)))
    finally:
        if dist.is_initialized():
            dist.destroy_process_group()


def test_two_ranks_max_and_aggregate():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r, w, worst, value, got, sharded in res:
        assert r == rank and w == world
        assert worst == 2.0  # max over ranks, seen by every rank
        assert value == pytest.approx(1000 * world / 2e-3)
        # the shares cover every mesh exactly once; the job's rate is every
        # mesh over the slowest rank's time
        flat = sorted(i for s in got for i in s)
        assert flat == list(range(10))
        assert sharded == pytest.approx(10 / 2e-3)


def test_shard_range_edges():
    sys.path.insert(0, REPO)
    import bench
    for n in (0, 1, 5, 4096):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                seen.extend(bench.shard_range(n, r, world))
            assert seen == list(range(n))


def test_reference_arm_non_zero_rank_prints_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "1", "--grid", "33"], env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""


def test_reference_arm_line_on_small_grid():
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "1", "--grid", "65"], env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["value"] == line["value"] > 0
    assert line["config"]["triangles"] == 2 * 64 * 64


def test_reference_arm_loads_no_product_library():
    """The reference arm reads the workload's stream from a file (made by a
    child process when missing) and times the CPU decoder: no library of
    this repository's product (encoder or GPU decoder) is loaded into it."""
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    code = ("import sys; sys.path.insert(0, %r); import bench; "
            "bench.main(['--impl', 'reference', '--steps', '1', '--warmup', '1', '--grid', '33']); "
            "print('MAPS', 'libstride_encode' in open('/proc/self/maps').read(), "
            "'libstride_gb300' in open('/proc/self/maps').read())" % REPO)
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    maps = [ln for ln in out.stdout.splitlines() if ln.startswith("MAPS")]
    assert maps == ["MAPS False False"]
