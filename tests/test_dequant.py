"""The decoder's exact-dequantisation routine (csrc/stride_dequant.h) equals
the reference float64 expression on every code of many random headers."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("dq") / "dq.so")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                    "-I", os.path.join(REPO, "meshpress_gb300", "csrc"),
                    os.path.join(HERE, "dequant_harness.c"), "-o", out, "-lm"], check=True)
    lib = ctypes.CDLL(out)
    lib.dq_check.restype = ctypes.c_int64
    lib.dq_check.argtypes = [ctypes.c_float] * 4 + [ctypes.c_uint32] * 3 + [ctypes.c_void_p,
                                                                             ctypes.POINTER(ctypes.c_int64)]
    return lib


def _reference(c, sc, gm, gr, gb, n):
    q = np.arange(n, dtype=np.int64)
    mx = (1 << gb) - 1
    if mx == 0:
        vn = np.full(n, float(gm))
    else:
        vn = float(gm) + q.astype(np.float64) / mx * float(gr)
    return (vn * float(sc) + float(c)).astype(np.float32)


def test_every_code_matches_float64_expression(harness):
    rng = np.random.default_rng(7)
    total = fast = 0
    for it in range(160):
        gb = int(rng.integers(0, 17)) if it % 8 else int(rng.integers(17, 25))
        c = np.float32(rng.normal(0, 10 ** rng.uniform(-3, 3))) if it % 5 else np.float32(0)
        sc = np.float32(10 ** rng.uniform(-3, 3))
        gm = np.float32(rng.uniform(-1, 0))
        gr = np.float32(rng.uniform(0.01, 2))
        n = min(1 << gb, 1 << 17)
        out = np.empty(n, np.float32)
        nf = ctypes.c_int64()
        bad = harness.dq_check(c, sc, gm, gr, gb, 0, n, out.ctypes.data, ctypes.byref(nf))
        assert bad == 0
        ref = _reference(c, sc, gm, gr, gb, n)
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
        total += n
        fast += nf.value
    assert fast / total > 0.99  # the float64 fallback stays rare


def test_headers_of_golden_streams(harness):
    import oracle
    from tests import _golden
    for name in _golden.names():
        h = oracle.parse_header(_golden.load(name)["data"])
        for d in range(3):
            gb = int(h.g_bits[d])
            n = 1 << gb if gb <= 16 else 1 << 16
            out = np.empty(n, np.float32)
            nf = ctypes.c_int64()
            bad = harness.dq_check(h.center[d], h.scale, h.g_min[d], h.g_range[d], gb, 0, n,
                                   out.ctypes.data, ctypes.byref(nf))
            assert bad == 0
            ref = _reference(h.center[d], h.scale, h.g_min[d], h.g_range[d], gb, n)
            assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
