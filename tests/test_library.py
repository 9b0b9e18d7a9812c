"""The C-ABI library loads without a GPU, exports every entry point that
include/stride_gb300.h declares, and validates headers on the host."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle
from meshpress_gb300 import _build, _lib
from tests import _golden

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(REPO, "include", "stride_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z_][\w \*]*?\b((?:stride|pldt5)_\w+)\s*\(", text, flags=re.M)))


def test_library_builds_and_exports_every_declared_symbol(built_libs):
    names = declared_functions()
    assert len(names) >= 25
    lib = ctypes.CDLL(_build.decoder_library())
    for n in names:
        assert hasattr(lib, n), f"{n} declared but not exported"
    assert set(names) == {s[0] for s in _lib.SIGNATURES}


def test_inspect_matches_oracle_header(built_libs):
    for name in _golden.names():
        data = _golden.load(name)["data"]
        info = _lib.inspect(data)
        h = oracle.parse_header(data)
        assert info.n_meshlets == h.n_meshlets
        assert info.n_v == h.n_v_total and info.n_t == h.n_t
        assert list(info.g_bits) == list(h.g_bits)
        assert list(info.pred_n) == h.pred_n.reshape(-1).tolist()
        assert list(info.pred_k) == h.pred_k.tolist()


def test_inspect_rejects_bad_streams(built_libs):
    data = bytearray(_golden.load("grid33_b12")["data"])
    bad = bytearray(data)
    bad[0:4] = (0x504C4454).to_bytes(4, "big")  # a PLDT stream is not DPR4
    with pytest.raises(_lib.StrideFormatError) as e:
        _lib.inspect(bytes(bad))
    assert e.value.code == _lib.STRIDE_ERR_MAGIC
    bad = bytearray(data)
    bad[4] = 2
    with pytest.raises(_lib.StrideFormatError) as e:
        _lib.inspect(bytes(bad))
    assert e.value.code == _lib.STRIDE_ERR_VERSION
    with pytest.raises(_lib.StrideFormatError) as e:
        _lib.inspect(bytes(data[:50]))
    assert e.value.code == _lib.STRIDE_ERR_TRUNCATED
    with pytest.raises(_lib.StrideFormatError) as e:
        _lib.inspect(bytes(data[:90]))  # offset table cut short
    assert e.value.code == _lib.STRIDE_ERR_TRUNCATED
    bad = bytearray(data)
    bad[50] = 30  # 30-bit codes
    with pytest.raises(_lib.StrideFormatError) as e:
        _lib.inspect(bytes(bad))
    assert e.value.code == _lib.STRIDE_ERR_UNSUPPORTED


def test_decoder_fails_loudly_without_library(monkeypatch):
    monkeypatch.setattr(_build, "DECODER_LIB", "/nonexistent/libstride_gb300.so")
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError):
        _lib.load()


def test_kernel_count(built_libs):
    """The default launch shape follows the meshlet count: below 128 groups
    of 32 meshlets and from 1,024 on, two kernel launches (scan, which also
    fills any per-code dequantisation tables, then the fused connectivity +
    vertex kernel); in between three (scan, connectivity, vertices)."""
    for name in ("grid129_b12", "grid9_b12", "grid17_canon_b16", "tri1_b12"):
        assert _lib.inspect(_golden.load(name)["data"]).kernels == 2
    from meshpress_gb300 import encoder, synth
    V, T = synth.noise_heightfield(1025, seed=3)  # 331 groups
    data = encoder.encode(V, T, precision_error=synth.bbox_bits_error(12), precision_mode="bbox_frac").data
    info = _lib.inspect(data)
    assert 128 * 32 <= info.n_meshlets < 1024 * 32
    assert info.kernels == 3


def test_global_reads_through_l2_only():
    """The serving engine rewrites arena ranges (streams, mesh tables,
    dequantisation tables) for a new launch while launches on other streams
    still run on the same SMs, so the library is built with every plain
    global load cached in L2 only, and its kernels read no global data
    through L1 or the read-only cache."""
    assert "-dlcm=cg" in _build.NVCC_FLAGS
    for name in os.listdir(_build.CSRC):
        if name.endswith((".cu", ".cuh")):
            src = open(os.path.join(_build.CSRC, name)).read()
            for op in ("__ldg(", "__ldca(", "ld.global.ca", "ld.global.nc"):
                assert op not in src, f"{name} reads global memory with {op}"
