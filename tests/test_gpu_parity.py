"""GPU decode through the C ABI, bit-exact against the oracle and the golden
vectors of the reference decoder.

Parity bar: triangle indices equal, float32 positions bit-identical, integer
codes equal (exactness, no tolerance).
"""
import numpy as np
import pytest

import oracle
from meshpress_gb300 import _lib, encoder, synth
from tests import _golden, _meshes

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


def gpu_decode(torch, data, cfg=None, codes=True):
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    dec = ParaDeltaV5GpuDecoder(data)
    if cfg is not None:
        dec.set_launch_config(cfg)
    idx = torch.full((dec.n_t_total, 3), 0x7FFFFFFF, dtype=torch.int32, device="cuda")
    pos = torch.full((dec.n_v_total, 3), float("nan"), dtype=torch.float32, device="cuda")
    c = torch.full((dec.n_v_total, 3), -1, dtype=torch.int32, device="cuda") if codes else None
    dec.decode_into(idx, pos, codes=c)
    out = (pos.cpu().numpy(), idx.cpu().numpy().view(np.uint32))
    if codes:
        out = out + (c.cpu().numpy(),)
    dec.close()
    return out


def assert_same_as_oracle(data, pos, idx, codes=None):
    opos, oidx, ocodes = oracle.decode(data, with_codes=True)
    bad = np.nonzero(pos.view(np.uint32) != opos.view(np.uint32))[0]
    assert bad.size == 0, f"{bad.size} position rows differ (first {bad[:5]})"
    assert np.array_equal(idx.astype(np.int64), oidx)
    if codes is not None:
        assert np.array_equal(codes.astype(np.int64), ocodes)


@pytest.mark.parametrize("name", _golden.names())
def test_golden_vectors_bit_exact(torch_cuda, name):
    g = _golden.load(name)
    pos, idx, codes = gpu_decode(torch_cuda, g["data"])
    _golden.check_against(g, pos, idx, codes)


def test_decode_to_host_and_device_agree(torch_cuda):
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    g = _golden.load("grid129_b12")
    dec = ParaDeltaV5GpuDecoder(g["data"])
    pos, idx = dec.decode_to_host()
    assert pos.dtype == np.float32 and idx.dtype == np.uint32
    _golden.check_against(g, pos, idx)
    tris, verts = dec.decode_to_device()
    assert tris.dtype == torch_cuda.uint32 and verts.dtype == torch_cuda.float32
    assert np.array_equal(verts.cpu().numpy().view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(tris.view(torch_cuda.int32).cpu().numpy().view(np.uint32), idx)
    # repeated decodes reuse buffers and stay identical
    for _ in range(3):
        p2, i2 = dec.decode_to_host()
        assert np.array_equal(p2.view(np.uint32), pos.view(np.uint32)) and np.array_equal(i2, idx)


@pytest.mark.parametrize("grid", [513, 1449])
def test_decode_to_host_pinned_overlap(torch_cuda, grid):
    """Pinned host outputs: the index copy runs beside the vertex kernel on
    the handle's copy streams (from about 3 M triangles, 1449^2 here, part by
    part of the connectivity kernel, and after a reload part by part of the
    upload); results equal the device decode bit for bit."""
    torch = torch_cuda
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    V, T = synth.noise_heightfield(grid, seed=4)
    data = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data
    dec = ParaDeltaV5GpuDecoder(data)
    tris, verts = (x.clone() for x in dec.decode_to_device())
    h_pos = torch.empty((dec.n_v_total, 3), dtype=torch.float32, pin_memory=True)
    h_idx = torch.empty((dec.n_t_total, 3), dtype=torch.int32, pin_memory=True)
    for reload in (False, False, True, True):
        if reload:  # a large stream then goes up by parts, each decoded when its bytes are in
            dec.reload(data)
        h_pos.fill_(float("nan"))
        h_idx.fill_(-1)
        pos, idx = dec.decode_to_host(out=(h_pos.numpy(), h_idx.numpy().view(np.uint32)))
        assert np.array_equal(pos.view(np.uint32), verts.cpu().numpy().view(np.uint32))
        assert np.array_equal(idx, tris.view(torch.int32).cpu().numpy().view(np.uint32))
    # a device decode after such a reload waits for the whole upload
    dec.reload(data)
    t2, v2 = dec.decode_to_device()
    assert torch.equal(t2.view(torch.int32), tris.view(torch.int32))
    assert torch.equal(v2.view(torch.int32), verts.view(torch.int32))
    dec.close()


ENC_CASES = {
    "grid129_b12": (lambda: synth.heightfield_grid(129, seed=1), dict(precision_error=B12, precision_mode="bbox_frac")),
    "grid257_b10": (lambda: synth.noise_heightfield(257, seed=5), dict(precision_error=synth.bbox_bits_error(10),
                                                                      precision_mode="bbox_frac")),
    "grid257_b14": (lambda: synth.noise_heightfield(257, seed=5), dict(precision_error=synth.bbox_bits_error(14),
                                                                      precision_mode="bbox_frac")),
    "grid257_b16": (lambda: synth.noise_heightfield(257, seed=5), dict(precision_error=synth.bbox_bits_error(16),
                                                                      precision_mode="bbox_frac")),
    "grid129_b20_wide": (lambda: synth.heightfield_grid(129, seed=6),
                         dict(precision_error=synth.bbox_bits_error(20), precision_mode="bbox_frac")),
    "ico5_shuffled_b12": (lambda: synth.icosphere(5, seed=2), dict(precision_error=B12, precision_mode="bbox_frac")),
    "torus_b12_canon": (lambda: synth.torus(120, 45, R=4.0, r=1.0),
                        dict(precision_error=B12, precision_mode="bbox_frac", predictor="canonical")),
    "grid65_world": (lambda: synth.heightfield_grid(65, seed=2), dict(precision_error=0.0005)),
    "small_meshlets": (lambda: synth.icosphere(4, seed=8), dict(precision_error=B12, precision_mode="bbox_frac",
                                                               max_verts=40, max_tris=64)),
}


@pytest.mark.parametrize("name", sorted(ENC_CASES))
def test_encoded_meshes_match_oracle(torch_cuda, name):
    make, kw = ENC_CASES[name]
    V, T = make()
    e = encoder.encode(V, T, **kw)
    pos, idx, codes = gpu_decode(torch_cuda, e.data)
    assert_same_as_oracle(e.data, pos, idx, codes)
    assert np.array_equal(codes, e.codes)  # codes equal the encoder's input codes
    assert _meshes.same_triangle_set(T, idx.astype(np.int64), e.l2g)
    assert _meshes.crack_free(pos, e.l2g)
    if name.startswith(("ico", "torus", "small")):
        assert _meshes.welded_is_closed_manifold(pos, idx)


def _cfg(w, pers, stage, code, per_sm=0):
    c = _lib.LaunchCfg()
    c.warps_per_cta, c.persistent, c.ctas_per_sm, c.stage_bytes, c.code_bytes = w, pers, per_sm, stage, code
    return c


@pytest.mark.parametrize("cfg", [
    (1, 0, 20 * 1024, 16 * 1024), (2, 0, 16 * 1024, 8 * 1024), (4, 1, 12 * 1024, 6 * 1024),
    (1, 1, 256, 2048),           # tiny stage: meshlets fall back to global reads
    (2, 0, 64 * 1024, 516),      # code plane of one 256-vertex meshlet (odd word count): one per round
    (4, 2, 12 * 1024, 6 * 1024),  # fused connectivity + vertex kernel
    (4, 2, 256, 2048),           # fused, global reads
    (4, 2, 64 * 1024, 516),      # fused, one meshlet per round
    (2, 3, 0, 0),                # group kernel: one warp per group, two warps per CTA
    (1, 3, 0, 0),                # group kernel, one warp per CTA
], ids=["w1", "w2", "w4p", "global_reads", "one_per_round", "fused", "fused_global_reads",
        "fused_one_per_round", "group", "group_w1"])
def test_launch_shapes_give_identical_output(torch_cuda, cfg):
    V, T = synth.icosphere(5, seed=11)
    e = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac")
    pos, idx, codes = gpu_decode(torch_cuda, e.data, cfg=_cfg(*cfg))
    assert_same_as_oracle(e.data, pos, idx, codes)


@pytest.mark.parametrize("cfg", [(2, 1, 16 * 1024, 1028), (1, 0, 256, 32 * 1024), (4, 2, 16 * 1024, 1028),
                                 (2, 3, 0, 0)],
                         ids=["one_per_round", "global_reads", "fused_one_per_round", "group"])
def test_wide_codes_launch_shapes(torch_cuda, cfg):
    """20-bit codes (32-bit code plane) under the smallest plane and stage."""
    V, T = synth.heightfield_grid(129, seed=6)
    e = encoder.encode(V, T, precision_error=synth.bbox_bits_error(20), precision_mode="bbox_frac")
    pos, idx, codes = gpu_decode(torch_cuda, e.data, cfg=_cfg(*cfg))
    assert_same_as_oracle(e.data, pos, idx, codes)


@pytest.fixture(scope="module")
def large_heightfield():
    V, T = synth.noise_heightfield(2049, seed=3)
    e = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac")
    return e, oracle.decode_mt(e.data, 0)


@pytest.mark.parametrize("pers", [2, 1], ids=["fused", "two_kernels"])
def test_config_sweep_large_heightfield(torch_cuda, large_heightfield, pers):
    """2049 x 2049 heightfield (8,388,608 triangles) at 12 bits: full-size
    bit-exact decode against the oracle, with the fused kernel (default;
    1,347 groups take its five-CTA build) and with the two kernels."""
    e, (opos, oidx) = large_heightfield
    pos, idx, codes = gpu_decode(torch_cuda, e.data, cfg=_cfg(4, pers, 16 * 1024, 12 * 1024))
    assert np.array_equal(pos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(idx.astype(np.int64), oidx)
    assert np.array_equal(codes, e.codes)
    assert _meshes.crack_free(pos, e.l2g)


def test_icosphere_level8(torch_cuda):
    """Displaced, vertex-shuffled icosphere at level 8 (1,310,720 triangles)."""
    V, T = synth.icosphere(8, seed=2)
    e = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac")
    pos, idx, codes = gpu_decode(torch_cuda, e.data)
    opos, oidx = oracle.decode_mt(e.data, 0)
    assert np.array_equal(pos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(idx.astype(np.int64), oidx)
    assert _meshes.welded_is_closed_manifold(pos, idx)


# ---------------------------------------------------------------- errors ----

def test_rejects_bad_magic_and_version(torch_cuda):
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    data = bytearray(_golden.load("grid33_b12")["data"])
    bad = bytearray(data)
    bad[0:4] = (0x504C4454).to_bytes(4, "big")
    with pytest.raises(ValueError):
        ParaDeltaV5GpuDecoder(bytes(bad))
    bad = bytearray(data)
    bad[4] = 4
    with pytest.raises(ValueError):
        ParaDeltaV5GpuDecoder(bytes(bad))
    with pytest.raises(ValueError):
        ParaDeltaV5GpuDecoder(bytes(data), meshlets_per_block=17)


def _try_gpu(torch, data):
    try:
        return gpu_decode(torch, data, codes=False), None
    except _lib.StrideFormatError as e:
        return None, e


def _try_oracle(data):
    try:
        return oracle.decode(data), None
    except oracle.OracleError as e:
        return None, e


def test_truncated_and_offset_corruption(torch_cuda):
    g = _golden.load("grid129_b12")
    data = g["data"]
    r, e = _try_gpu(torch_cuda, data[: len(data) - 200])
    assert r is None and e is not None
    bad = bytearray(data)
    off = 86 + 4 * 5
    bad[off:off + 4] = (int.from_bytes(bad[off:off + 4], "big") + 3).to_bytes(4, "big")
    r, e = _try_gpu(torch_cuda, bytes(bad))
    # a shifted entry points into another meshlet's bits: whatever the header
    # read there says, the stream must be rejected
    assert r is None and e.code in (_lib.STRIDE_ERR_OFFSET, _lib.STRIDE_ERR_CORRUPT, _lib.STRIDE_ERR_UNSUPPORTED)
    bad = bytearray(data)
    bad[86:90] = (0).to_bytes(4, "big")
    r, e = _try_gpu(torch_cuda, bytes(bad))
    assert r is None and e.code == _lib.STRIDE_ERR_OFFSET


def test_reloads_in_a_row(torch_cuda):
    """Reloads without a decode between them: a large stream (uploaded by
    parts on the handle's copy stream), then a small one (uploaded on the
    decode stream, after the large one's parts), then the large one again;
    each decode, to host or device, equals the oracle."""
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    V, T = synth.noise_heightfield(1449, seed=8)
    big = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data
    small = _golden.load("grid129_b12")["data"]
    dec = ParaDeltaV5GpuDecoder(small)
    for seq in ([big, small], [small, big], [big, big]):
        for data in seq:
            dec.reload(data)
        last = seq[-1]
        opos, oidx = oracle.decode_mt(last, 0)
        pos, idx = dec.decode_to_host()
        assert np.array_equal(pos.view(np.uint32), opos.view(np.uint32))
        assert np.array_equal(idx.astype(np.int64), oidx)
        dec.reload(last)
        tris, verts = dec.decode_to_device()
        assert np.array_equal(verts.cpu().numpy().view(np.uint32), opos.view(np.uint32))
        assert np.array_equal(tris.view(torch_cuda.int32).cpu().numpy().astype(np.int64), oidx)
    dec.close()


@pytest.mark.parametrize("grid", [129, 1449])
def test_decode_to_host_reports_corruption(torch_cuda, grid):
    """A shifted offset-table entry in the last quarter of the meshlets (the
    last connectivity part of a large host decode): decode_to_host fails
    with the code the device decode reports, and the handle decodes the
    good stream afterwards."""
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    V, T = synth.noise_heightfield(grid, seed=4)
    data = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data
    dec = ParaDeltaV5GpuDecoder(data)
    m = (3 * dec.n_meshlets) // 4 + 1
    bad = bytearray(data)
    off = 86 + 4 * m
    bad[off:off + 4] = (int.from_bytes(bad[off:off + 4], "big") + 3).to_bytes(4, "big")
    dec.reload(bytes(bad))
    with pytest.raises(_lib.StrideFormatError) as on_host:
        dec.decode_to_host()
    with pytest.raises(_lib.StrideFormatError) as on_device:
        dec.decode_to_device()
    assert on_host.value.code == on_device.value.code
    assert on_host.value.code in (_lib.STRIDE_ERR_OFFSET, _lib.STRIDE_ERR_CORRUPT, _lib.STRIDE_ERR_UNSUPPORTED)
    dec.reload(data)
    pos, idx = dec.decode_to_host()
    opos, oidx = oracle.decode_mt(data, 0)
    assert np.array_equal(pos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(idx.astype(np.int64), oidx)
    dec.close()


def test_bit_flip_fuzz(torch_cuda):
    """Random single-bit corruptions: the GPU either rejects the stream or
    returns exactly what the reference semantics (oracle) return; whenever
    the oracle rejects, the GPU rejects too."""
    g = _golden.load("grid33_b12")
    data = g["data"]
    rng = np.random.default_rng(123)
    hdr_bits = (86 + 4 * 8) * 8
    accepted = rejected = 0
    for _ in range(120):
        b = bytearray(data)
        bit = int(rng.integers(hdr_bits, len(b) * 8))
        b[bit >> 3] ^= 0x80 >> (bit & 7)
        b = bytes(b)
        gr, ge = _try_gpu(torch_cuda, b)
        orr, oe = _try_oracle(b)
        if oe is not None:
            assert ge is not None, f"bit {bit}: oracle rejects ({oe}) but GPU accepted"
        if ge is None:
            accepted += 1
            assert orr is not None
            assert np.array_equal(gr[0].view(np.uint32), orr[0].view(np.uint32))
            assert np.array_equal(gr[1].astype(np.int64), orr[1])
        else:
            rejected += 1
    assert rejected > 0


@pytest.mark.parametrize("name", ["grid129_b12", "ico3_b12", "torus_b10"])
def test_device_side_table_matches_oracle(torch_cuda, name):
    """The substream starts the vertex kernel finds on the device equal the
    side table the oracle derives from the same bytes."""
    torch = torch_cuda
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    g = _golden.load(name)
    dec = ParaDeltaV5GpuDecoder(g["data"])
    dec.decode_to_device()
    resid, subs = dec.side_table()
    torch.cuda.synchronize()
    st = oracle.side_table(g["data"])
    assert np.array_equal(resid.cpu().numpy().astype(np.uint64), st["resid_bit"])
    assert np.array_equal(subs.cpu().numpy().view(np.uint16), st["sub_offs"])
    dec.close()


def test_reference_attributes_and_normalised_decode(torch_cuda):
    """decode(normalised=True) returns what the reference's decode() returns
    (utils/paradelta_v5_cuda.py:686-712): normalised float32 positions --
    decode_dup's float64 g_min + q / mx * g_range, rounded once -- and int32
    triangles; the attributes the reference's sweep script reads exist."""
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    torch = torch_cuda
    g = _golden.load("grid129_b12")
    data = g["data"]
    dec = ParaDeltaV5GpuDecoder(data)
    vn, tris = dec.decode(normalised=True)
    torch.cuda.synchronize()
    assert vn.dtype == torch.float32 and tris.dtype == torch.int32 and dec.d_verts_norm is vn
    _, oidx, ocodes = oracle.decode(data, with_codes=True)
    h = oracle.parse_header(data)
    ref = np.empty(ocodes.shape, np.float64)
    for d in range(3):
        mx = (1 << int(h.g_bits[d])) - 1
        ref[:, d] = float(h.g_min[d]) if mx == 0 else float(h.g_min[d]) + ocodes[:, d].astype(np.float64) / mx * float(h.g_range[d])
    assert np.array_equal(vn.cpu().numpy().view(np.uint32), ref.astype(np.float32).view(np.uint32))
    assert np.array_equal(tris.cpu().numpy().astype(np.int64), oidx)
    # world space, as decode_to_host returns it, is unchanged by the mode
    opos, _ = oracle.decode(data)
    verts, _ = dec.decode()
    assert np.array_equal(verts.cpu().numpy().view(np.uint32), opos.view(np.uint32))
    assert bytes(dec.d_buf.cpu().numpy()) == data
    assert dec._shared_bytes > 0 and dec._persistent_blocks > 0
    dec.close()
