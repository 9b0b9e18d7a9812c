"""Many meshes in one launch (stride_batch_*): every mesh of a mixed batch
decodes bit-exactly like it does alone, under every launch path (eager,
persistent work stealing, CUDA graph replay, autotuned shape)."""
import ctypes

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
def mixed_streams():
    """Forty meshes from the many-mesh generator (sizes 100 .. 20 K
    triangles), plus one with 20-bit codes and one single-triangle mesh."""
    specs = synth.mixed_batch_specs(40, seed=9, t_min=100, t_max=2e4)
    out = []
    for kind, params in specs:
        V, T = synth.build_spec(kind, params)
        out.append(encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data)
    V, T = synth.heightfield_grid(65, seed=5)
    out.insert(7, encoder.encode(V, T, precision_error=synth.bbox_bits_error(20), precision_mode="bbox_frac").data)
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)
    out.insert(3, encoder.encode(V, np.array([[0, 1, 2]]), precision_error=B12, precision_mode="bbox_frac").data)
    return out


def _check_meshes(b, streams, tris, verts):
    t = tris.cpu().numpy().view(np.uint32)
    v = verts.cpu().numpy()
    for i, data in enumerate(streams):
        opos, oidx = oracle.decode(data)
        ti = t[b.t_offset[i]:b.t_offset[i + 1]]
        vi = v[b.v_offset[i]:b.v_offset[i + 1]]
        assert np.array_equal(ti.astype(np.int64), oidx), f"mesh {i} triangles"
        assert np.array_equal(vi.view(np.uint32), opos.view(np.uint32)), f"mesh {i} positions"


def test_batch_matches_oracle_per_mesh(torch_cuda, mixed_streams):
    from meshpress_gb300.batch import BatchDecoder
    b = BatchDecoder(mixed_streams)
    tris, verts = b.decode()
    _check_meshes(b, mixed_streams, tris, verts)
    b.close()


@pytest.mark.parametrize("cfg", [(1, 0, 16 * 1024, 8 * 1024), (2, 1, 12 * 1024, 12 * 1024), (4, 1, 8 * 1024, 6 * 1024),
                                 (4, 2, 8 * 1024, 6 * 1024)],
                         ids=["w1", "w2p", "w4p", "w4fused"])
def test_batch_launch_shapes(torch_cuda, mixed_streams, cfg):
    from meshpress_gb300.batch import BatchDecoder
    b = BatchDecoder(mixed_streams)
    c = _lib.LaunchCfg()
    c.warps_per_cta, c.persistent, c.ctas_per_sm, c.stage_bytes, c.code_bytes = cfg[0], cfg[1], 0, cfg[2], 2 * cfg[3]
    b.set_config(c)
    tris, verts = b.decode()
    _check_meshes(b, mixed_streams, tris, verts)
    b.close()


def test_graph_replay_and_autotune_identical(torch_cuda, mixed_streams):
    torch = torch_cuda
    from meshpress_gb300.batch import BatchDecoder
    b = BatchDecoder(mixed_streams)
    ref_t, ref_v = (x.clone() for x in b.decode())
    best, ms = b.autotune(iters=1)
    assert ms > 0 and best.warps_per_cta in (1, 2, 4)
    assert b.config().as_dict() == best.as_dict()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.d_tris.fill_(0)
        b.d_verts.fill_(float("nan"))
        b.capture_graph(s)
        for _ in range(3):
            b.d_tris.fill_(0)
            b.launch_graph(s, check=True)
    s.synchronize()
    assert torch.equal(b.d_tris, ref_t)
    assert torch.equal(b.d_verts.view(torch.int32), ref_v.view(torch.int32))
    b.close()


def test_batch_reports_the_corrupt_mesh(torch_cuda, mixed_streams):
    from meshpress_gb300.batch import BatchDecoder
    streams = list(mixed_streams)
    streams[5] = streams[5][: len(streams[5]) - 64]  # truncated: meshlet offsets point past the end
    b = BatchDecoder(streams)
    i, p = b._ptrs()
    _lib.check(b._lib.stride_batch_decode(b._h, b._stream(), i, p))
    bm, bl = ctypes.c_uint32(), ctypes.c_uint32()
    rc = b._lib.stride_batch_status(b._h, 1, ctypes.byref(bm), ctypes.byref(bl))
    assert rc in (_lib.STRIDE_ERR_OFFSET, _lib.STRIDE_ERR_CORRUPT, _lib.STRIDE_ERR_UNSUPPORTED)
    assert bm.value == 5
    b.close()


def test_batch_of_one_equals_single_decoder(torch_cuda):
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    from meshpress_gb300.batch import BatchDecoder
    V, T = synth.icosphere(6, seed=31)
    data = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data
    dt, dv = ParaDeltaV5GpuDecoder(data).decode_to_device()
    b = BatchDecoder([data])
    bt, bv = b.decode()
    assert torch_cuda.equal(bt.view(torch_cuda.int32), dt.view(torch_cuda.int32))
    assert torch_cuda.equal(bv.view(torch_cuda.int32), dv.view(torch_cuda.int32))
    b.close()


@pytest.fixture(scope="module")
def large_streams(mixed_streams):
    """Two 1025^2 heightfields around the mixed meshes: about 4.6 M
    triangles, so a host decode runs its connectivity in parts whose
    boundaries fall inside meshes."""
    out = []
    for seed in (1, 2):
        V, T = synth.noise_heightfield(1025, seed=seed)
        out.append(encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data)
    return [out[0]] + list(mixed_streams) + [out[1]]


@pytest.mark.parametrize("which", ["mixed", "large"])
def test_batch_decode_to_host(torch_cuda, mixed_streams, large_streams, which):
    """Host outputs (pinned, copied while the decode runs) equal the device
    decode bit for bit, for the mixed batch and for one large enough for the
    connectivity to run in parts."""
    torch = torch_cuda
    from meshpress_gb300.batch import BatchDecoder
    streams = mixed_streams if which == "mixed" else large_streams
    b = BatchDecoder(streams)
    ref_t, ref_v = (x.cpu().numpy() for x in b.decode())
    h_pos = torch.empty((b.n_v_total, 3), dtype=torch.float32, pin_memory=True)
    h_idx = torch.empty((b.n_t_total, 3), dtype=torch.int32, pin_memory=True)
    for _ in range(2):
        h_pos.fill_(float("nan"))
        h_idx.fill_(-1)
        pos, idx = b.decode_to_host(out=(h_pos.numpy(), h_idx.numpy().view(np.uint32)))
        assert np.array_equal(idx, ref_t.view(np.uint32))
        assert np.array_equal(pos.view(np.uint32), ref_v.view(np.uint32))
    # pageable outputs: the same bytes
    pos, idx = b.decode_to_host()
    assert np.array_equal(idx, ref_t.view(np.uint32)) and np.array_equal(pos.view(np.uint32), ref_v.view(np.uint32))
    if which == "large":
        _check_meshes(b, streams, torch.from_numpy(idx.view(np.int32)), torch.from_numpy(pos))
        # an arena image then goes up by parts, each part decoded when its bytes are in
        img = b.make_image()
        h_img = torch.empty(img.size, dtype=torch.uint8, pin_memory=True)
        h_img.numpy()[:] = img
        for _ in range(2):
            b.upload(h_img.data_ptr(), img.size)
            h_pos.fill_(float("nan"))
            h_idx.fill_(-1)
            pos, idx = b.decode_to_host(out=(h_pos.numpy(), h_idx.numpy().view(np.uint32)))
            assert np.array_equal(idx, ref_t.view(np.uint32))
            assert np.array_equal(pos.view(np.uint32), ref_v.view(np.uint32))
        # a device decode after such an upload waits for all of it
        b.upload(h_img.data_ptr(), img.size)
        tris, verts = b.decode()
        assert np.array_equal(tris.cpu().numpy().view(np.uint32), ref_t.view(np.uint32))
        assert np.array_equal(verts.cpu().numpy().view(np.uint32), ref_v.view(np.uint32))
    b.close()


def test_batch_decode_to_host_reports_the_corrupt_mesh(torch_cuda, large_streams):
    from meshpress_gb300.batch import BatchDecoder
    streams = list(large_streams)
    streams[-2] = streams[-2][: len(streams[-2]) - 64]
    b = BatchDecoder(streams)
    with pytest.raises(_lib.StrideFormatError) as e:
        b.decode_to_host()
    assert e.value.code in (_lib.STRIDE_ERR_OFFSET, _lib.STRIDE_ERR_CORRUPT, _lib.STRIDE_ERR_UNSUPPORTED)
    assert f"mesh {len(streams) - 2}," in str(e.value)
    bm, bl = ctypes.c_uint32(), ctypes.c_uint32()
    assert b._lib.stride_batch_status(b._h, 1, ctypes.byref(bm), ctypes.byref(bl)) == e.value.code
    assert bm.value == len(streams) - 2
    b.close()
