"""Meshlet-native outputs (the consumer step after decode): ranges equal the
prefix sums of the meshlet headers, bounds equal the per-meshlet min / max
of the decoded positions, and frustum culling equals the same box test done
in numpy (float32, same operation order)."""
import numpy as np
import pytest

import oracle
from meshpress_gb300 import encoder, synth

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
def decoded(torch_cuda):
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    V, T = synth.icosphere(6, seed=21)
    data = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data
    dec = ParaDeltaV5GpuDecoder(data)
    tris, verts = dec.decode_to_device()
    yield data, dec, tris, verts
    dec.close()


def test_meshlet_ranges(torch_cuda, decoded):
    data, dec, tris, verts = decoded
    v, t = dec.meshlet_ranges()
    st = oracle.side_table(data)
    ev = np.concatenate([[0], np.cumsum(st["n_local"].astype(np.int64))])
    et = np.concatenate([[0], np.cumsum(st["n_tris"].astype(np.int64))])
    assert np.array_equal(v.cpu().numpy(), ev) and np.array_equal(t.cpu().numpy(), et)
    # every triangle of meshlet m indexes its own vertex rows
    idx = tris.view(torch_cuda.int32).cpu().numpy().astype(np.int64)
    for m in range(0, dec.n_meshlets, max(1, dec.n_meshlets // 50)):
        rows = idx[et[m]:et[m + 1]]
        assert rows.min() >= ev[m] and rows.max() < ev[m + 1]


def _bounds_np(pos, ev):
    out = np.empty((len(ev) - 1, 6), np.float32)
    for m in range(len(ev) - 1):
        p = pos[ev[m]:ev[m + 1]]
        out[m, :3] = p.min(axis=0)
        out[m, 3:] = p.max(axis=0)
    return out


def test_meshlet_bounds(torch_cuda, decoded):
    data, dec, tris, verts = decoded
    b = dec.meshlet_bounds(verts).cpu().numpy()
    v, _ = dec.meshlet_ranges()
    ref = _bounds_np(verts.cpu().numpy(), v.cpu().numpy())
    assert np.array_equal(b.view(np.uint32), ref.view(np.uint32))


def _cull_np(b, planes):
    vis = (b[:, 0] <= b[:, 3]) & (b[:, 1] <= b[:, 4]) & (b[:, 2] <= b[:, 5])
    P = np.asarray(planes, np.float32).reshape(6, 4)
    for a, bb, c, d in P:
        px = np.where(a >= 0, b[:, 3], b[:, 0])
        py = np.where(bb >= 0, b[:, 4], b[:, 1])
        pz = np.where(c >= 0, b[:, 5], b[:, 2])
        s = ((a * px + bb * py) + c * pz) + d  # float32, left to right
        vis &= ~(s < 0)
    return vis


@pytest.mark.parametrize("half", [0.8, 1.0, 2.0])
def test_frustum_culling(torch_cuda, decoded, half):
    from meshpress_gb300 import cull_meshlets
    data, dec, tris, verts = decoded
    b = dec.meshlet_bounds(verts)
    # a box-shaped frustum [-half, half]^3 around the origin, slightly tilted
    planes = np.array([[1, 0.05, 0, half], [-1, 0, 0.05, half], [0, 1, 0, half],
                       [0.05, -1, 0, half], [0, 0, 1, half], [0, 0.05, -1, half]], np.float32)
    vis, cnt = cull_meshlets(b, planes)
    n = dec.n_meshlets
    bits = vis.cpu().numpy().view(np.uint32)
    got = np.array([(bits[m // 32] >> (m % 32)) & 1 for m in range(n)], bool)
    want = _cull_np(b.cpu().numpy(), planes)
    assert np.array_equal(got, want)
    assert int(cnt.cpu()[0]) == int(want.sum())
    assert 0 < want.sum() <= n
