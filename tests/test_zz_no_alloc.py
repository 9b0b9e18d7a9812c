"""The allocation-free decode entry point (stride_decode_static).

Callers such as a renderer's per-frame streaming loop or a plugin inside a
host application that owns device memory cannot call cudaMalloc/cudaFree
(they synchronise the device, or the host forbids them).  This entry point
serves them from a fixed device array inside the library.  These tests call
it through the C ABI and check that its output equals the ordinary
(allocating) entry point's, bit for bit -- the tolerance every parity test
here uses -- on calls in a row, one of them on a second stream after the
first stream's call has used the shared array, and check that the device's
free memory does not change during a call.

Kept in its own file, collected last, so a failure here comes after every
other test has run.
"""
import ctypes

import numpy as np
import pytest

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
    return torch


def _outputs(torch, info):
    idx = torch.full((int(info.n_t), 3), 0x7FFFFFFF, dtype=torch.int32, device="cuda")
    pos = torch.full((int(info.n_v), 3), float("nan"), dtype=torch.float32, device="cuda")
    return idx, pos


def _static_decode(torch, data, stream=None, free_check=False):
    """One call of the allocation-free entry point into fresh output tensors
    (allocated before the call).  With free_check, the device's free memory
    must be the same before and after the call: the call allocates nothing."""
    lib = _lib.load()
    info = _lib.inspect(data)
    idx, pos = _outputs(torch, info)
    stream = stream if stream is not None else torch.cuda.current_stream()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = lib.stride_decode_static(data, len(data), ctypes.c_void_p(int(stream.cuda_stream)),
                                  ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(pos.data_ptr()))
    free1 = torch.cuda.mem_get_info()[0]
    _lib.check(rc, "stride_decode_static")
    if free_check:
        assert free1 == free0, f"device free memory changed by {free0 - free1} bytes during the call"
    torch.cuda.synchronize()
    return idx.cpu().numpy().view(np.uint32), pos.cpu().numpy()


def _allocating_decode(torch, data):
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    dec = ParaDeltaV5GpuDecoder(data)
    idx, pos = _outputs(torch, dec.info)
    dec.decode_into(idx, pos)
    dec.close()
    return idx.cpu().numpy().view(np.uint32), pos.cpu().numpy()


def test_static_entry_matches_allocating_entry(torch_cuda):
    meshes = [synth.noise_heightfield(257, seed=21), synth.icosphere(5, seed=22)]
    streams = [encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data for V, T in meshes]
    side = torch_cuda.cuda.Stream()
    for data in streams:
        ref_idx, ref_pos = _allocating_decode(torch_cuda, data)
        # two calls in a row share (and reuse) the fixed array; the second
        # runs on another stream after the first one's, and from the second
        # call on the device's free memory must not change during a call
        for k, stream in enumerate((None, side, None)):
            idx, pos = _static_decode(torch_cuda, data, stream=stream, free_check=k > 0)
            assert np.array_equal(idx, ref_idx)
            assert np.array_equal(pos.view(np.uint32), ref_pos.view(np.uint32))


def test_static_entry_decodes_the_2049_heightfield(torch_cuda):
    """The largest workload of this decoder (8.4 million triangles) fits the
    fixed array."""
    V, T = synth.noise_heightfield(2049, seed=3)
    data = encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data
    ref_idx, ref_pos = _allocating_decode(torch_cuda, data)
    for k in range(2):
        idx, pos = _static_decode(torch_cuda, data, free_check=k > 0)
        assert np.array_equal(idx, ref_idx)
        assert np.array_equal(pos.view(np.uint32), ref_pos.view(np.uint32))


def test_static_entry_rejects_streams_beyond_its_scratch(torch_cuda):
    V, T = synth.heightfield_grid(33, seed=23)
    data = bytearray(encoder.encode(V, T, precision_error=B12, precision_mode="bbox_frac").data)
    data[74:78] = (60_000_000).to_bytes(4, "big")  # header claims 60 M vertices (walk scratch > 64 MiB)
    lib = _lib.load()
    rc = lib.stride_decode_static(bytes(data), len(data), None, ctypes.c_void_p(1), ctypes.c_void_p(1))
    assert rc == _lib.STRIDE_ERR_NOMEM
    assert "fixed" in _lib.last_error()
