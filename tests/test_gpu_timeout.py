"""Bounded device waits report STRIDE_ERR_TIMEOUT and leave the context usable.

Every wait inside the decode kernels -- a bulk copy's mbarrier in the vertex
phase, the fused kernel's wait for a finished connectivity group -- spins at
most a set number of SM clocks (stride_set_wait_limit; about a second by
default) and then gives up with an error status instead of hanging.  Here the
limit is set to 0, so the first wait that does not succeed at once gives up:
the decode must come back with STRIDE_ERR_TIMEOUT, and the next decode with
the default limit must be bit-exact.  No wait is made to run forever: the
limit ends it.
"""
import numpy as np
import pytest

import oracle
from meshpress_gb300 import _lib, encoder, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshpress_gb300 import _build
    _build.build_decoder()
    oracle.build()
    return torch


def _shape(w, pers, stage=16 * 1024, code=12 * 1024):
    c = _lib.LaunchCfg()
    c.warps_per_cta, c.persistent, c.ctas_per_sm, c.stage_bytes, c.code_bytes = w, pers, 0, stage, code
    return c


@pytest.mark.parametrize("shape", [(4, 2), (4, 1)], ids=["fused", "two_kernels"])
def test_zero_wait_limit_times_out_then_decodes_exactly(torch_cuda, shape):
    torch = torch_cuda
    from meshpress_gb300 import ParaDeltaV5GpuDecoder
    V, T = synth.noise_heightfield(1025, seed=3)
    data = encoder.encode(V, T, precision_error=synth.bbox_bits_error(12), precision_mode="bbox_frac").data
    dec = ParaDeltaV5GpuDecoder(data)
    dec.set_launch_config(_shape(*shape))
    lib = _lib.load()
    idx = torch.empty((dec.n_t_total, 3), dtype=torch.int32, device="cuda")
    pos = torch.empty((dec.n_v_total, 3), dtype=torch.float32, device="cuda")
    _lib.check(lib.stride_set_wait_limit(dec._h, 0))
    with pytest.raises(_lib.StrideDeviceError) as err:
        dec.decode_into(idx, pos)
    assert err.value.code == _lib.STRIDE_ERR_TIMEOUT
    # the context is intact: the default limit decodes the same stream exactly
    _lib.check(lib.stride_set_wait_limit(dec._h, 1 << 31))
    dec.decode_into(idx, pos)
    opos, oidx = oracle.decode_mt(data, 0)
    assert np.array_equal(pos.cpu().numpy().view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(idx.cpu().numpy().view(np.uint32).astype(np.int64), oidx)
    dec.close()
