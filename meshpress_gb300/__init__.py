"""GB300 (sm_103a) decoder for the STRIDE "DPR4" v3 mesh bitstream.

``ParaDeltaV5GpuDecoder`` is the drop-in for the reference class of the same
name (utils/paradelta_v5_cuda.py:580-718); given the reference class's own
PLDT v5 bytes it returns a ``PldtV5Decoder``.  ``BatchDecoder`` decodes many
streams in one launch; ``StrideServer`` is the continuous-batching service.
"""
from .decoder import ParaDeltaV5GpuDecoder, cull_meshlets, decode_to_device  # noqa: F401
from .pldt5 import PldtV5Decoder  # noqa: F401
from ._lib import StrideDeviceError, StrideFormatError  # noqa: F401
