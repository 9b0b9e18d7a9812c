"""Host-side helpers of bench.py (no GPU)."""
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
import bench  # noqa: E402


def test_kernel_split_one_kernel():
    # scan, the one decode kernel (its time in the second slot), 0
    names, dom, nbytes = bench.kernel_split(np.array([0.014, 0.22, 0.0]), True, 1000, 10, 20)
    assert names == ("scan_kernel", "flow_kernel") and dom == 1  # the default shape
    assert nbytes == 1000 + 12 * (10 + 20)  # stream in, both outputs out
    names, dom, _ = bench.kernel_split(np.array([0.014, 0.22, 0.0]), True, 1000, 10, 20, persistent=3)
    assert names == ("scan_kernel", "group_kernel") and dom == 1


def test_kernel_split_two_kernels():
    names, dom, nbytes = bench.kernel_split(np.array([0.01, 0.14, 0.13]), False, 1000, 10, 20)
    assert names[dom] == "conn_kernel" and nbytes == 1000 + 12 * 20  # stream in, indices out
    names, dom, nbytes = bench.kernel_split(np.array([0.01, 0.12, 0.13]), False, 1000, 10, 20)
    assert names[dom] == "vert_kernel" and nbytes == 12 * 10  # positions out
