"""Helpers for the golden fixtures written by tests/golden/make_golden.py."""
import glob
import hashlib
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    """The STRIDE (DPR4 v3) fixtures (the PLDT v5 ones are named v5_* and v5x_*)."""
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        b = os.path.basename(f)[:-4]
        if b.endswith(".l2g") or b == "bitcodec" or b.startswith(("v5_", "v5x_")):
            continue
        out.append(b)
    return out


def load(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["data"] = d["blob"].tobytes()
    d["meta"] = json.loads(str(d["meta"]))
    return d


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def check_against(g, pos, idx, codes=None):
    """Bit-exact comparison of a decode with a golden fixture."""
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    idx = np.ascontiguousarray(idx).astype(np.int64)
    assert pos.shape == (int(g["n_v"]), 3) and idx.shape == (int(g["n_t"]), 3)
    if "pos" in g:
        bad = np.nonzero(pos.view(np.uint32) != g["pos"].view(np.uint32))
        assert bad[0].size == 0, f"{bad[0].size} position words differ, first at {bad[0][:5]}"
        assert np.array_equal(idx, g["idx"])
    assert sha(pos) == str(g["pos_sha256"])
    assert sha(idx) == str(g["idx_sha256"])
    if codes is not None and str(g["codes_sha256"]):
        assert sha(np.asarray(codes).astype(np.int64)) == str(g["codes_sha256"])
