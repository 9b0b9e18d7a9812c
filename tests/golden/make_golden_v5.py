"""Generate the golden PLDT v5 fixtures from the reference itself.

PLDT v5 is the format the reference's CuPy decoder ``ParaDeltaV5GpuDecoder``
reads (magic 0x504C4454, version 5: a global boundary table, per-meshlet
boundary references, strip connectivity and a float64 lin3 predictor).
Run in the development container (the reference checkout and numpy are
needed; numba is replaced by the stand-in next to this file):

    python tests/golden/make_golden_v5.py

For every case this script builds a seeded synthetic mesh with
``meshpress_gb300.synth``, encodes it with the reference encoder
(``prepare_paradelta_arrays`` + ``encode_from_prepared_v5``,
encoder/paradelta_v5.py:144-279), decodes the bytes with the reference CPU
decoder ``decode_paradelta_v5`` (encoder/paradelta_v5.py:286-462) and writes
``v5_<case>.npz`` with the bytes and the decoded float32 positions and int64
triangle indices.

The reference is copied to a temporary directory first (its helpers may
write caches next to their sources).
"""
from __future__ import annotations

import json
import os
import shutil
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE = "/root/reference"

sys.path.insert(0, REPO)
from meshpress_gb300 import synth  # noqa: E402


def _import_reference():
    tmp = tempfile.mkdtemp(prefix="pldt5_ref_")
    for sub in ("encoder", "utils", "reader"):
        shutil.copytree(os.path.join(REFERENCE, sub), os.path.join(tmp, sub))
    sys.path.insert(0, os.path.join(HERE, "numba_standin"))
    sys.path.insert(0, tmp)
    from encoder.paradelta_codec import prepare_paradelta_arrays
    from encoder.paradelta_v5 import decode_paradelta_v5, encode_from_prepared_v5
    return prepare_paradelta_arrays, encode_from_prepared_v5, decode_paradelta_v5


def case(ref, name, V, T, *, precision_error, precision_mode, max_verts=256, max_tris=256):
    prepare, encode_v5, decode_v5 = ref
    t0 = time.time()
    prep = prepare(V, T, max_verts=max_verts, max_tris=max_tris,
                   precision_error=precision_error, precision_mode=precision_mode)
    data = encode_v5(prep)
    t1 = time.time()
    Vd, Td = decode_v5(data)
    t2 = time.time()
    meta = dict(kind="pldt_v5", n_src_v=int(len(V)), n_src_t=int(len(T)),
                g_bits=[int(b) for b in prep["g_bits"]], n_meshlets=int(prep["n_meshlets"]),
                n_boundary=int(prep["n_boundary"]), bytes=len(data), precision_error=precision_error,
                precision_mode=precision_mode, max_verts=max_verts, max_tris=max_tris,
                encode_s=round(t1 - t0, 2), decode_s=round(t2 - t1, 3))
    print(f"v5_{name}: {meta}")
    path = os.path.join(HERE, f"v5_{name}.npz")
    np.savez_compressed(path, blob=np.frombuffer(data, dtype=np.uint8), pos=Vd.astype(np.float32),
                        idx=Td.astype(np.int64), meta=np.array(json.dumps(meta)))
    print(f"  wrote {path} ({os.path.getsize(path)} B)")


def main():
    ref = _import_reference()
    b12 = synth.bbox_bits_error(12)
    V, T = synth.heightfield_grid(9, seed=2)
    case(ref, "grid9_b12", V, T, precision_error=b12, precision_mode="bbox_frac")
    V, T = synth.heightfield_grid(33, seed=5)
    case(ref, "grid33_b12", V, T, precision_error=b12, precision_mode="bbox_frac")
    case(ref, "grid33_mv64", V, T, precision_error=b12, precision_mode="bbox_frac", max_verts=64, max_tris=64)
    V, T = synth.heightfield_grid(65, seed=7)
    case(ref, "grid65_world", V, T, precision_error=0.0005, precision_mode="world")
    V, T = synth.noise_heightfield(33, seed=9)
    case(ref, "noise33_b16", V, T, precision_error=synth.bbox_bits_error(16), precision_mode="bbox_frac",
         max_verts=96, max_tris=128)
    V, T = synth.icosphere(3, seed=4)
    case(ref, "ico3_b12", V, T, precision_error=b12, precision_mode="bbox_frac")
    V, T = synth.torus(24, 12)
    case(ref, "torus_b10", V, T, precision_error=synth.bbox_bits_error(10), precision_mode="bbox_frac",
         max_verts=48, max_tris=64)
    V, T = synth.noise_heightfield(129, seed=11)
    case(ref, "noise129_mv128", V, T, precision_error=b12, precision_mode="bbox_frac", max_verts=128, max_tris=128)
    V, T = synth.icosphere(5, seed=6)
    case(ref, "ico5_b14", V, T, precision_error=synth.bbox_bits_error(14), precision_mode="bbox_frac")
    V = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.5]])
    T = np.array([[0, 1, 2]])
    case(ref, "tri1_b12", V, T, precision_error=b12, precision_mode="bbox_frac")


if __name__ == "__main__":
    main()
