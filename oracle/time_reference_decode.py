"""Times the reference's own CPU decoder on the 129 x 129 heightfield stream.

The unmodified ``decode_dup`` (encoder/paradelta_v5_dup.py:471-618) of the
reference checkout -- pure Python, one core -- decodes the committed golden
stream ``grid129_b12`` (made by the reference encoder, 32,768 triangles),
next to this repository's C restatement of it (the oracle) on one thread
and on all host cores, and the results are written as one JSON record.
Test infrastructure: the reference is read from MESHPRESS_REFERENCE
(default /root/reference) and the record is committed under profiles/.

    python oracle/time_reference_decode.py [out.json]
"""
from __future__ import annotations

import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REFERENCE = os.environ.get("MESHPRESS_REFERENCE", "/root/reference")


def _best(fn, reps: int):
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return min(ts), float(np.median(ts))


def main(out_path: str) -> int:
    sys.path.insert(0, REPO)
    sys.path.insert(0, REFERENCE)
    from encoder.paradelta_v5_dup import decode_dup  # the reference, unmodified

    import oracle
    from tests import _golden
    oracle.build()
    data = _golden.load("grid129_b12")["data"]
    V, T = decode_dup(data)
    opos, oidx = oracle.decode(data)
    same = bool(np.array_equal(V.view(np.uint32), opos.view(np.uint32)) and np.array_equal(T, oidx))
    n_t = int(len(T))
    ref_best, ref_med = _best(lambda: decode_dup(data), 5)
    port1_best, port1_med = _best(lambda: oracle.decode(data), 50)
    cores = os.cpu_count() or 1
    portn_best, portn_med = _best(lambda: oracle.decode_mt(data, cores), 50)
    rec = {
        "workload": "heightfield_129x129_12bit (golden grid129_b12: reference-encoded, 32,768 triangles)",
        "stream_bytes": len(data), "triangles": n_t, "same_output": same,
        "reference_decode_dup": {"kind": "reference", "cores": 1, "ms_best": round(ref_best * 1e3, 3),
                                 "ms_median": round(ref_med * 1e3, 3),
                                 "M_tris_per_s": round(n_t / ref_best / 1e6, 4),
                                 "what": "encoder/paradelta_v5_dup.py decode_dup, unmodified, pure Python"},
        "port_one_thread": {"kind": "port", "cores": 1, "ms_best": round(port1_best * 1e3, 3),
                            "ms_median": round(port1_med * 1e3, 3),
                            "M_tris_per_s": round(n_t / port1_best / 1e6, 3),
                            "what": "oracle/stride_oracle.c, sequential"},
        "port_all_cores": {"kind": "port", "cores": cores, "ms_best": round(portn_best * 1e3, 3),
                           "ms_median": round(portn_med * 1e3, 3),
                           "M_tris_per_s": round(n_t / portn_best / 1e6, 3),
                           "what": "oracle/stride_oracle.c, meshlet-parallel"},
        "host": {"machine": platform.machine(), "python": platform.python_version(), "cpu_count": cores},
        "command": "python oracle/time_reference_decode.py",
    }
    with open(out_path, "w") as f:
        json.dump(rec, f, indent=1)
        f.write("\n")
    print(json.dumps(rec))
    return 0 if same else 1


if __name__ == "__main__":
    sys.exit(main(sys.argv[1] if len(sys.argv) > 1 else
                  os.path.join(REPO, "profiles", "cpu_reference_decode_dup_heightfield_129_12bit.json")))
