"""Generate the golden PLDT v5 fixtures from the reference itself.

PLDT v5 is the format the reference's CuPy decoder ``ParaDeltaV5GpuDecoder``
reads (magic 0x504C4454, version 5: a global boundary table, per-meshlet
boundary references, strip connectivity and a float64 lin3 predictor).
Run in the development container (the reference checkout and numpy are
needed; numba is replaced by the stand-in next to this file):

    python tests/golden/make_golden_v5.py            # encoded meshes (v5_*)
    python tests/golden/make_golden_v5.py --crafted  # crafted corner cases (v5x_*)

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
REFERENCE = os.environ.get("MESHPRESS_REFERENCE", "/root/reference")  # the reference checkout

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


def _bit_writer():
    from utils.bit_codec import BitWriter
    return BitWriter


# ---------------------------------------------------------------------------
# Crafted streams: syntactically valid PLDT v5 bytes with corners that real
# encodes rarely reach (strip_len 0, FIFO eviction, interior vertices the
# walk never reaches, meshlets without boundary or without interior
# vertices, a 0-bit axis, all three residual tags, a negative fixed-width
# minimum, Rice codewords with unary prefixes over 32 bits).  The reference
# decode_paradelta_v5 is the authority for the expected output.
# ---------------------------------------------------------------------------
def craft_v5(BitWriter, rng, *, n_meshlets, n_boundary, g_bits, max_local=60, allow_len0=False,
             allow_unreached=False, long_prefix=False):
    f32 = lambda a: [float(np.float32(x)) for x in a]  # noqa: E731
    center = f32(rng.normal(0, 2, 3))
    scale = float(np.float32(rng.uniform(0.5, 8.0)))
    per_coord_err = float(np.float32(rng.uniform(1e-4, 1e-2)))
    g_min = f32(rng.uniform(-1, 0, 3))
    g_range = f32(rng.uniform(0.3, 2.0, 3))
    lin3 = f32(np.array([1.0, 1.0, -1.0]) + rng.normal(0, 0.05, 3))
    body = BitWriter()
    rel = []
    n_t = 0
    n_int_total = 0
    for m in range(n_meshlets):
        rel.append(body.bit_pos())
        n_bnd = 0 if (m == 1 or n_boundary == 0) else int(rng.integers(1, min(n_boundary, 24) + 1))
        n_int = 0 if m == 2 else int(rng.integers(3, max_local))
        n_local = n_bnd + n_int
        if n_local < 3:
            n_int += 3 - n_local
            n_local = 3
        refs = sorted(rng.choice(n_boundary, n_bnd, replace=False).tolist()) if n_bnd else []
        idx_bits = max(1, int(n_local).bit_length())
        # strips over random tokens, simulating the decoder's FIFO
        fifo, strips, tris = [], [], 0
        reach = n_local if not allow_unreached else max(3, n_local - 4)
        seen = set()
        while (len(seen) < reach or not strips) and len(strips) < 200:
            slen = int(rng.integers(0 if allow_len0 else 1, 20))
            toks = []

            def pick():
                unseen = [i for i in range(reach) if i not in seen]
                if fifo and rng.uniform() < 0.45:
                    fi = int(rng.integers(0, len(fifo)))
                    v, tok = fifo[fi], (0, fi)
                else:
                    v = int(unseen[int(rng.integers(0, len(unseen)))]) if unseen and rng.uniform() < 0.8 \
                        else int(rng.integers(0, reach))
                    tok = (1, v)
                if v in fifo:
                    fifo.remove(v)
                fifo.append(v)
                if len(fifo) > 16:
                    fifo.pop(0)
                seen.add(v)
                return tok

            for _ in range(3):
                toks.append((None, pick()))
            for _ in range(max(slen - 1, 0)):
                toks.append((int(rng.integers(0, 2)), pick()))
            strips.append((slen, toks))
            tris += max(slen, 1)
        n_t += tris
        n_int_total += n_int
        body.write_fixed(n_bnd, 16)
        body.write_fixed(n_int, 16)
        body.write_fixed(tris, 16)
        body.write_fixed(len(strips), 16)
        if n_bnd:
            body.write_fixed(refs[0], 32)
            if n_bnd > 1:
                k = int(rng.integers(0, 5))
                body.write_fixed(k, 8)
                for a, b in zip(refs[:-1], refs[1:]):
                    body.write_rice(b - a - 1, k)
        for slen, toks in strips:
            body.write_fixed(slen, 16)
            for edge, (flag, val) in toks:
                if edge is not None:
                    body.write_bits(edge, 1)
                body.write_bits(flag, 1)
                body.write_bits(val, 5 if flag == 0 else idx_bits)
        if n_int:
            for d in range(3):
                tag = int(rng.integers(0, 3)) if not long_prefix or d else 1
                codes = rng.integers(-40, 40, n_int)
                if tag == 0:
                    mn = int(codes.min()) - int(rng.integers(0, 3))
                    bw = max(1, int(int(codes.max() - mn)).bit_length())
                    body.write_fixed(0, 8)
                    body.write_fixed(mn & 0xFFFF, 16)
                    body.write_fixed(bw, 8)
                    for c in codes:
                        body.write_fixed(int(c) - mn, bw)
                else:
                    k = 0 if long_prefix and d == 0 else int(rng.integers(0, 4))
                    body.write_fixed(tag, 8)
                    body.write_fixed(k, 8)
                    for c in codes:
                        u = (int(c) << 1) ^ (int(c) >> 63)
                        if long_prefix and d == 0 and rng.uniform() < 0.2:
                            u = int(rng.integers(66, 140))  # unary prefix over 32 bits
                        (body.write_rice if tag == 1 else body.write_exp_golomb)(u, k)
    w = BitWriter()
    w.write_fixed(0x504C4454, 32)
    w.write_fixed(5, 8)
    w.write_fixed(0, 8)
    for c in center:
        w.write_f32(c)
    w.write_f32(scale)
    w.write_f32(per_coord_err)
    for v in g_min:
        w.write_f32(v)
    for v in g_range:
        w.write_f32(v)
    for b in g_bits:
        w.write_fixed(int(b), 8)
    w.write_fixed(n_boundary + n_int_total, 32)
    w.write_fixed(n_t, 32)
    w.write_fixed(n_boundary, 32)
    w.write_fixed(n_meshlets, 32)
    for v in lin3:
        w.write_f32(v)
    if n_boundary:
        for d in range(3):
            codes = rng.integers(0, 1 << g_bits[d], n_boundary) if g_bits[d] else np.zeros(n_boundary, np.int64)
            w.write_fixed(int(codes[0]), int(g_bits[d]))
            if n_boundary > 1:
                k = int(rng.integers(0, 8))
                w.write_fixed(k, 8)
                for a, b in zip(codes[:-1], codes[1:]):
                    dlt = int(b) - int(a)
                    w.write_rice((dlt << 1) ^ (dlt >> 63), k)
    pad = (-w.bit_pos()) & 7
    if pad:
        w.write_bits(0, pad)
    start = w.bit_pos() + 32 * n_meshlets
    for r in rel:
        w.write_fixed(start + r, 32)
    return w.finalize() + body.finalize()


def crafted(ref, name, seed, **kw):
    _, _, decode_v5 = ref
    BitWriter = _bit_writer()
    rng = np.random.default_rng(seed)
    data = craft_v5(BitWriter, rng, **kw)
    Vd, Td = decode_v5(data)
    meta = dict(kind="pldt_v5_crafted", seed=seed, bytes=len(data), n_v=int(len(Vd)), n_t=int(len(Td)),
                **{k: (v if not isinstance(v, np.ndarray) else v.tolist()) for k, v in kw.items()})
    print(f"v5x_{name}: {meta}")
    path = os.path.join(HERE, f"v5x_{name}.npz")
    np.savez_compressed(path, blob=np.frombuffer(data, dtype=np.uint8), pos=Vd.astype(np.float32),
                        idx=Td.astype(np.int64), meta=np.array(json.dumps(meta)))


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


def main_crafted(ref):
    crafted(ref, "a", 101, n_meshlets=6, n_boundary=40, g_bits=[12, 11, 10], allow_len0=True)
    crafted(ref, "b", 102, n_meshlets=5, n_boundary=30, g_bits=[10, 0, 9], allow_unreached=True)
    crafted(ref, "c", 103, n_meshlets=4, n_boundary=1, g_bits=[16, 16, 16], long_prefix=True)
    crafted(ref, "d", 104, n_meshlets=7, n_boundary=0, g_bits=[12, 12, 12], max_local=200, allow_len0=True)


def main():
    ref = _import_reference()
    if "--crafted" in sys.argv:
        main_crafted(ref)
        return
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
