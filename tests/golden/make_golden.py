"""Generate the golden STRIDE (DPR4 v3) fixtures from the reference itself.

Run in the development container (the reference checkout and numpy are
needed; numba is replaced by the stand-in next to this file):

    python tests/golden/make_golden.py [--quick]

For every case this script

1. builds a seeded synthetic mesh with ``meshpress_gb300.synth`` (or crafts a
   syntactically valid stream with edge-case features, see ``craft_stream``),
2. encodes it with the reference encoder (``prepare_paradelta_arrays`` +
   ``encode_dup``, i.e. what ``STRIDEEncoder.encode`` calls),
3. decodes the bytes with the reference CPU decoder ``decode_dup``
   (encoder/paradelta_v5_dup.py:471-618),
4. writes ``<case>.npz`` with the bytes, the decoded float32 positions and
   triangle indices (or their SHA-256 for the large cases), and the encoder's
   integer codes in decode order (``global_codes[local_to_global]`` per
   meshlet).

The reference is copied to a temporary directory first because its predictor
fit writes a sample cache next to its sources (encoder/_irlp_fit.py:43-49).
"""
from __future__ import annotations

import argparse
import hashlib
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
    tmp = tempfile.mkdtemp(prefix="stride_ref_")
    for sub in ("encoder", "utils", "reader"):
        shutil.copytree(os.path.join(REFERENCE, sub), os.path.join(tmp, sub))
    sys.path.insert(0, os.path.join(HERE, "numba_standin"))
    sys.path.insert(0, tmp)
    from encoder.paradelta_codec import prepare_paradelta_arrays
    from encoder.paradelta_v5_dup import decode_dup, encode_dup
    from utils.bit_codec import BitWriter
    return prepare_paradelta_arrays, encode_dup, decode_dup, BitWriter


def _sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _save(name, data, V, T, codes, meta, full):
    out = {
        "blob": np.frombuffer(data, dtype=np.uint8),
        "pos_sha256": np.array(_sha(V.astype(np.float32))),
        "idx_sha256": np.array(_sha(T.astype(np.int64))),
        "codes_sha256": np.array(_sha(codes.astype(np.int64))) if codes is not None else np.array(""),
        "n_v": np.array(len(V)), "n_t": np.array(len(T)),
        "meta": np.array(json.dumps(meta)),
    }
    if full:
        out["pos"] = V.astype(np.float32)
        out["idx"] = T.astype(np.int64)
        if codes is not None:
            out["codes"] = codes.astype(np.int64)
    else:
        # A few rows for readable failure messages.
        out["pos_head"] = V[:64].astype(np.float32)
        out["idx_head"] = T[:64].astype(np.int64)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"  wrote {path} ({os.path.getsize(path)} B)")


def mesh_case(ref, name, V, T, *, precision_error, precision_mode,
              predictor="generalized", full=True, max_verts=256, max_tris=256):
    prepare, encode_dup, decode_dup, _ = ref
    t0 = time.time()
    prep = prepare(V, T, max_verts=max_verts, max_tris=max_tris,
                   precision_error=precision_error,
                   precision_mode=precision_mode)
    data = encode_dup(prep, predictor=predictor)
    t1 = time.time()
    Vd, Td = decode_dup(data)
    t2 = time.time()
    gc = np.asarray(prep["global_codes"], dtype=np.int64)
    codes = np.concatenate([gc[np.asarray(p["local_to_global"], dtype=np.int64)]
                            for p in prep["plans"]])
    l2g = np.concatenate([np.asarray(p["local_to_global"], dtype=np.int64)
                          for p in prep["plans"]])
    meta = dict(kind="mesh", n_src_v=int(len(V)), n_src_t=int(len(T)),
                g_bits=[int(b) for b in prep["g_bits"]],
                n_meshlets=int(prep["n_meshlets"]), bytes=len(data),
                precision_error=precision_error, precision_mode=precision_mode,
                predictor=predictor, encode_s=round(t1 - t0, 2),
                decode_dup_s=round(t2 - t1, 4))
    print(f"{name}: {meta}")
    _save(name, data, Vd, Td, codes, meta, full)
    # The source mesh is regenerated from the seeded generator in tests; the
    # local->global map lets tests check crack-freeness and triangle sets.
    np.savez_compressed(os.path.join(HERE, f"{name}.l2g.npz"), l2g=l2g.astype(np.int32))


# ---------------------------------------------------------------------------
# Crafted streams: syntactically valid DPR4 v3 bytes exercising corners of
# the format that a real encode rarely hits (EG with tag 0/3, K > 0 with
# negative weights, FIFO eviction, strip_len 0, empty meshlets, unvisited
# local vertices, a 0-bit axis, long unary runs).  The bytes are decoded by
# the reference decode_dup, which is the authority for the expected output.
# ---------------------------------------------------------------------------

def _bits_for(n_local: int) -> int:
    return max(1, int(n_local).bit_length())


def craft_stream(BitWriter, rng, *, n_meshlets, g_bits, pred_n, pred_K,
                 max_local=100, allow_unvisited=False, allow_empty=False,
                 allow_len0=False, big_residuals=False):
    center = rng.normal(0, 3, 3).astype(np.float32)
    scale = np.float32(rng.uniform(0.5, 20.0))
    g_min = rng.uniform(-1, 0, 3).astype(np.float32)
    g_range = rng.uniform(0.2, 2.0, 3).astype(np.float32)
    body = BitWriter()
    offs = []
    total_local = 0
    total_tris = 0
    for m in range(n_meshlets):
        offs.append(body.bit_pos())
        if allow_empty and m == 1:
            n_local = 0
        else:
            n_local = int(rng.integers(3, max_local + 1))
        ib = _bits_for(n_local)
        codes = np.zeros((n_local, 3), dtype=np.int64)
        for d in range(3):
            codes[:, d] = rng.integers(0, (1 << g_bits[d]), n_local) if g_bits[d] else 0
        # --- connectivity: random strips over random tokens.
        fifo = []
        seen = set()
        walk = []
        strips = []
        if n_local:
            target = n_local if not allow_unvisited else max(3, n_local - 5)
            budget = 250
            while (len(seen) < target or not strips) and budget > 0 and len(strips) < 400:
                slen_field = int(rng.integers(0 if allow_len0 else 1, 24))
                slen_field = min(slen_field, budget)
                toks = []

                def pick():
                    unseen = [i for i in range(target) if i not in seen]
                    if fifo and rng.uniform() < 0.4:
                        fi = int(rng.integers(0, len(fifo)))
                        v = fifo[fi]
                        tok = (0, fi)
                    else:
                        if unseen and rng.uniform() < 0.8:
                            v = int(unseen[int(rng.integers(0, len(unseen)))])
                        else:
                            v = int(rng.integers(0, target))
                        tok = (1, v)
                    if v in fifo:
                        fifo.remove(v)
                    fifo.append(v)
                    if len(fifo) > 16:
                        fifo.pop(0)
                    return v, tok

                r = []
                for _ in range(3):
                    v, t = pick()
                    r.append((v, t))
                toks += [t for _, t in r]
                prev = [v for v, _ in r]
                for v in prev:
                    if v not in seen:
                        walk.append((v, "none", ()))
                        seen.add(v)
                tris = 1
                for _ in range(slen_field - 1):
                    ec = int(rng.integers(0, 2))
                    nv, tok = pick()
                    if ec == 0:
                        a, b, c = prev[1], prev[2], prev[0]
                    else:
                        a, b, c = prev[0], prev[2], prev[1]
                    toks.append(("e", ec))
                    toks.append(tok)
                    if nv not in seen:
                        walk.append((nv, "para", (a, b, c)))
                        seen.add(nv)
                    prev = [a, b, nv]
                    tris += 1
                strips.append((slen_field, toks, tris))
                budget -= tris
        n_tris = sum(s[2] for s in strips)
        total_tris += n_tris
        total_local += n_local
        body.write_fixed(n_local, 16)
        body.write_fixed(n_tris, 16)
        body.write_fixed(len(strips), 16)
        for slen_field, toks, _ in strips:
            body.write_fixed(slen_field, 16)
            for t in toks:
                if t[0] == "e":
                    body.write_bits(t[1], 1)
                elif t[0] == 0:
                    body.write_bits(0, 1)
                    body.write_bits(t[1], 5)
                else:
                    body.write_bits(1, 1)
                    body.write_bits(t[1], ib)
        # --- residuals from the codes, using the decoder's walk order.
        anchor = codes[walk[0][0]] if walk else np.zeros(3, np.int64)
        deltas, paras = [], []
        prev = None
        first = True
        for v, kind, refs in walk:
            tc = codes[v]
            if kind == "none":
                if first:
                    first = False
                else:
                    deltas.append(tc - prev)
            else:
                a, b, c = refs
                pr = np.empty(3, np.int64)
                for d in range(3):
                    s = (int(pred_n[d][0]) * int(codes[a][d]) + int(pred_n[d][1]) * int(codes[b][d])
                         + int(pred_n[d][2]) * int(codes[c][d]))
                    K = int(pred_K[d])
                    pr[d] = s if K == 0 else (s + (1 << (K - 1))) >> K
                paras.append(tc - pr)
            prev = tc
        for d in range(3):
            body.write_fixed(int(anchor[d]), int(g_bits[d]))
        tk = []
        for _ in range(6):
            tag = int(rng.choice([0, 1, 1, 2, 3]))
            k = int(rng.integers(0, 3 if big_residuals else 12))
            tk.append((tag, k))
        for tag, k in tk:
            body.write_fixed(tag, 8)
            body.write_fixed(k, 8)
        streams = [(np.array(deltas, np.int64).reshape(-1, 3), 0),
                   (np.array(paras, np.int64).reshape(-1, 3), 3)]
        for arr, base in streams:
            for d in range(3):
                tag, k = tk[base + d]
                for i in range(arr.shape[0]):
                    u = int(arr[i, d])
                    u = (u << 1) if u >= 0 else ((-u) << 1) - 1
                    if tag == 1:
                        body.write_rice(u, k)
                    else:
                        body.write_exp_golomb(u, k)
    body_bytes = body.finalize()
    w = BitWriter()
    w.write_fixed(0x44505234, 32)
    w.write_fixed(3, 8)
    w.write_fixed(0, 8)
    for c in center:
        w.write_f32(float(c))
    w.write_f32(float(scale))
    w.write_f32(0.001)
    for v in g_min:
        w.write_f32(float(v))
    for v in g_range:
        w.write_f32(float(v))
    for b in g_bits:
        w.write_fixed(int(b), 8)
    for d in range(3):
        for j in range(3):
            w.write_fixed(int(pred_n[d][j]) & 0xFFFF, 16)
    for d in range(3):
        w.write_fixed(int(pred_K[d]) & 0xFF, 8)
    w.write_fixed(total_local, 32)
    w.write_fixed(total_tris, 32)
    w.write_fixed(n_meshlets, 32)
    start = w.bit_pos() + 32 * n_meshlets
    for o in offs:
        w.write_fixed(start + o, 32)
    return w.finalize() + body_bytes


def crafted_case(ref, name, seed, **kw):
    _, _, decode_dup, BitWriter = ref
    rng = np.random.default_rng(seed)
    data = craft_stream(BitWriter, rng, **kw)
    V, T = decode_dup(data)
    meta = dict(kind="crafted", seed=seed, bytes=len(data),
                **{k: (v if not isinstance(v, np.ndarray) else v.tolist()) for k, v in kw.items()})
    print(f"{name}: n_v={len(V)} n_t={len(T)} bytes={len(data)}")
    _save(name, data, V, T, None, meta, True)


def bitcodec_case(ref):
    """Known-answer vectors of the reference bit codec (its import self-test,
    utils/bit_codec.py:262-288, plus Rice/EG values with long prefixes)."""
    _, _, _, BitWriter = ref
    w = BitWriter()
    ops = []
    w.write_fixed(0xABCD, 16); ops.append(("fixed", 16, 0xABCD))
    for u, k in ((0, 3), (1, 0), (42, 4), (1000, 2), (77, 0), (5, 11)):
        w.write_rice(u, k); ops.append(("rice", k, u))
    for u, k in ((0, 0), (7, 2), (123456, 3), (1, 7), (65535, 0)):
        w.write_exp_golomb(u, k); ops.append(("eg", k, u))
    w.write_zigzag(-12345, 16); ops.append(("fixed", 16, ((12345) << 1) - 1))
    w.write_f32(3.14159); ops.append(("fixed", 32, int(np.float32(3.14159).view(np.uint32))))
    data = w.finalize()
    np.savez_compressed(os.path.join(HERE, "bitcodec.npz"),
                        blob=np.frombuffer(data, dtype=np.uint8),
                        ops=np.array(json.dumps(ops)))
    print("bitcodec: ", len(ops), "ops")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="skip the 129x129 cases")
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    ref = _import_reference()
    only = set(args.only.split(",")) if args.only else None

    def want(n):
        return only is None or n in only

    if want("bitcodec"):
        bitcodec_case(ref)
    b12 = synth.bbox_bits_error(12)
    if want("tri1_b12"):
        V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.25]], dtype=np.float64)
        mesh_case(ref, "tri1_b12", V, np.array([[0, 1, 2]]), precision_error=b12,
                  precision_mode="bbox_frac")
    if want("grid9_b12"):
        V, T = synth.heightfield_grid(9, seed=11)
        mesh_case(ref, "grid9_b12", V, T, precision_error=b12, precision_mode="bbox_frac")
    if want("grid33_b12"):
        V, T = synth.heightfield_grid(33, seed=12)
        mesh_case(ref, "grid33_b12", V, T, precision_error=b12, precision_mode="bbox_frac")
    if want("grid17_canon_b16"):
        V, T = synth.heightfield_grid(17, seed=13)
        mesh_case(ref, "grid17_canon_b16", V, T, precision_error=synth.bbox_bits_error(16),
                  precision_mode="bbox_frac", predictor="canonical")
    if want("ico3_b12"):
        V, T = synth.icosphere(3, seed=14)
        mesh_case(ref, "ico3_b12", V, T, precision_error=b12, precision_mode="bbox_frac")
    if want("torus_b10"):
        V, T = synth.torus(24, 12, R=3.0, r=1.0)
        mesh_case(ref, "torus_b10", V, T, precision_error=synth.bbox_bits_error(10),
                  precision_mode="bbox_frac")
    if want("grid65_world"):
        V, T = synth.heightfield_grid(65, seed=15)
        mesh_case(ref, "grid65_world", V, T, precision_error=0.0005, precision_mode="world")
    if want("crafted_a"):
        crafted_case(ref, "crafted_a", 101, n_meshlets=5, g_bits=[12, 12, 11],
                     pred_n=[[1, 1, -1]] * 3, pred_K=[0, 0, 0])
    if want("crafted_b"):
        crafted_case(ref, "crafted_b", 102, n_meshlets=7, g_bits=[16, 0, 9],
                     pred_n=[[40, 37, -13], [-3, 70, -2], [33, 33, -2]], pred_K=[6, 6, 6],
                     allow_unvisited=True, allow_empty=True, allow_len0=True)
    if want("crafted_c"):
        crafted_case(ref, "crafted_c", 103, n_meshlets=4, g_bits=[14, 14, 14],
                     pred_n=[[200, 200, -145], [1, 1, -1], [-64, 300, 20]], pred_K=[8, 0, 9],
                     big_residuals=True, max_local=40)
    if not args.quick:
        if want("grid129_b12"):
            V, T = synth.heightfield_grid(129, seed=1)
            mesh_case(ref, "grid129_b12", V, T, precision_error=b12,
                      precision_mode="bbox_frac", full=False)
        if want("grid129_world"):
            V, T = synth.heightfield_grid(129, seed=1)
            mesh_case(ref, "grid129_world", V, T, precision_error=0.0005,
                      precision_mode="world", full=False)


if __name__ == "__main__":
    main()
