"""Mesh checks shared by the tests: triangle sets, crack-freeness, closedness."""
import numpy as np


def sorted_tris(T):
    s = np.sort(np.asarray(T, dtype=np.int64), axis=1)
    return s[np.lexsort(s.T[::-1])]


def same_triangle_set(src_tris, dec_idx, l2g):
    """Decoded triangles, mapped back to source vertex ids, equal the source
    triangles as unordered triples (winding is not preserved by STRIDE)."""
    return np.array_equal(sorted_tris(src_tris), sorted_tris(np.asarray(l2g, np.int64)[dec_idx]))


def crack_free(pos, l2g):
    """Every copy of a source vertex decodes to the same float32 bit pattern."""
    order = np.argsort(l2g, kind="stable")
    g = np.asarray(l2g)[order]
    p = np.ascontiguousarray(pos[order]).view(np.uint32)
    same_src = g[1:] == g[:-1]
    return bool(np.all(p[1:][same_src] == p[:-1][same_src]))


def welded_is_closed_manifold(pos, idx):
    """Weld vertices by exact bit pattern; every edge must have exactly two
    triangles (closed 2-manifold)."""
    bits = np.ascontiguousarray(pos).view(np.uint32)
    _, weld = np.unique(bits, axis=0, return_inverse=True)
    weld = weld.reshape(-1)
    t = weld[np.asarray(idx, np.int64)]
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    e.sort(axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    return bool(np.all(counts == 2))
