"""A model of resolving the connectivity FIFO 32 tokens at a time, checked
against the oracle on the golden streams.

The 16-entry move-to-tail FIFO of the connectivity tokens (_read_vert,
encoder/paradelta_codec.py:330-340) is held right-aligned here: slot 15 the
newest entry, slots 16 - len .. 15 valid.  When a raw token's id is not in
the FIFO -- what an encoder writes, and what the kernels' fast pass assumes
and checks -- every token changes the slots by a map that depends on no id:
a raw token moves every slot down by one and enters at slot 15; a FIFO
token with index fi moves slot 16 - len + fi to slot 15, len being the
number of raw tokens before it (at most 16).  Maps compose, so a warp could
resolve a window of 32 tokens by a five-step prefix over slot maps and then
every FIFO token's id by one lookup.  This test runs that model, window by
window with the prefix a warp would take, on every meshlet of the golden
streams (made by the reference encoder) and compares every token's id with
the triangles the oracle decodes; a meshlet whose raw id is still in the
FIFO must be detected by the model and confirmed by the sequential FIFO.
"""
import numpy as np
import pytest

import oracle
from tests import _golden

FIFO = 16
WINDOW = 32


class Bits:
    """MSB-first bit reader over bytes (utils/bit_codec.py's order)."""

    def __init__(self, data: bytes, pos: int):
        self.v = int.from_bytes(data, "big")
        self.n = 8 * len(data)
        self.pos = pos

    def read(self, k: int) -> int:
        self.pos += k
        return (self.v >> (self.n - self.pos)) & ((1 << k) - 1)


def meshlet_tokens(data: bytes, start_bit: int):
    """Tokens of one meshlet: (raw, value, strip, position in the strip)."""
    r = Bits(data, start_bit)
    n_local = r.read(16)
    r.read(16)
    n_strips = r.read(16)
    ib = max(1, n_local.bit_length())
    toks = []
    for st in range(n_strips):
        strip_len = r.read(16)
        for j in range(3 + max(strip_len - 1, 0)):
            if j >= 3:
                r.read(1)  # edge code
            raw = r.read(1) == 1
            toks.append((raw, r.read(ib) if raw else r.read(5), st, j))
    return n_local, toks


def compose(g, f):
    """g after f: slot s of the result takes f's source for g's slot."""
    return [f[x] if x < FIFO else x for x in g]


def resolve_by_slot_maps(toks):
    """Ids of every token from slot maps (sources: a slot of the window's
    entry state, or FIFO + the index of a raw token), or None for a token
    whose raw id is already held (a suspect meshlet)."""
    state = [None] * FIFO  # ids at the window's start, right-aligned
    n_raw = 0
    out = []
    for w0 in range(0, len(toks), WINDOW):
        win = toks[w0:w0 + WINDOW]
        maps, lens = [], []
        for t, (raw, val, _, _) in enumerate(win):
            length = min(FIFO, n_raw)
            lens.append(length)
            if raw:
                m = list(range(1, FIFO)) + [FIFO + t]
                n_raw += 1
            else:
                at = FIFO - length + val
                m = [s if s < at else s + 1 for s in range(FIFO - 1)] + [at]
            maps.append(m)
        # inclusive prefix, five Hillis-Steele steps as a warp would take them
        pre = [list(m) for m in maps]
        step = 1
        while step < len(win):
            pre = [compose(pre[t], pre[t - step]) if t >= step else pre[t] for t in range(len(win))]
            step *= 2
        ident = list(range(FIFO))

        def ids_of(src):
            return [state[x] if x < FIFO else win[x - FIFO][1] for x in src]

        for t, (raw, val, _, _) in enumerate(win):
            before = ids_of(pre[t - 1] if t else ident)
            if raw:
                held = val in before[FIFO - lens[t]:]
                out.append(None if held else val)
            else:
                assert val < lens[t], "FIFO index past the entries"
                out.append(before[FIFO - lens[t] + val])
        state = ids_of(pre[-1])
    return out


def resolve_sequentially(toks):
    """The reference FIFO, one token after another; also whether a raw id
    was already held."""
    fifo, out, held_raw = [], [], False
    for raw, val, _, _ in toks:
        v = val if raw else fifo[val]
        if raw and v in fifo:
            held_raw = True
        if v in fifo:
            fifo.remove(v)
        elif len(fifo) == FIFO:
            fifo.pop(0)
        fifo.append(v)
        out.append(v)
    return out, held_raw


def ids_from_triangles(idx, toks, t_base, v_base):
    """Each token's id as the oracle's triangles hold it: a strip's three
    roots are its first triangle, each later token the third vertex of its
    triangle."""
    out, t = [], t_base - 1
    for _, _, _, j in toks:
        if j == 0:
            t += 1
        if j < 3:
            out.append(int(idx[t][j]) - v_base)
        else:
            t += 1
            out.append(int(idx[t][2]) - v_base)
    return out


HEADER_BYTES = 86  # the offset table follows: one big-endian bit offset per meshlet


@pytest.mark.parametrize("name", _golden.names())
def test_slot_map_resolution_matches_the_oracle(name):
    oracle.build()
    data = _golden.load(name)["data"]
    n_meshlets = oracle.parse_header(data).n_meshlets
    starts = np.frombuffer(data, ">u4", count=n_meshlets, offset=HEADER_BYTES)
    _, idx = oracle.decode(data)
    v_base = t_base = 0
    suspects = tokens = 0
    for m in range(n_meshlets):
        n_local, toks = meshlet_tokens(data, int(starts[m]))
        model = resolve_by_slot_maps(toks)
        seq, held_raw = resolve_sequentially(toks)
        assert seq == ids_from_triangles(idx, toks, t_base, v_base)  # the sequential FIFO is the oracle's
        if None in model:  # detected by the model, and real
            assert held_raw
            suspects += 1
        else:
            assert not held_raw and model == seq
        tokens += len(toks)
        v_base += n_local
        t_base += sum(1 for _, _, _, j in toks if j == 0 or j >= 3)
    assert t_base == len(idx) and v_base == oracle.parse_header(data).n_v_total
    assert tokens > 0 and suspects <= n_meshlets


def encoder_tokens(ids, held_raw_at=()):
    """Tokens an encoder writes for this id sequence: a FIFO index for an id
    the FIFO holds, else the raw id; at the positions in `held_raw_at` the
    raw id even though the FIFO holds it."""
    fifo, toks = [], []
    for k, v in enumerate(ids):
        if v in fifo and k not in held_raw_at:
            toks.append((False, fifo.index(v), 0, 3))
        else:
            toks.append((True, v, 0, 3))
        if v in fifo:
            fifo.remove(v)
        elif len(fifo) == FIFO:
            fifo.pop(0)
        fifo.append(v)
    return toks


def test_slot_maps_on_long_random_walks():
    """Seeded id sequences with heavy reuse and eviction across many
    windows: the model equals the sequential FIFO, and a raw id the FIFO
    still holds is always caught."""
    rng = np.random.default_rng(7)
    caught = 0
    for trial in range(200):
        n_ids = int(rng.integers(2, 64))
        ids = [int(x) for x in rng.integers(0, n_ids, int(rng.integers(1, 400)))]
        toks = encoder_tokens(ids)
        seq, held = resolve_sequentially(toks)
        assert seq == ids and not held
        assert resolve_by_slot_maps(toks) == ids
        hits = [k for k, t in enumerate(toks) if not t[0]]
        if hits:
            at = int(rng.choice(hits))
            bad = encoder_tokens(ids, held_raw_at={at})
            seq, held = resolve_sequentially(bad)
            assert held and None in resolve_by_slot_maps(bad)
            caught += 1
    assert caught > 100
