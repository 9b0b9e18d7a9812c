// STRIDE (DPR4 v3) group kernel: one warp decodes a group of 32 meshlets
// from the bytes to positions and triangle indices, one lane per meshlet,
// with no other warp involved (launch shape `persistent == 3`).
//
// Per group the warp runs
//
//  1. connectivity: each lane streams its meshlet through a 256-byte ring in
//     shared memory (16-byte cp.async, L2 only) and runs decode_dup's strip
//     loop (encoder/paradelta_v5_dup.py:513-542) one token per iteration:
//     strip headers, token widths, the 16-entry move-to-tail FIFO
//     (_read_vert, encoder/paradelta_codec.py:330-340), triangles and first
//     occurrences.  Triangles and walk entries collect in 16-entry rings
//     that go out as 16-byte quads every eight tokens.
//
//  2. vertices: the lane's residual bits are already in its ring; the lane
//     reads the anchor and the six (tag, k) pairs, skips the three delta
//     substreams to reach px, then reconstructs axis x, y and z in turn in
//     walk order (IRLP, paradelta_v5_dup.py:91-104 and 581-600).  The axes run
//     one after another because each axis' two cursors end where the next
//     axis' substreams begin (dx -> dy -> dz, px -> py -> pz): only the
//     three delta substreams are ever skipped.  After each axis the warp
//     writes that coordinate of the group's vertices, meshlet by meshlet,
//     with exact dequantisation (stride_dequant.h).
//
// The FIFO is a 16-byte move-to-front register (depth 0 = newest): a FIFO
// token moves its entry to the front, a raw token pushes its id.  A raw id
// that is still in the FIFO must move instead of being pushed; encoders
// never write one (the reference's _emit_vert uses the FIFO whenever it
// holds the id, encoder/paradelta_codec.py:219-229), so the warp runs a fast
// pass that pushes every raw id and keeps an "in FIFO" flag per local id;
// a lane whose raw token finds its flag set is decoded again by an exact
// pass that searches the FIFO on every raw token.  Both passes produce
// decode_dup's results on every stream decode_dup accepts.
#include <cuda_runtime.h>

#include <algorithm>

#include "stride_common.cuh"
#include "stride_device.cuh"
#include "stride_gb300.h"

namespace stride {
namespace {

// ---------------------------------------------------------------------------
// Per-warp shared memory.  Connectivity: byte rings | flags | triangle ring |
// walk ring.  Vertices: byte rings (the residual bits) | code planes.
// ---------------------------------------------------------------------------
constexpr uint32_t kGRing = 16u;              // triangle / walk ring entries per lane
constexpr uint32_t kGRow = kGRing + 4u;       // ring row in words (quads stay 16-byte aligned)
constexpr uint32_t kGBlock = 8u;              // tokens between flushes: a partial quad + 8 fit 16
constexpr uint32_t kGFlagStride = 260u;       // bytes per lane: 256 flags, odd word count
constexpr uint32_t kGRingBytes = 32u * kLaneRingWords * 4u;
constexpr uint32_t kGWorkBytes = 32u * kGFlagStride + 2u * 32u * kGRow * 4u;
constexpr uint32_t kGWarpBytes = kGRingBytes + kGWorkBytes;  // 21,632 bytes

// ---------------------------------------------------------------------------
// Residual reader over the stream in global memory: peek(pos) = the 32 bits
// from stream bit pos.
// ---------------------------------------------------------------------------
struct GlobRd {
    const uint32_t* w;  // the stream's first byte (16-byte aligned)
    __device__ __forceinline__ uint32_t peek(uint32_t pos) const { return peek32<false>(w, pos); }
};

// One Rice(k) / Exp-Golomb(k) codeword of any length (utils/bit_codec.py:
// 226-250); tk bit 7 selects Exp-Golomb, bits 0..5 hold k.
template <class R>
__device__ int read_code_any(const R& rd, uint32_t& pos, uint32_t tk, uint32_t limit, uint32_t& u) {
    const bool eg = (tk & 0x80u) != 0u;
    const uint32_t k = tk & 0x3Fu;
    const uint32_t x = rd.peek(pos);
    uint32_t z;
    if (x != 0u) {
        z = __clz(x);
    } else {  // unary prefix of 32 or more zeros
        z = 32u;
        for (;;) {
            if (pos + z >= limit) return kErrCorrupt;
            const uint32_t y = rd.peek(pos + z);
            if (y) {
                z += __clz(y);
                break;
            }
            z += 32u;
        }
    }
    const uint32_t nb = (eg ? z : 0u) + k;  // value bits after the terminating one
    if (nb > 32u) return kErrUnsupported;
    const uint32_t p1 = pos + z + 1u;
    uint32_t val = 0u;
    if (nb) val = (z + 1u + nb <= 32u) ? (x << (z + 1u)) >> (32u - nb) : rd.peek(p1) >> (32u - nb);
    const unsigned long long base = eg ? ((1ull << z) - 1ull) : static_cast<unsigned long long>(z);
    const unsigned long long uu = (base << k) + val;
    if (uu >> 32) return kErrUnsupported;
    pos = p1 + nb;
    if (pos > limit) return kErrCorrupt;
    u = static_cast<uint32_t>(uu);
    return 0;
}

// A codeword that fits the 32-bit window (prefix, terminator and value),
// without a branch; a longer one sets `longc` and leaves r undefined.
template <class R>
__device__ __forceinline__ bool code_fast(const R& rd, uint32_t& pos, uint32_t tk, uint32_t limit, int32_t& r,
                                          bool& longc) {
    const uint32_t x = rd.peek(pos);
    const uint32_t z = __clz(x);
    const uint32_t k = tk & 0x3Fu;
    const bool eg = (tk & 0x80u) != 0u;
    const uint32_t nb = (eg ? z : 0u) + k;
    const uint32_t len = z + 1u + nb;
    const uint32_t t = __funnelshift_lc(0u, x, z + 1u);      // bits after the terminator
    const uint32_t val = __funnelshift_rc(t, 0u, 32u - nb);  // the top nb of them
    const uint32_t base = eg ? ((1u << (z & 31u)) - 1u) : z;
    const uint32_t u = (base << k) + val;
    const uint32_t np = pos + len;
    longc = longc | (len > 32u);
    const bool ok = np <= limit;
    pos = min(np, limit);
    r = unzigzag(u);
    return ok;
}

// Any codeword: the fast form, the general reader behind a branch.
template <class R>
__device__ __forceinline__ bool code_any(const R& rd, uint32_t& pos, uint32_t tk, uint32_t limit, int32_t& r) {
    bool longc = false;
    uint32_t p = pos;
    bool ok = code_fast(rd, p, tk, limit, r, longc);
    if (longc) {
        p = pos;
        uint32_t u = 0u;
        ok = read_code_any(rd, p, tk, limit, u) == 0;
        r = unzigzag(u);
    }
    pos = min(p, limit);
    return ok;
}

// Skip n codewords: Rice(0) codewords by counting one bits (each ends at
// one), others one at a time.
template <class R>
__device__ __forceinline__ bool skip_any(const R& rd, uint32_t& pos, uint32_t tk, uint32_t n, uint32_t limit) {
    if (tk == 0u) {  // Rice(0)
        while (n > 0u) {
            const uint32_t x = rd.peek(pos);
            const uint32_t c = __popc(x);
            if (c < n) {
                pos += 32u;
                n -= c;
            } else {
                uint32_t y = x, at = 0u, need = n;
#pragma unroll
                for (uint32_t wd = 16u; wd >= 1u; wd >>= 1) {
                    const uint32_t t = __popc(y >> (32u - wd));  // ones in the top wd bits
                    const bool skip = t < need;
                    need -= skip ? t : 0u;
                    y = skip ? (y << wd) : y;
                    at += skip ? wd : 0u;
                }
                pos += at + 1u;  // through the n-th one
                n = 0u;
            }
            if (pos > limit) {
                pos = limit;
                return false;
            }
        }
        return true;
    }
    for (; n > 0u; n--) {
        int32_t r;
        if (!code_any(rd, pos, tk, limit, r)) return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// 1. connectivity of the warp's lanes
// ---------------------------------------------------------------------------
struct GLane {
    GroupLane L;
    uint32_t s0lo;      // low bits of the lane's 16-byte aligned first byte (arena offset)
    uint32_t rot;       // ring rotation (words)
    uint32_t anchor;    // first bit after the connectivity
    uint32_t kind0, n_walk;
    bool bad, suspect;
};

// Ring chunk c of the lane (its data starts at arena offset s0).
__device__ __forceinline__ void gfetch(const DecodeArgs& a, uint32_t* ring, unsigned long long s0, uint32_t avail,
                                       uint32_t rot, uint32_t c) {
    ring_fetch(ring, a.arena + s0, avail, rot, c);
}

// Word r (rotated index) of a lane's byte ring, in bit order.
__device__ __forceinline__ uint32_t ring_word(const uint32_t* ring, uint32_t r) {
    return bswap32(ring[r & (kLaneRingWords - 1u)]);
}

// Connectivity of the warp's lanes, one token per iteration.  Validity is
// checked lazily: out-of-range ids and FIFO indices are folded into a
// running max / min, the position and the counts are compared once at the
// end, and the output flushes never write past the meshlet's triangles or
// walk entries, so a corrupt lane runs on harmlessly until its count is
// used up and is then rejected.
template <bool kExact>
__device__ __forceinline__ void gconn(const DecodeArgs& a, GLane& G, bool act, uint32_t* __restrict__ ring,
                                      uint8_t* __restrict__ flags, uint32_t* __restrict__ tr,
                                      uint32_t* __restrict__ wr, const uint4* __restrict__ mtf_masks) {
    const GroupLane& L = G.L;
    const uint32_t n_local = L.d.counts0 & 0xFFFFu;
    const uint32_t n_tris = L.d.counts0 >> 16;
    const uint32_t ib = max(1u, 32u - __clz(n_local));  // _idx_bits_for (paradelta_codec.py:124-125)
    const uint32_t rsh = 32u - ib, ib1 = 1u + ib;
    const uint32_t end = L.d.end_bit;
    const unsigned long long s0 = (L.blob_off + (L.d.start_bit >> 3)) & ~15ull;
    const unsigned long long e16 = (L.blob_off + ((end + 7u) >> 3) + 15ull) & ~15ull;
    const uint32_t avail = act ? static_cast<uint32_t>(e16 - s0) : 0u;
    const uint32_t rot = G.rot;
    const uint32_t base0 = static_cast<uint32_t>((s0 - L.blob_off) * 8ull);  // stream bit of the lane's data bit 0
    if (act) {  // flags of the lane's local ids (a valid token's id is below n_local)
        for (uint32_t i = 0; i < (n_local + 3u) >> 2; i++) reinterpret_cast<uint32_t*>(flags)[i] = 0u;
        gfetch(a, ring, s0, avail, rot, 0u);
        gfetch(a, ring, s0, avail, rot, 1u);
    }
    cp_async_wait_all();
    uint32_t req = 2u;
    // bit window: words wi, wi+1, wi+2 of the lane's data (in bit order) in
    // w0, w1, w2; `off` bits of w0 consumed; ri = rotated ring index of wi+2
    const uint32_t q0 = act ? L.d.start_bit + 48u - base0 : 0u;
    uint32_t wi = q0 >> 5, off = q0 & 31u;
    uint32_t ri = wi + 2u + rot;
    uint32_t w0 = ring_word(ring, ri - 2u), w1 = ring_word(ring, ri - 1u), w2 = ring_word(ring, ri);
    uint32_t* walk_out = a.walk_scratch + L.wp_base;
    const uint32_t vloc = act ? static_cast<uint32_t>(L.v_base - L.P->v_offset) : 0u;
    const uint32_t ph = static_cast<uint32_t>(L.t_base) & 3u;  // ring slot of triangle 0
    uint32_t sl = L.d.n_strips;  // strips left
    uint32_t tl = 0u;            // tokens left in the strip
    uint32_t tx = 0u;            // position of the next token in its strip: 0..2 roots, 3 body
    uint32_t P = 0u;             // strip state p0 | p1 << 8 | p2 << 16
    uint32_t tcnt = 0u, wcnt = 0u, kind0 = 0u, tf = 0u, wf = 0u;
    uint32_t ridmax = 0u, flacc = 0u;
    int32_t smin = 0;
    MtfFifo fifo;
    // `live` turns false for good once the lane's strips are read: past that
    // a lane keeps running the loop body on whatever bits follow (no branch
    // per token, so the compiler can overlap consecutive tokens' chains),
    // but commits nothing -- no output, no count, no window movement
    bool live = act && sl > 0u;
    // n_tris + 2 n_strips iterations finish (or fail) every lane; the warp
    // runs whole blocks of kGBlock tokens
    const uint32_t iters = __reduce_max_sync(kFull, act ? n_tris + 2u * L.d.n_strips : 0u);
    for (uint32_t it = 0u; it < iters; it += kGBlock) {
#pragma unroll
        for (uint32_t i = 0; i < kGBlock; i++) {
            // a 32-bit window holds a strip header (16 bits) plus the next
            // token (at most 1 + 9 bits), or an edge code plus a token
            const uint32_t x0 = __funnelshift_l(w1, w0, off);
            const bool hdr = tl == 0u;  // strip header (paradelta_v5_dup.py:519)
            const uint32_t sb = max(x0 >> 16, 1u) - 1u;  // body tokens of the strip
            tl = hdr ? sb + 3u : tl;
            sl -= hdr ? 1u : 0u;
            const uint32_t tix = hdr ? 0u : tx;
            uint32_t x = hdr ? (x0 << 16) : x0;
            uint32_t used = hdr ? 16u : 0u;
            const bool body = tix == 3u;
            const uint32_t ec = x >> 31;  // edge code of a strip-body token (:528)
            x = body ? (x << 1) : x;
            used += body ? 1u : 0u;
            const bool raw = static_cast<int32_t>(x) < 0;
            const uint32_t y = x << 1;
            const uint32_t rid = y >> rsh;
            const uint32_t fi = y >> 27;
            used += raw ? ib1 : 6u;
            // decode_dup raises IndexError on a FIFO index past the entries
            // and on a local id past n_local: kept as a running min / max
            const int32_t sd = static_cast<int32_t>(fifo.len) - 1 - static_cast<int32_t>(fi);
            const bool rl = raw & live;
            smin = min(smin, (raw | !live) ? 0 : sd);
            ridmax = max(ridmax, rl ? rid + 1u : 0u);  // 0: no raw token
            const uint32_t s = static_cast<uint32_t>(sd) & 15u;  // depth of a FIFO token's entry
            const uint32_t v = raw ? (rid & 0xFFu) : fifo.at(s);
            const uint32_t ev = fifo.f3 >> 24;  // depth 15: leaves when a new id enters a full FIFO
            bool fresh = raw;                  // a raw id not in the FIFO
            uint32_t p;
            if constexpr (kExact) {
                const uint32_t at = raw ? fifo.find(v) : 16u;
                fresh = raw & (at == 16u);
                p = raw ? (fresh ? min(fifo.len, 15u) : at) : s;
            } else {
                p = raw ? min(fifo.len, 15u) : s;
            }
            fifo.mtf_masked(v, mtf_masks[p]);
            const bool evict = fresh & (fifo.len == 16u);
            fifo.len += (fresh & (fifo.len < 16u)) ? 1u : 0u;
            // flags: bit 0 the id has occurred, bit 1 it is in the FIFO
            // (fast pass); a FIFO token's id has always occurred
            const uint32_t fl = flags[v];
            const bool isnew = rl & ((fl & 1u) == 0u);
            if constexpr (!kExact) {
                flacc |= rl ? fl : 0u;  // bit 1: a raw id found in the FIFO
                if (evict) flags[ev] = 1u;
                if (raw) flags[v] = 3u;
            } else {
                if (raw) flags[v] = 1u;
            }
            // strip state, triangle and first occurrence (:523-541): edge
            // code 0 -> (p1, p2 | p0), 1 -> (p0, p2 | p1); a root token
            // puts v at byte tix
            const uint32_t sel = body ? (0x7421u ^ ec) : (0x7210u + ((4u - tix) << (4u * tix)));
            const uint32_t cref = __byte_perm(P, 0u, 0x4440u | ec);
            const uint32_t Pn = __byte_perm(P, v, sel);
            const bool emit = (tix >= 2u) & live;
            if (emit) tr[(ph + tcnt) & (kGRing - 1u)] = Pn;
            tcnt += emit ? 1u : 0u;
            // roots are 'none' (stored as v,v,v,v); strip bodies 'para' with
            // (a, b, c) = (p0, p1, cref) of the new strip state
            const uint32_t e = body ? __byte_perm(Pn, cref, 0x4102u) : __byte_perm(v, 0u, 0u);
            if (isnew) wr[wcnt & (kGRing - 1u)] = e;
            wcnt += isnew ? 1u : 0u;
            kind0 += (isnew & !body) ? 1u : 0u;
            P = Pn;
            tl--;
            tx = min(tix + 1u, 3u);
            // advance: at most one word boundary per token (used <= 26)
            off += live ? used : 0u;
            const bool cross = off >= 32u;
            off &= 31u;
            ri += cross ? 1u : 0u;
            const uint32_t nw = ring_word(ring, ri);
            w0 = cross ? w1 : w0;
            w1 = cross ? w2 : w1;
            w2 = cross ? nw : w2;
            live = live & ((tl | sl) != 0u);
        }
        if (act) {  // never past the meshlet's triangles or walk entries
            flush_tris<kGRing>(a.idx, L.t_base, tr, tf, min(tcnt, n_tris), vloc, false);
            flush_walk<kGRing>(walk_out, wr, wf, min(wcnt, n_local), false);
        }
        if (((it / kGBlock) & 1u) != 0u && it + kGBlock < iters) {
            // every 16 tokens (at most 13 words): the refill issued 16 tokens
            // ago has landed; fetch one more chunk when fewer than 33 words
            // lie ahead of the window's next load
            cp_async_wait_all();
            if (live && kLaneChunkWords * req < ri - rot + 34u) {
                gfetch(a, ring, s0, avail, rot, req);
                req++;
            }
            cp_async_commit();
        }
    }
    const bool running = live;
    cp_async_wait_all();
    if (act) {
        flush_tris<kGRing>(a.idx, L.t_base, tr, tf, min(tcnt, n_tris), vloc, true);
        flush_walk<kGRing>(walk_out, wr, wf, min(wcnt, n_local), true);
        const uint32_t anchor = base0 + 32u * (ri - 2u - rot) + off;
        G.anchor = anchor;
        G.kind0 = kind0;
        G.n_walk = wcnt;
        // every strip read, exactly n_tris triangles, ids and FIFO indices in
        // range, and the connectivity inside the meshlet
        G.bad = running || tcnt != n_tris || smin < 0 || ridmax > n_local || anchor > end;
        G.suspect = (flacc & 2u) != 0u;
    }
}

// ---------------------------------------------------------------------------
// 2. vertices
// ---------------------------------------------------------------------------
// A lane's residual bits, copied to a linear stage in bit order: word j at
// st[j]; positions are bits from the stage start.
struct LinRd {
    const uint32_t* st;
    __device__ __forceinline__ uint32_t peek(uint32_t p) const {
        return __funnelshift_l(st[(p >> 5) + 1u], st[p >> 5], p);  // the shift is p mod 32
    }
};

// Integer codes of axis d in walk order into `plane`: every walk vertex is a
// root (delta from the previous walk vertex; the first one is the anchor)
// or a parallelogram vertex predicted from three earlier ones.  cd / cp are
// the axis' delta and parallelogram cursors; they end at the next axis'
// substreams.  Codewords are read with a branch-free reader that fits them
// in one 32-bit window; validity (codes in range, codewords that fit) is
// folded into running maxima and checked after the loop -- a lane whose
// longest codeword did not fit walks the axis again with the general
// reader.  Four walk entries per 16-byte load, two loads in flight.
struct AxisCode {
    int32_t n0, n1, n2, K, half, anc;
    uint32_t cmax;
    uint32_t kd, kp;    // Rice / Exp-Golomb parameter of the delta / parallelogram substream
    uint32_t egd, egp;  // all ones for Exp-Golomb
};

template <bool kWide>
__device__ __forceinline__ bool gwalk_lin(const LinRd& rd, const AxisCode& c, const uint4* __restrict__ wq,
                                          uint32_t n_walk, uint32_t n_local, PlaneT<kWide>* __restrict__ plane,
                                          uint32_t lim, uint32_t& cd, uint32_t& cp) {
    if (n_walk < n_local) {  // vertices the walk never reaches keep code 0
        uint32_t* z = reinterpret_cast<uint32_t*>(plane);
        const uint32_t nz = (n_local * static_cast<uint32_t>(sizeof(PlaneT<kWide>)) + 3u) >> 2;
        for (uint32_t i = 0; i < nz; i++) z[i] = 0u;
    }
    if (n_walk == 0u) return true;
    const uint32_t cd0 = cd, cp0 = cp;
    int32_t prev = c.anc;
    uint32_t cmx = 0u, lmx = 0u;
    // the first walk entry is the anchor (no residual)
    uint4 q = __ldcg(wq);
    const uint32_t v0 = q.x & 0xFFu;
    plane[v0] = static_cast<PlaneT<kWide>>(c.anc);
    uint4 qn = n_walk > 4u ? __ldcg(wq + 1) : q;
    // one loop body for every entry: entry j is word j % 4 of quad j / 4,
    // the next quad in flight
    for (uint32_t j = 1u; j < n_walk; j++) {
        if ((j & 3u) == 0u) {
            q = qn;
            if (j + 4u < n_walk) qn = __ldcg(wq + (j >> 2) + 1u);
        }
        const uint32_t e = (j & 2u) ? ((j & 1u) ? q.w : q.z) : ((j & 1u) ? q.y : q.x);
        const uint32_t v = e & 0xFFu;
        const uint32_t ra = (e >> 8) & 0xFFu, rb = (e >> 16) & 0xFFu, rc = e >> 24;
        const bool para = ra != v;  // roots are stored as (v, v, v, v)
        const int32_t ca = static_cast<int32_t>(plane[ra]);
        const int32_t cb = static_cast<int32_t>(plane[rb]);
        const int32_t cc = static_cast<int32_t>(plane[rc]);
        const int32_t pr = (c.n0 * ca + c.n1 * cb + c.n2 * cc + c.half) >> c.K;
        const uint32_t p = para ? cp : cd;
        const uint32_t x = rd.peek(p);
        const uint32_t z = __clz(x);
        const uint32_t k = para ? c.kp : c.kd;
        const uint32_t eg = para ? c.egp : c.egd;
        const uint32_t nb = k + (z & eg);
        const uint32_t len = z + 1u + nb;
        const uint32_t t = __funnelshift_lc(0u, x, z + 1u);  // bits after the terminator
        const uint32_t val = __funnelshift_lc(t, 0u, nb);    // the top nb of them
        const uint32_t base = eg ? (1u << (z & 31u)) - 1u : z;
        const uint32_t u = (base << k) + val;
        lmx = max(lmx, len);
        // a cursor that overruns the meshlet stops at lim + 1, past every
        // valid end: the checks after the walk and after the last axis see it
        const uint32_t np = min(p + len, lim + 1u);
        cp = para ? np : cp;
        cd = para ? cd : np;
        const int32_t code = (para ? pr : prev) + static_cast<int32_t>((u >> 1) ^ (0u - (u & 1u)));
        cmx = max(cmx, static_cast<uint32_t>(code));
        plane[v] = static_cast<PlaneT<kWide>>(code);
        prev = code;
    }
    bool ok = cmx <= c.cmax && static_cast<uint32_t>(c.anc) <= c.cmax && max(cd, cp) <= lim;
    if (lmx > 32u) {  // rare: a codeword longer than the window; the axis again, general reader
        cd = cd0;
        cp = cp0;
        prev = c.anc;
        ok = static_cast<uint32_t>(c.anc) <= c.cmax;
        for (uint32_t j = 1u; j < n_walk && ok; j++) {
            const uint32_t e = __ldcg(reinterpret_cast<const uint32_t*>(wq) + j);
            const uint32_t v = e & 0xFFu;
            const uint32_t ra = (e >> 8) & 0xFFu, rb = (e >> 16) & 0xFFu, rc = e >> 24;
            const bool para = ra != v;
            const int32_t pr = (c.n0 * static_cast<int32_t>(plane[ra]) + c.n1 * static_cast<int32_t>(plane[rb]) +
                                c.n2 * static_cast<int32_t>(plane[rc]) + c.half) >> c.K;
            uint32_t pp = para ? cp : cd;
            int32_t r = 0;
            ok = code_any(rd, pp, para ? (c.kp | (c.egp & 0x80u)) : (c.kd | (c.egd & 0x80u)), lim, r);
            if (para) cp = pp; else cd = pp;
            const int32_t code = (para ? pr : prev) + r;
            ok = ok && static_cast<uint32_t>(code) <= c.cmax;
            plane[v] = static_cast<PlaneT<kWide>>(code);
            prev = code;
        }
    }
    return ok;
}

// The general form for lanes whose residual bits did not fit a stage:
// stream positions, any reader (global memory), every codeword through the
// branch-free reader with a branch to the general one.
template <class R, bool kWide>
__device__ __noinline__ bool gwalk_any(const R& rd, const AxisCode& c, const uint32_t* __restrict__ walk,
                                       uint32_t n_walk, uint32_t n_local, PlaneT<kWide>* __restrict__ plane,
                                       uint32_t lim, uint32_t& cd, uint32_t& cp) {
    for (uint32_t i = 0; i < n_local; i++) plane[i] = 0;
    if (n_walk == 0u) return true;
    plane[__ldcg(walk) & 0xFFu] = static_cast<PlaneT<kWide>>(c.anc);
    int32_t prev = c.anc;
    bool ok = static_cast<uint32_t>(c.anc) <= c.cmax;
    for (uint32_t j = 1u; j < n_walk && ok; j++) {
        const uint32_t e = __ldcg(walk + j);
        const uint32_t v = e & 0xFFu;
        const uint32_t ra = (e >> 8) & 0xFFu, rb = (e >> 16) & 0xFFu, rc = e >> 24;
        const bool para = ra != v;
        const int32_t pr = (c.n0 * static_cast<int32_t>(plane[ra]) + c.n1 * static_cast<int32_t>(plane[rb]) +
                            c.n2 * static_cast<int32_t>(plane[rc]) + c.half) >> c.K;
        uint32_t pp = para ? cp : cd;
        int32_t r = 0;
        ok = code_any(rd, pp, para ? (c.kp | (c.egp & 0x80u)) : (c.kd | (c.egd & 0x80u)), lim, r);
        if (para) cp = pp; else cd = pp;
        const int32_t code = (para ? pr : prev) + r;
        ok = ok && static_cast<uint32_t>(code) <= c.cmax;
        plane[v] = static_cast<PlaneT<kWide>>(code);
        prev = code;
    }
    return ok;
}

// Vertex phase of the lanes in `rmask`.  Staged lanes (kLin) read their
// residual bits from their linear stage (`sbase` = stream bit of its first
// word); the others read the stream.  Each lane: header, the skip to px,
// then axes x, y, z; after each axis the warp writes that coordinate of
// every round lane's vertices.
template <bool kLin, bool kWide>
__device__ __forceinline__ void gvert(const DecodeArgs& a, GLane& G, const uint32_t* st, uint32_t sbase, bool act,
                                      uint32_t rmask, uint8_t* planes, uint32_t code_off, int lane) {
    const GroupLane& L = G.L;
    const MeshParams* P = L.P;
    const uint32_t n_local = L.d.counts0 & 0xFFFFu;
    const uint32_t lim = L.d.end_bit - sbase;
    LinRd lr;
    lr.st = st;
    GlobRd gr;
    gr.w = reinterpret_cast<const uint32_t*>(a.arena + L.blob_off);
    int32_t anc0 = 0, anc1 = 0, anc2 = 0;
    uint32_t tk0 = 0u, tk1 = 0u, tk2 = 0u, tk3 = 0u, tk4 = 0u, tk5 = 0u;
    uint32_t cd = 0u, cp = 0u;
    bool ok = act;
    uint32_t so01 = 0xFFFFFFFFu, so23 = 0xFFFFFFFFu, so4 = 0xFFFFu;  // side table, packed
    auto peek = [&](uint32_t q) { return kLin ? lr.peek(q) : gr.peek(q); };
    if (act) {
        // anchor codes and the six (tag, k) pairs (paradelta_v5_dup.py:544-557)
        uint32_t pos = G.anchor - sbase;
        const uint32_t gb0 = __ldcg(&P->g_bits[0]), gb1 = __ldcg(&P->g_bits[1]), gb2 = __ldcg(&P->g_bits[2]);
        anc0 = gb0 ? static_cast<int32_t>(peek(pos) >> (32u - gb0)) : 0;
        pos += gb0;
        anc1 = gb1 ? static_cast<int32_t>(peek(pos) >> (32u - gb1)) : 0;
        pos += gb1;
        anc2 = gb2 ? static_cast<int32_t>(peek(pos) >> (32u - gb2)) : 0;
        pos += gb2;
        uint32_t tk[6];
#pragma unroll
        for (int i = 0; i < 6; i++) {
            const uint32_t t = peek(pos) >> 16;
            pos += 16u;
            const uint32_t k = t & 0xFFu;
            ok = ok && k <= static_cast<uint32_t>(kMaxResidK);
            tk[i] = ((t >> 8) == 1u ? 0u : 0x80u) | (k & 0x3Fu);
        }
        tk0 = tk[0]; tk1 = tk[1]; tk2 = tk[2]; tk3 = tk[3]; tk4 = tk[4]; tk5 = tk[5];
        ok = ok && pos <= lim;
        pos = min(pos, lim);
        const uint32_t n_delta = G.kind0 ? G.kind0 - 1u : 0u;  // the anchor has no delta
        cd = pos;
        cp = pos;
        if (kLin) {
            if (ok) ok = skip_any(lr, cp, tk0, n_delta, lim);
            if (ok) ok = skip_any(lr, cp, tk1, n_delta, lim);
            if (ok) ok = skip_any(lr, cp, tk2, n_delta, lim);
        } else {
            if (ok) ok = skip_any(gr, cp, tk0, n_delta, lim);
            if (ok) ok = skip_any(gr, cp, tk1, n_delta, lim);
            if (ok) ok = skip_any(gr, cp, tk2, n_delta, lim);
        }
    }
    PlaneT<kWide>* plane = reinterpret_cast<PlaneT<kWide>*>(planes + code_off);
    const uint4* wq = reinterpret_cast<const uint4*>(a.walk_scratch + L.wp_base);
    const uint32_t base = G.anchor - sbase;
    for (uint32_t d = 0; d < 3u; d++) {
        if (ok) {
            const uint32_t rd16 = min(cd - base, 0xFFFFu), rp16 = min(cp - base, 0xFFFFu);
            so01 = d == 1u ? (so01 & 0xFFFF0000u) | rd16 : so01;          // dy
            so01 = d == 2u ? (so01 & 0x0000FFFFu) | (rd16 << 16) : so01;  // dz
            so23 = d == 0u ? (so23 & 0xFFFF0000u) | rp16 : so23;          // px
            so23 = d == 1u ? (so23 & 0x0000FFFFu) | (rp16 << 16) : so23;  // py
            so4 = d == 2u ? rp16 : so4;                                   // pz
            AxisCode c;
            c.n0 = __ldcg(&P->pred_n[3 * d]);
            c.n1 = __ldcg(&P->pred_n[3 * d + 1]);
            c.n2 = __ldcg(&P->pred_n[3 * d + 2]);
            c.K = __ldcg(&P->pred_k[d]);
            c.half = __ldcg(&P->pred_half[d]);
            c.cmax = __ldcg(&P->code_max[d]);
            c.anc = d == 0u ? anc0 : (d == 1u ? anc1 : anc2);
            const uint32_t td = d == 0u ? tk0 : (d == 1u ? tk1 : tk2);
            const uint32_t tp = d == 0u ? tk3 : (d == 1u ? tk4 : tk5);
            c.kd = td & 0x3Fu;
            c.kp = tp & 0x3Fu;
            c.egd = (td & 0x80u) ? 0xFFFFFFFFu : 0u;
            c.egp = (tp & 0x80u) ? 0xFFFFFFFFu : 0u;
            if (kLin)
                ok = gwalk_lin<kWide>(lr, c, wq, G.n_walk, n_local, plane, lim, cd, cp);
            else
                ok = gwalk_any<GlobRd, kWide>(gr, c, reinterpret_cast<const uint32_t*>(wq), G.n_walk, n_local,
                                              plane, lim, cd, cp);
        }
        __syncwarp();
        emit_axis<kWide>(a, L, rmask, planes, code_off, d, lane);
    }
    if (act) {
        // pz, the last substream, must end where the next meshlet starts (:507)
        const bool last_of_mesh = L.m - P->meshlet_begin + 1u == P->n_meshlets;
        if (ok && (last_of_mesh ? cp > lim : cp != lim)) ok = false;
        if (!ok) report(a.status, kErrCorrupt, L.m);
        // the meshlet record's walk facts and side table (substream starts
        // after the anchor)
        MeshletDesc* md = a.descs + L.m;
        md->anchor_bit = G.anchor;
        md->walk = G.kind0 | (G.n_walk << 16);
        md->sub_offs[0] = static_cast<uint16_t>(so01);
        md->sub_offs[1] = static_cast<uint16_t>(so01 >> 16);
        md->sub_offs[2] = static_cast<uint16_t>(so23);
        md->sub_offs[3] = static_cast<uint16_t>(so23 >> 16);
        md->sub_offs[4] = static_cast<uint16_t>(so4);
    }
}

template <bool kWide>
__device__ void group_decode(const DecodeArgs& a, uint32_t g, int lane, uint8_t* region, const uint4* mtf_masks) {
    uint32_t* ring = reinterpret_cast<uint32_t*>(region) + lane * kLaneRingWords;
    uint8_t* work = region + kGRingBytes;
    uint8_t* flags = work + lane * kGFlagStride;
    uint32_t* tr = reinterpret_cast<uint32_t*>(work + 32u * kGFlagStride) + lane * kGRow;
    uint32_t* wr = reinterpret_cast<uint32_t*>(work + 32u * kGFlagStride + 32u * kGRow * 4u) + lane * kGRow;
    GLane G;
    load_group_lane(a, g, lane, G.L);
    G.rot = (static_cast<uint32_t>(lane) * 4u) & 31u;
    G.anchor = G.kind0 = G.n_walk = 0u;
    G.bad = G.suspect = false;
    bool ok = G.L.valid;
    if (ok && !placement_ok(a, G.L)) {
        report(a.status, kErrCorrupt, G.L.m);
        ok = false;
    }
    if (!__any_sync(kFull, ok)) return;
    gconn<false>(a, G, ok, ring, flags, tr, wr, mtf_masks);
    // lanes whose raw tokens met an id still in the FIFO: the exact pass
    const bool redo = ok && G.suspect;
    if (__any_sync(kFull, redo)) gconn<true>(a, G, redo, ring, flags, tr, wr, mtf_masks);
    if (ok && G.bad) {
        report(a.status, kErrCorrupt, G.L.m);
        ok = false;
    }
    __syncwarp();
    // Vertex phase: the whole region holds, per round lane, a code plane
    // (odd word count: the lanes' walks visit about the same local ids at
    // the same time) and a stage of its residual bits (16-byte units, three
    // words past the bits: reads peek up to 64 bits past lim + 1).
    const GroupLane& L = G.L;
    const uint32_t n_local = L.d.counts0 & 0xFFFFu;
    const uint32_t csz = 4u * (((n_local * static_cast<uint32_t>(sizeof(PlaneT<kWide>)) + 3u) >> 2) | 1u);
    const unsigned long long src16 = (L.blob_off + (G.anchor >> 3)) & ~15ull;
    const unsigned long long end16 = (L.blob_off + ((L.d.end_bit + 7u) >> 3) + 12ull + 15ull) & ~15ull;
    const uint32_t ssz = ok ? static_cast<uint32_t>(end16 - src16) : 0u;
    const uint32_t sbase = static_cast<uint32_t>((src16 - L.blob_off) * 8ull);
    uint32_t todo = __ballot_sync(kFull, ok);
    while (todo) {
        const bool in = (todo >> lane) & 1u;
        uint32_t cc = in ? csz : 0u, cs = in ? ssz : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t1 = __shfl_up_sync(kFull, cc, o);
            const uint32_t t2 = __shfl_up_sync(kFull, cs, o);
            if (lane >= o) {
                cc += t1;
                cs += t2;
            }
        }
        uint32_t rmask = __ballot_sync(kFull, in && align16(cc) + cs <= kGWarpBytes);
        const bool lin = rmask != 0u;
        if (!lin) rmask = 1u << (__ffs(todo) - 1);  // one lane whose bits do not fit: global reads
        todo &= ~rmask;
        const bool act = (rmask >> lane) & 1u;
        const uint32_t code_off = act ? cc - csz : 0u;
        if (lin) {
            const uint32_t ptot = align16(__reduce_max_sync(kFull, act ? cc : 0u));
            uint32_t* st = reinterpret_cast<uint32_t*>(region + ptot + (act ? cs - ssz : 0u));
            if (act)
                for (uint32_t o = 0; o < ssz; o += 16u)
                    cp_async16(st + (o >> 2), a.arena + src16 + o, 16u);
            cp_async_wait_all();
            if (act)  // in bit order, once
                for (uint32_t j = 0; j < (ssz >> 2); j++) st[j] = bswap32(st[j]);
            __syncwarp();
            gvert<true, kWide>(a, G, st, sbase, act, rmask, region, code_off, lane);
        } else {
            gvert<false, kWide>(a, G, nullptr, 0u, act, rmask, region, code_off, lane);
        }
        __syncwarp();  // the next round reuses the region
    }
}

// Warp w of CTA b takes group order position w * gridDim.x + b first (the
// costliest groups spread over the SMs), then positions from the counter.
template <bool kWide>
__global__ void __launch_bounds__(64, 5) group_kernel(DecodeArgs a, uint32_t warps) {
    extern __shared__ __align__(128) uint8_t smem[];
    __shared__ uint4 mtf_masks[16];
    const uint32_t warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < 16u) mtf_masks[threadIdx.x] = mtf_mask_row(threadIdx.x);
    __syncthreads();
    uint8_t* region = smem + warp * kGWarpBytes;
    const uint32_t n_groups = (a.total_meshlets + 31u) / 32u;
    const uint32_t n_first = warps * gridDim.x;
    uint32_t f = warp * gridDim.x + blockIdx.x;
    for (;;) {
        if (f >= n_groups) break;
        if (*reinterpret_cast<volatile unsigned long long*>(&a.status->err) != 0ull) break;
        group_decode<kWide>(a, group_at(f, n_groups), lane, region, mtf_masks);
        uint32_t nf = 0u;
        if (lane == 0) nf = n_first + atomicAdd(&a.status->work_conn, 1u);
        f = __shfl_sync(kFull, nf, 0);
    }
}

template <bool kWide>
cudaError_t launch_group_t(const DecodeArgs& a, const LaunchCfg& cfg, cudaStream_t s) {
    static size_t configured[64] = {0};
    static int per_sm_cache[64] = {0};
    const uint32_t warps = cfg.warps_per_cta >= 2 ? 2u : 1u;
    const size_t smem = static_cast<size_t>(warps) * kGWarpBytes;
    int dev = 0;
    cudaGetDevice(&dev);
    dev = dev < 0 || dev >= 64 ? 0 : dev;
    if (configured[dev] < smem) {
        cudaError_t e =
            cudaFuncSetAttribute(group_kernel<kWide>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(group_kernel<kWide>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        configured[dev] = smem;
        per_sm_cache[dev] = 0;
    }
    int per_sm = cfg.ctas_per_sm;
    if (per_sm <= 0) {
        if (per_sm_cache[dev] <= 0) {
            int n = 1;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, group_kernel<kWide>, static_cast<int>(32u * warps), smem);
            per_sm_cache[dev] = n > 0 ? n : 1;
        }
        per_sm = per_sm_cache[dev];
    }
    const uint32_t n_groups = (a.total_meshlets + 31u) / 32u;
    uint32_t grid = (n_groups + warps - 1u) / warps;
    const uint32_t cap = static_cast<uint32_t>(per_sm * device_sm_count());
    if (grid > cap) grid = cap;
    if (grid == 0) return cudaSuccess;
    group_kernel<kWide><<<grid, 32u * warps, smem, s>>>(a, warps);
    note_launch(static_cast<uint32_t>(smem), grid);
    return cudaGetLastError();
}

}  // namespace

size_t group_smem_bytes(const LaunchCfg& cfg) {
    return static_cast<size_t>(cfg.warps_per_cta >= 2 ? 2u : 1u) * kGWarpBytes;
}

cudaError_t launch_group(const DecodeArgs& a, const LaunchCfg& cfg, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return a.wide_codes ? launch_group_t<true>(a, cfg, s) : launch_group_t<false>(a, cfg, s);
}

}  // namespace stride
