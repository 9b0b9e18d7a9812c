// STRIDE (DPR4 v3) decode kernels for sm_103a.
//
// A decode is a memset of the status word, then:
//
//  1. scan_kernel -- one thread per meshlet: offset table entry and 48-bit
//     meshlet header (n_local, n_tris, n_strips), range checks, exclusive
//     scans of n_local / n_tris (output placement) and of n_local rounded up
//     to four (walk scratch placement), and a per-256-meshlet rank by token
//     count (groups of 32 similar meshlets).  Extra blocks of the same launch
//     fill per-code dequantisation tables.
//
//  2. flow_kernel (default) -- one persistent launch for both phases.  A CTA's
//     two warp pairs decode connectivity groups (32 meshlets, one per lane):
//     the parser warp streams each lane's meshlet through a per-lane ring
//     (cp.async) and runs the token chain -- strip headers, token widths, the
//     16-entry move-to-tail FIFO in registers (_read_vert,
//     encoder/paradelta_codec.py:330-340) -- and the assembler warp replays
//     strip state, triangles and first occurrences (decode_dup's strip loop,
//     encoder/paradelta_v5_dup.py:513-542).  Finished groups go into a
//     completion list; when no connectivity group is left, the CTA decodes
//     the vertices of listed groups: the residual bits staged once by bulk
//     copies, three axis warps skipping to their substreams and
//     reconstructing integer codes in walk order (IRLP,
//     encoder/paradelta_v5_dup.py:91-104 and 581-600), then writing exact
//     positions (stride_dequant.h).
//
//     The same per-group code also runs as two kernels (conn_kernel, then
//     vert_kernel), the launch shape of host-output decodes and of the
//     autotuner's other candidates.
//
// Every global read goes through L2 only (the serving engine rewrites arena
// ranges while other launches run; see the bit access helpers below).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include "stride_common.cuh"
#include "stride_device.cuh"
#include "stride_gb300.h"

namespace stride {
namespace {

// ---------------------------------------------------------------------------
// Named barriers between the two warps of a connectivity pair (producer
// arrives, consumer waits; 64 threads).  Pair p uses ids 1 + 4p .. 4 + 4p:
// slot 0, 1 = record chunk 0, 1 full; slot 2, 3 = chunk 0, 1 empty.  The
// ids are immediates: an id in a register makes the CTA reserve all 16 of
// the SM's per-CTA barriers, which caps a two-pair CTA at four per SM.
// ---------------------------------------------------------------------------
template <int kId>
__device__ __forceinline__ void bar_sync_imm() {
    asm volatile("bar.sync %0, 64;" ::"n"(kId) : "memory");
}
template <int kId>
__device__ __forceinline__ void bar_arrive_imm() {
    asm volatile("bar.arrive %0, 64;" ::"n"(kId) : "memory");
}

template <int kBase, bool kArrive>
__device__ __forceinline__ void pair_bar_at(uint32_t slot) {
    switch (slot) {
        case 0: kArrive ? bar_arrive_imm<kBase>() : bar_sync_imm<kBase>(); break;
        case 1: kArrive ? bar_arrive_imm<kBase + 1>() : bar_sync_imm<kBase + 1>(); break;
        case 2: kArrive ? bar_arrive_imm<kBase + 2>() : bar_sync_imm<kBase + 2>(); break;
        default: kArrive ? bar_arrive_imm<kBase + 3>() : bar_sync_imm<kBase + 3>(); break;
    }
}

// warp-uniform pair and slot; G pairs per CTA (1 or 2)
template <int G, bool kArrive>
__device__ __forceinline__ void pair_bar(uint32_t pair, uint32_t slot) {
    if (kArrive) __threadfence_block();  // shared-memory writes before the arrive reach the waiting warp
    if (G == 1 || pair == 0u) {
        pair_bar_at<1, kArrive>(slot);
    } else {
        pair_bar_at<5, kArrive>(slot);
    }
}

// Named barrier of a pair's two warps for taking and finishing groups
// (immediate ids 9 and 10, past the record barriers 1..8).
__device__ __forceinline__ void claim_bar(uint32_t pair) {
    if (pair == 0u) {
        bar_sync_imm<9>();
    } else {
        bar_sync_imm<10>();
    }
}

// ---------------------------------------------------------------------------
// 1. scan kernel
// ---------------------------------------------------------------------------
__device__ int scan_meshlet(const uint8_t* __restrict__ arena, const MeshParams& P, uint32_t lm, MeshletDesc& d) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(arena + P.blob_off);
    const uint32_t nbits = static_cast<uint32_t>(P.nbits);
    const uint32_t tbit = kHeaderBytes * 8u;
    const uint32_t off = peek32<false>(w, tbit + 32u * lm);
    const uint32_t next = (lm + 1u < P.n_meshlets) ? peek32<false>(w, tbit + 32u * (lm + 1u)) : nbits;
    // decode_dup reads meshlets back to back from the end of the table, so
    // the table must start there and increase (paradelta_v5_dup.py:496-507)
    if ((lm == 0u && off != P.body_bit) || off < P.body_bit || next > nbits || off > nbits - 48u ||
        next < off + 48u)
        return kErrOffset;
    const uint32_t h0 = peek32<false>(w, off);
    const uint32_t n_local = h0 >> 16;
    const uint32_t n_tris = h0 & 0xFFFFu;
    const uint32_t n_strips = peek32<false>(w, off + 32u) >> 16;
    if (n_local > static_cast<uint32_t>(kMaxLocal) || n_tris > static_cast<uint32_t>(kMaxTris))
        return kErrUnsupported;
    if (n_strips > n_tris) return kErrCorrupt;  // every strip emits >= 1 triangle
    d.start_bit = off;
    d.end_bit = next;
    d.counts0 = n_local | (n_tris << 16);
    d.n_strips = n_strips;
    return 0;
}

// Exclusive scan over the block; returns the thread's prefix and the total.
__device__ __forceinline__ unsigned long long block_scan(unsigned long long x, unsigned long long* wsum,
                                                         unsigned long long& total) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    constexpr int kWarps = kScanThreads / 32;
    unsigned long long inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(kFull, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        unsigned long long v = lane < kWarps ? wsum[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long t = __shfl_up_sync(kFull, v, o);
            if (lane >= o) v += t;
        }
        if (lane < kWarps) wsum[lane] = v;
    }
    __syncthreads();
    const unsigned long long excl = inc - x + (warp ? wsum[warp - 1] : 0ull);
    total = wsum[kWarps - 1];
    __syncthreads();
    return excl;
}

// Dequantisation tables: block b of mesh lut_meshes[b / bx] evaluates codes
// (b % bx) * 256 + threadIdx.x of its three axes, exactly.
__device__ __forceinline__ void lut_block(const DecodeArgs& a, uint32_t b, uint32_t bx) {
    const MeshParams& P = a.meshes[a.lut_meshes[b / bx]];
    const uint32_t i = (b % bx) * 256u + threadIdx.x;
    const uint32_t e0 = 1u << P.g_bits[0], e1 = 1u << P.g_bits[1], e2 = 1u << P.g_bits[2];
    if (i >= e0 + e1 + e2) return;
    const uint32_t d = i < e0 ? 0u : (i < e0 + e1 ? 1u : 2u);
    const uint32_t q = i - (d >= 1u ? e0 : 0u) - (d >= 2u ? e1 : 0u);
    a.lut[P.lut_off + i] = stride_dequant(&P.dq[d], q);
}

// Blocks [0, nb) scan the meshlets of scan blocks b0 .. b0 + nb - 1; the
// blocks after them (lut_bx per mesh with tables) fill the dequantisation
// tables in the same launch.  A decode scans in one launch (b0 = 0, every
// block) or in launches over consecutive block ranges, each continuing the
// block prefixes of the ones before it.
//
// Slots: the decode kernels take meshlets in groups of 32 slots, one lane
// each, and a warp runs as many token iterations as its longest meshlet.
// Each block therefore orders its 256 meshlets by token count (triangles
// plus two per strip; ties by index) and slot i of the block holds the
// meshlet of rank i, so a group's lanes have about the same work.  Outputs
// are placed per meshlet, so the order changes no result.
__global__ void __launch_bounds__(kScanThreads) scan_kernel(DecodeArgs a, uint32_t b0, uint32_t nb,
                                                             uint32_t lut_bx) {
    // The fused kernel may be scheduled once every block of this launch has
    // started (it waits for this grid's completion before it reads
    // anything): its launch latency then overlaps this kernel, and it never
    // holds an SM that a block of this launch still needs.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (blockIdx.x >= nb) {  // block-uniform
        lut_block(a, blockIdx.x - nb, lut_bx);
        return;
    }
    __shared__ unsigned long long wsum[kScanThreads / 32];
    __shared__ __align__(16) uint32_t skey[kScanThreads];
    __shared__ uint32_t sslot[kScanThreads];
    __shared__ int is_last;
    const uint32_t tid = threadIdx.x;
    const uint32_t blk = b0 + blockIdx.x;
    const uint32_t m = blk * kScanThreads + tid;
    uint32_t nl = 0u, nt = 0u;
    MeshletDesc d;
    memset(&d, 0, sizeof(d));
    if (m < a.total_meshlets) {
        const uint32_t mi = a.meshlet_mesh ? __ldcg(a.meshlet_mesh + m) : 0u;
        const MeshParams& P = a.meshes[mi];
        const int e = scan_meshlet(a.arena, P, m - P.meshlet_begin, d);
        if (e) {
            report(a.status, e, m);
            d.counts0 = 0u;  // keeps the prefixes finite; the decode is abandoned
        } else {
            nl = d.counts0 & 0xFFFFu;
            nt = d.counts0 >> 16;
        }
    }
    unsigned long long t1, t2;
    const unsigned long long e1 = block_scan((static_cast<unsigned long long>(nt) << 32) | nl, wsum, t1);
    const unsigned long long e2 = block_scan((nl + 3u) & ~3u, wsum, t2);
    // rank by (tokens, index); meshlets past the end rank last
    {
        const uint32_t tokens = nt + 2u * d.n_strips;  // <= 256 + 2 * 256
        const uint32_t key = (m < a.total_meshlets ? tokens : 0xFFFFFFu) << 8 | tid;
        skey[tid] = key;
        __syncthreads();
        uint32_t rank = 0u;
        const uint4* k4 = reinterpret_cast<const uint4*>(skey);
#pragma unroll 8
        for (uint32_t j = 0; j < kScanThreads / 4u; j++) {
            const uint4 q = k4[j];
            rank += (q.x < key) + (q.y < key) + (q.z < key) + (q.w < key);
        }
        sslot[rank] = tid;
        __syncthreads();
        d.slot_meshlet = blk * kScanThreads + sslot[tid];
    }
    if (m < a.total_meshlets) {
        d.v_pref = static_cast<uint32_t>(e1);
        d.t_pref = static_cast<uint32_t>(e1 >> 32);
        d.wp_pref = static_cast<uint32_t>(e2);
        uint4* dst = reinterpret_cast<uint4*>(a.descs + m);
        const uint4* src = reinterpret_cast<const uint4*>(&d);
        dst[0] = src[0];
        dst[1] = src[1];
        dst[2] = src[2];
        dst[3] = src[3];
    }
    if (tid == 0)
        a.blk_sums[blk] = make_uint4(static_cast<uint32_t>(t1), static_cast<uint32_t>(t1 >> 32),
                                     static_cast<uint32_t>(t2), 0u);
    // The last block to finish turns the block sums into block prefixes
    // (the ticket counts the blocks of this decode's scan launches so far).
    // Only the block sum, thread 0's own write, is read inside this grid,
    // so only thread 0 fences before taking its ticket (the descriptors are
    // read by the next kernels); a fence on every thread made every block
    // wait for its 16 KB of descriptors to reach L2.
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        is_last = atomicAdd(&a.status->ticket, 1u) == b0 + nb - 1u;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    unsigned long long cv = 0ull, ct = 0ull, cw = 0ull;
    if (b0) {  // the totals of the blocks before this launch's
        const BlockPrefix* pp = a.blk_prefix + b0 - 1u;
        const uint4 q = __ldcg(a.blk_sums + b0 - 1u);
        cv = __ldcg(&pp->v) + q.x;
        ct = __ldcg(&pp->t) + q.y;
        cw = __ldcg(&pp->wp) + q.z;
    }
    for (uint32_t base = 0; base < nb; base += kScanThreads) {
        const uint32_t i = base + tid;
        const uint4 s = i < nb ? __ldcg(a.blk_sums + b0 + i) : make_uint4(0u, 0u, 0u, 0u);
        // per-chunk sums stay below 2^32 (256 blocks x 65536), so pack pairs
        unsigned long long ta, tb;
        const unsigned long long ea = block_scan((static_cast<unsigned long long>(s.y) << 32) | s.x, wsum, ta);
        const unsigned long long eb = block_scan(s.z, wsum, tb);
        if (i < nb) {
            BlockPrefix p;
            p.v = cv + (ea & 0xFFFFFFFFull);
            p.t = ct + (ea >> 32);
            p.wp = cw + eb;
            p.pad = 0ull;
            a.blk_prefix[b0 + i] = p;
        }
        cv += ta & 0xFFFFFFFFull;
        ct += ta >> 32;
        cw += tb;
    }
}

// ---------------------------------------------------------------------------
// 2. connectivity kernel
// ---------------------------------------------------------------------------

// connectivity warp pair: lane byte rings | token records (two chunks) |
// chunk counts (4 words) | first-occurrence bits (8 words per lane) |
// triangle ring | walk ring.  22,544 bytes: five two-pair CTAs fit an SM.
constexpr uint32_t kChunkWords = 16u;  // iterations per chunk (kChunk)
__host__ __device__ constexpr uint32_t conn_pair_bytes() {
    return 32u * kLaneRingWords * 4u + 2u * kChunkWords * 32u * 4u + 16u + 8u * 32u * 4u + 2u * 32u * kRingRow * 4u;
}

__host__ __device__ inline uint32_t vert_stage_bytes(uint32_t stage_bytes) { return stage_bytes / 2u; }

// One axis warp's code plane.
__host__ __device__ inline uint32_t vert_axis_bytes(uint32_t code_bytes) { return align16(code_bytes); }

// Vertex CTA: residual stage | three axis planes | mbarrier.
__host__ __device__ inline uint32_t vert_cta_bytes(uint32_t stage_bytes, uint32_t code_bytes) {
    return align16(vert_stage_bytes(stage_bytes) + 32u) + 3u * vert_axis_bytes(code_bytes) + 16u;
}

// Connectivity as a producer/consumer pair of warps per group of 32
// meshlets.  The parser warp runs the serial part of every lane's token
// chain -- bit cursor, strip headers, token widths, the 16-entry FIFO in
// registers (_read_vert, encoder/paradelta_codec.py:330-340) -- and writes
// one 32-bit record per lane and iteration into a two-chunk ring in shared
// memory; the assembler warp replays the records: strip state, triangles,
// first occurrences (walk), output rings.  The two chains run on different
// warps, so each is about half as long as the fused one.
//
// Validity is checked lazily, as running extremes compared once at the end:
// the parser's FIFO indices, local ids, cursor and strips, the assembler's
// triangle count.  Until then a corrupt lane runs on harmlessly: every id
// the parser passes on is clamped below n_local, and the assembler's
// flushes never write past the meshlet's triangles or walk entries.
//
// Record: bits 0..8 the local id (a raw token's as read, up to ib <= 9
// bits; a FIFO token's from the FIFO), bit 9 raw, bit 10 the edge bit (a
// strip-body token's edge code), bits 11..12 token position in its strip
// (0..2 the three roots, 3 a strip-body token), bit 13 live (clear: no
// token).
constexpr uint32_t kChunk = kChunkWords;  // iterations per ring chunk
constexpr uint32_t kChunkDone = 1u << 31;  // count word: the parser has finished
constexpr uint32_t kRecRaw = 1u << 9, kRecLive = 1u << 13;

// Pair barrier slots: chunk c full, chunk c empty.
__device__ __forceinline__ uint32_t bar_full(uint32_t c) { return c; }
__device__ __forceinline__ uint32_t bar_empty(uint32_t c) { return 2u + c; }

// Parser warp.  Each active lane streams its meshlet's bytes through its
// ring: chunks 0 and 1 before the first token, then after every record
// chunk (at most kChunk tokens of at most 26 bits, i.e. 13 words) one more
// chunk whenever fewer than 33 words lie ahead of the window.  The copies of
// one refill are waited for at the next, so each has a full record chunk
// of time to land; a refill overwrites the chunk two behind, which the
// window has passed (its last words are in registers).
//
// The FIFO is a move-to-front register whose unused bytes hold 0xFF.  In
// the fast pass (kExact false) a raw token's id is taken as new to the FIFO
// -- an encoder writes a FIFO index for an id it still holds -- and an id
// that is there after all (or equals the 0xFF filler) is only detected,
// which makes the lane suspect; a group with a suspect lane runs again with
// kExact, where a raw id is searched for and moved from where it is.
// Returns the suspect flag (always false with kExact).
template <int G, bool kExact>
__device__ bool conn_parse(const DecodeArgs& a, const GroupLane& L, bool act, uint32_t* __restrict__ ring,
                           uint32_t* __restrict__ recs, uint32_t* __restrict__ counts, uint32_t pair, int lane,
                           const uint4* __restrict__ mtf_masks) {
    const uint32_t n_local = L.d.counts0 & 0xFFFFu;
    const uint32_t ib = max(1u, 32u - __clz(n_local));  // _idx_bits_for (paradelta_codec.py:124-125)
    const uint32_t rsh = 32u - ib, ib1 = 1u + ib;
    const uint32_t end = L.d.end_bit;
    const unsigned long long s0 = (L.blob_off + (L.d.start_bit >> 3)) & ~15ull;
    const unsigned long long e16 = (L.blob_off + ((end + 7u) >> 3) + 15ull) & ~15ull;
    const uint32_t avail = act ? static_cast<uint32_t>(e16 - s0) : 0u;  // inactive lanes read nothing
    const uint8_t* src = a.arena + (act ? s0 : 0ull);
    const uint32_t rot = (static_cast<uint32_t>(lane) * 4u) & 31u;
    ring_fetch(ring, src, avail, rot, 0u);
    ring_fetch(ring, src, avail, rot, 1u);
    cp_async_wait_all();
    uint32_t req = 2u;  // chunks requested
    // bit window: words wi, wi + 1, wi + 2 of the lane's data (in bit order)
    // in w0, w1, w2; `off` bits of w0 consumed; ri = rotated ring index of
    // wi + 2 (word j of the data sits at ring[(j + rot) & 63])
    const uint32_t base0 = static_cast<uint32_t>((s0 - L.blob_off) * 8ull);  // stream bit of the data's bit 0
    const uint32_t q0 = act ? L.d.start_bit + 48u - base0 : 0u;
    uint32_t off = q0 & 31u;
    uint32_t ri = (q0 >> 5) + 2u + rot;
    auto rw = [ring](uint32_t r) { return bswap32(ring[r & (kLaneRingWords - 1u)]); };
    uint32_t w0 = rw(ri - 2u), w1 = rw(ri - 1u), w2 = rw(ri);
    uint32_t strips_left = L.d.n_strips;
    uint32_t tok_left = 0u, tx = 0u;
    int32_t smin = 0;  // smallest depth a FIFO token named (negative: past the entries)
    bool suspect = false;
    MtfFifo fifo;
    fifo.f0 = fifo.f1 = fifo.f2 = fifo.f3 = 0xFFFFFFFFu;
    bool live = act && strips_left > 0u;  // false for good once the lane's strips are read
    // A strip of length len takes len + 2 tokens and adds len triangles (one
    // for len 0), so n_tris + 2 n_strips iterations read every strip of a
    // valid lane: the warp runs the largest of those counts instead of
    // voting every iteration.  A lane still live after them is corrupt.
    const uint32_t iters = __reduce_max_sync(kFull, act ? (L.d.counts0 >> 16) + 2u * L.d.n_strips : 0u);
    uint32_t it = 0u;
    uint32_t k = 0u;  // chunk
    for (;;) {
        const uint32_t c = k & 1u;
        if (k >= 2u) pair_bar<G, false>(pair, bar_empty(c));  // the assembler is done with chunk k - 2
        uint32_t* rc = recs + c * kChunk * 32u + lane;
        const uint32_t n = min(kChunk, iters - it);
        // unrolled by four: 7% faster than the rolled loop, measured (8 ties,
        // 2 and 16 are slower)
#pragma unroll 4
        for (uint32_t i = 0; i < n; i++) {
            // No branch per token, so consecutive tokens' chains can overlap:
            // a lane that has finished keeps running the body on whatever
            // bits follow, but its window and FIFO no longer move and its
            // records are not live.  A 32-bit window holds a strip header (16
            // bits) plus the next token (at most 1 + 9 bits), or an edge code
            // plus a token.
            const uint32_t x0 = __funnelshift_l(w1, w0, off);
            const bool hdr = tok_left == 0u;                 // strip header (paradelta_v5_dup.py:519)
            const uint32_t sb = max(x0 >> 16, 1u) - 1u;       // body tokens of the strip
            tok_left = hdr ? sb + 3u : tok_left;
            strips_left -= hdr ? 1u : 0u;
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
            // (a running min here; the local ids are checked by the assembler)
            const int32_t sd = static_cast<int32_t>(fifo.len) - 1 - static_cast<int32_t>(fi);
            smin = min(smin, (raw | !live) ? 0 : sd);
            const uint32_t s = static_cast<uint32_t>(sd) & 15u;  // depth of a FIFO token's entry
            const uint32_t v = raw ? (rid & 0xFFu) : fifo.at(s);
            bool fresh = raw;  // a raw id not in the FIFO
            uint32_t p;
            if constexpr (kExact) {
                const uint32_t at = raw ? fifo.find(v) : 16u;
                fresh = raw & (at == 16u);
                p = raw ? (fresh ? min(fifo.len, 15u) : at) : s;
            } else {
                suspect = suspect | (raw & live & fifo.holds(v));
                p = raw ? min(fifo.len, 15u) : s;
            }
            fifo.mtf_masked(v, mtf_masks[live ? p : 16u]);  // row 16 is zero: no change
            fifo.len += (live & fresh & (fifo.len < 16u)) ? 1u : 0u;
            rc[i * 32u] = (raw ? (rid | kRecRaw) : v) | (ec << 10) | (tix << 11) | (live ? kRecLive : 0u);
            tok_left--;
            tx = min(tix + 1u, 3u);
            // advance: at most one word boundary per token (used <= 26)
            off += live ? used : 0u;
            const bool cross = off >= 32u;
            off &= 31u;
            ri += cross ? 1u : 0u;
            const uint32_t nw = rw(ri);
            w0 = cross ? w1 : w0;
            w1 = cross ? w2 : w1;
            w2 = cross ? nw : w2;
            live = live & ((tok_left | strips_left) != 0u);
        }
        it += n;
        const bool done = it >= iters;
        if (lane == 0) counts[c] = n | (done ? kChunkDone : 0u);
        pair_bar<G, true>(pair, bar_full(c));
        k++;
        if (done) break;
        // refill (the previous refill has had a record chunk to land): one
        // more chunk when fewer than 33 words lie ahead of the window's next
        // load
        cp_async_wait_all();
        if (live && kLaneChunkWords * req < ri - rot + 34u) {
            ring_fetch(ring, src, avail, rot, req);
            req++;
        }
        cp_async_commit();
    }
    cp_async_wait_all();  // no copy may land after the CTA's shared memory is gone
    // take the assembler's remaining chunk releases: the ring and the
    // barriers are clean
    for (uint32_t j = k >= 2u ? k - 2u : 0u; j < k; j++) pair_bar<G, false>(pair, bar_empty(j & 1u));
    if (act) {
        const uint32_t pos = base0 + 32u * (ri - 2u - rot) + off;  // the stream bit after the last token
        // every strip read, FIFO indices in range, inside the meshlet; a
        // suspect lane's FIFO (and so its checks) may be off: its group runs
        // again exactly
        const bool bad = live || smin < 0 || pos > end;
        if (bad && !suspect) {
            report(a.status, kErrCorrupt, L.m);
        } else if (!bad) {
            a.descs[L.m].anchor_bit = pos;
        }
    }
    return act && suspect;
}

// Assembler warp.
template <int G>
__device__ void conn_assemble(const DecodeArgs& a, const GroupLane& L, bool act, uint32_t* __restrict__ seen,
                              uint32_t* __restrict__ tring, uint32_t* __restrict__ wring,
                              const uint32_t* __restrict__ recs, const uint32_t* __restrict__ counts, uint32_t pair,
                              int lane) {
#pragma unroll
    for (int i = 0; i < 8; i++) seen[i * 32 + lane] = 0u;
    const uint32_t n_local = L.d.counts0 & 0xFFFFu;
    const uint32_t n_tris = L.d.counts0 >> 16;
    uint32_t* walk_out = a.walk_scratch + L.wp_base;
    // triangle indices are relative to the mesh's first vertex
    const uint32_t vloc = act ? static_cast<uint32_t>(L.v_base - L.P->v_offset) : 0u;
    const uint32_t ph = static_cast<uint32_t>(L.t_base) & 3u;  // ring slot of triangle 0
    uint32_t* tr = tring + lane * kRingRow;
    uint32_t* wr = wring + lane * kRingRow;
    uint32_t tf = 0u, wf = 0u;  // entries already written out
    uint32_t flush_in = kFlushEvery;
    uint32_t P = 0u;  // strip state p0 | p1 << 8 | p2 << 16
    uint32_t tcnt = 0u, wcnt = 0u, kind0 = 0u;
    const uint32_t vmax = n_local ? n_local - 1u : 0u;
    uint32_t ridmax = 0u;  // largest raw id + 1 (0: none)
    for (uint32_t k = 0u;; k++) {
        const uint32_t c = k & 1u;
        pair_bar<G, false>(pair, bar_full(c));
        const uint32_t cw = counts[c];
        const uint32_t n = cw & (kChunk | (kChunk - 1u));
        const uint32_t* rc = recs + c * kChunk * 32u + lane;
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t rec = rc[i * 32u];
            if (rec & kRecLive) {
                const uint32_t id = rec & 0x1FFu;
                // decode_dup raises IndexError on a local id past n_local: a
                // running max; ids stay below n_local, whatever the stream says
                ridmax = max(ridmax, (rec & kRecRaw) ? id + 1u : 0u);
                const uint32_t v = min(id, vmax);
                const uint32_t ti = (rec >> 11) & 3u;
                const bool body = ti == 3u;
                const uint32_t ec = body ? (rec >> 10) & 1u : 0u;
                // edge code 0 -> (p1, p2 | p0), 1 -> (p0, p2 | p1) (:530-535);
                // a root token puts v at its position
                const uint32_t sel = body ? (ec ? 0x7420u : 0x7421u) : (0x7210u + ((4u - ti) << (4u * ti)));
                const uint32_t cref = ec ? ((P >> 8) & 0xFFu) : (P & 0xFFu);
                const uint32_t Pn = __byte_perm(P, v, sel);
                const bool emit = body | (ti == 2u);
                if (emit) tr[(ph + tcnt) & 31u] = Pn;
                tcnt += emit ? 1u : 0u;
                // first occurrence -> next walk entry (:523-541).  Roots are 'none'
                // (stored as v,v,v,v); strip bodies 'para' with (a, b, c) = (p0, p1, cref).
                uint32_t* sp = seen + (v >> 5) * 32u + lane;
                const uint32_t sw = *sp;
                const uint32_t bit = 1u << (v & 31u);
                const bool isnew = (sw & bit) == 0u;
                if (isnew) *sp = sw | bit;
                const uint32_t e = body ? (v | ((Pn & 0xFFFFu) << 8) | (cref << 24)) : v * 0x01010101u;
                if (isnew) wr[wcnt & 31u] = e;
                wcnt += isnew ? 1u : 0u;
                kind0 += (isnew & !body) ? 1u : 0u;
                P = Pn;
            }
            if (--flush_in == 0u) {  // warp-uniform
                flush_in = kFlushEvery;
                if (act) {  // never past the meshlet's triangles or walk entries
                    flush_tris(a.idx, L.t_base, tr, tf, min(tcnt, n_tris), vloc, false);
                    flush_walk(walk_out, wr, wf, min(wcnt, n_local), false);
                }
            }
        }
        pair_bar<G, true>(pair, bar_empty(c));
        if (cw & kChunkDone) break;
    }
    if (act) {
        flush_tris(a.idx, L.t_base, tr, tf, min(tcnt, n_tris), vloc, true);
        flush_walk(walk_out, wr, wf, min(wcnt, n_local), true);
        // the triangle count and the raw ids do not depend on the FIFO: no
        // suspect here
        if (tcnt != n_tris || ridmax > n_local) report(a.status, kErrCorrupt, L.m);
        a.descs[L.m].walk = kind0 | (min(wcnt, n_local) << 16);
    }
}

// Connectivity of group g by one warp pair (its shared memory at `base`):
// every lane streams its own meshlet, so no meshlet is too large.  The fast
// pass first; if a lane of it is suspect, both warps run the group again
// with the exact FIFO (outputs and records are rewritten).  `redo` is the
// pair's word in shared memory.
template <int G>
__device__ __forceinline__ void conn_group(const DecodeArgs& a, uint32_t g, uint32_t pair, bool parser, int lane,
                                           uint8_t* base, const uint4* mtf_masks, volatile uint32_t* redo) {
    uint32_t* rings = reinterpret_cast<uint32_t*>(base);
    uint32_t* recs = rings + 32u * kLaneRingWords;
    uint32_t* counts = recs + 2u * kChunk * 32u;
    uint32_t* seen = counts + 4;
    uint32_t* tring = seen + 8 * 32;
    uint32_t* wring = tring + 32 * kRingRow;
    GroupLane L;
    load_group_lane(a, g, lane, L);
    bool ok = L.valid;
    if (ok && !placement_ok(a, L)) {
        if (parser) report(a.status, kErrCorrupt, L.m);
        ok = false;
    }
    if (!__any_sync(kFull, ok)) return;  // both warps see the same lanes
    if (parser) {
        const bool s = conn_parse<G, false>(a, L, ok, rings + lane * kLaneRingWords, recs, counts, pair, lane,
                                            mtf_masks);
        const bool any = __any_sync(kFull, s);
        if (lane == 0) *redo = any ? 1u : 0u;
    } else {
        conn_assemble<G>(a, L, ok, seen, tring, wring, recs, counts, pair, lane);
    }
    claim_bar(pair);  // the pass is over; the redo word is written
    const bool again = *redo != 0u;
    claim_bar(pair);  // both warps have read it
    if (!again) return;
    if (parser) {
        conn_parse<G, true>(a, L, ok, rings + lane * kLaneRingWords, recs, counts, pair, lane, mtf_masks);
    } else {
        conn_assemble<G>(a, L, ok, seen, tring, wring, recs, counts, pair, lane);
    }
}

// Pair p of a CTA (warps 2p and 2p + 1: parser, assembler) decodes group
// blockIdx.x * G + p in one round.  Past the kernel-entry barrier the pairs
// never wait for one another.
template <int G>
__global__ void __launch_bounds__(G * 64) conn_kernel(DecodeArgs a) {
    extern __shared__ __align__(128) uint8_t smem[];
    __shared__ uint4 mtf_masks[17];
    __shared__ uint32_t s_redo[2];
    if (threadIdx.x < 17u) mtf_masks[threadIdx.x] = threadIdx.x < 16u ? mtf_mask_row(threadIdx.x) : make_uint4(0u, 0u, 0u, 0u);
    const uint32_t pair = threadIdx.x >> 6;
    const bool parser = ((threadIdx.x >> 5) & 1u) == 0u;
    const int lane = threadIdx.x & 31;
    const bool failed = *reinterpret_cast<volatile unsigned long long*>(&a.status->err) != 0ull;
    if (__syncthreads_or(failed)) return;
    // groups [g0, g1): whole windows, so the order below is a bijection of them
    const uint32_t g1 = min(a.conn_g1, (a.total_meshlets + 31u) / 32u);
    const uint32_t g0 = min(a.conn_g0, g1);
    const uint32_t f = blockIdx.x * G + pair;
    if (f >= g1 - g0) return;  // both warps of the pair
    conn_group<G>(a, g0 + group_at(f, g1 - g0), pair, parser, lane, smem + pair * conn_pair_bytes(), mtf_masks,
                  s_redo + pair);
}

// ---------------------------------------------------------------------------
// 3. vertex kernel
// ---------------------------------------------------------------------------
// Per-lane state of one axis of one meshlet.
struct VertLane {
    int32_t anc;      // anchor code of the axis
    uint32_t td, tp;  // (tag, k) of the axis' delta / parallelogram substream: bit 7 Exp-Golomb, bits 0..5 k
    uint32_t cdd;     // delta cursor
    uint32_t cp;      // parallelogram cursor
    bool bad;
};

// Anchor code of axis d and the six (tag, k) pairs (paradelta_v5_dup.py:
// 544-557); returns the bit after them (the start of dx).
template <bool kShared>
__device__ __forceinline__ uint32_t vert_header(const GroupLane& L, uint32_t d, const uint32_t* w, uint32_t rbase,
                                                VertLane& S, uint32_t (&tk)[6]) {
    const uint32_t end = L.d.end_bit;
    const MeshParams* P = L.P;
    uint32_t pos = L.d.anchor_bit;
    bool bad = false;
    S.anc = 0;
#pragma unroll
    for (uint32_t e = 0; e < 3u; e++) {
        const uint32_t gb = P->g_bits[e];
        const int32_t v = gb ? static_cast<int32_t>(peek32<kShared>(w, pos + rbase) >> (32u - gb)) : 0;
        S.anc = e == d ? v : S.anc;
        pos += gb;
    }
#pragma unroll
    for (int i = 0; i < 6; i++) {
        const uint32_t t = peek32<kShared>(w, pos + rbase) >> 16;
        pos += 16u;
        const uint32_t k = t & 0xFFu;
        bad = bad || k > static_cast<uint32_t>(kMaxResidK);
        tk[i] = ((t >> 8) == 1u ? 0u : 0x80u) | (k & 0x3Fu);
    }
    S.td = d == 0u ? tk[0] : (d == 1u ? tk[1] : tk[2]);
    S.tp = d == 0u ? tk[3] : (d == 1u ? tk[4] : tk[5]);
    S.bad = bad || pos > end;
    return min(pos, end);
}

// Integer codes of axis d in walk order (IRLP, paradelta_v5_dup.py:91-104
// and 581-600).  Every walk vertex is a root (delta from the previous walk
// vertex; the first one is the anchor) or a parallelogram vertex predicted
// from three earlier ones.  Four walk entries per iteration (one 16-byte
// load); entries past the end are masked, not branched around, and root and
// parallelogram vertices differ only in selects.  The walk reads codewords
// with the branch-free reader; a lane that met a codeword longer than its
// window walks its axis again with the general reader (every plane entry
// the walk reaches is written again, in the same order).
template <bool kShared, bool kWide>
__device__ __forceinline__ void vert_axis(const DecodeArgs& a, const GroupLane& L, uint32_t d,
                                          const uint32_t* __restrict__ w, uint32_t rbase,
                                          PlaneT<kWide>* __restrict__ plane, VertLane& S) {
    const uint32_t n_local = L.d.counts0 & 0xFFFFu;
    const uint32_t n_walk = L.d.walk >> 16;
    const uint32_t end = L.d.end_bit;
    const MeshParams* P = L.P;
    if (n_walk < n_local) {  // vertices the walk never reaches keep code 0
        uint32_t* z = reinterpret_cast<uint32_t*>(plane);
        const uint32_t nz = (n_local * static_cast<uint32_t>(sizeof(PlaneT<kWide>)) + 3u) >> 2;
        for (uint32_t i = 0; i < nz; i++) z[i] = 0u;
    }
    const int32_t n0 = P->pred_n[3 * d], n1 = P->pred_n[3 * d + 1], n2 = P->pred_n[3 * d + 2];
    const int32_t K = P->pred_k[d], half = P->pred_half[d];
    const uint32_t cmax = P->code_max[d];
    const uint32_t td = S.td, tp = S.tp;
    const int32_t anc = S.anc;
    uint32_t cdd = S.cdd, cp = S.cp;
    int32_t prev = 0;
    bool fail = false;
    bool longc = false, fast = true;
    auto step = [&](uint32_t e, bool valid, bool anchor) {
        e = valid ? e : 0u;  // a masked entry reads plane[0] and commits nothing
        const uint32_t v = e & 0xFFu;
        const uint32_t ra = (e >> 8) & 0xFFu, rb = (e >> 16) & 0xFFu, rc = e >> 24;
        const bool para = ra != v;  // roots are stored as (v, v, v, v)
        const int32_t ca = static_cast<int32_t>(plane[ra]);
        const int32_t cb = static_cast<int32_t>(plane[rb]);
        const int32_t cc = static_cast<int32_t>(plane[rc]);
        const int32_t pred = para ? (n0 * ca + n1 * cb + n2 * cc + half) >> K : prev;
        uint32_t p = para ? cp : cdd;
        int32_t r;
        const bool okr = fast ? residual_fast<kShared>(w, rbase, p, para ? tp : td, end, r, longc)
                              : residual<kShared>(w, rbase, p, para ? tp : td, end, r);
        const bool commit = valid & !anchor;  // the anchor has no residual
        cp = (commit & para) ? p : cp;
        cdd = (commit & !para) ? p : cdd;
        const int32_t code = anchor ? anc : pred + r;
        // codes of a valid stream lie in [0, 2^g_bits)
        fail = fail | (valid & ((!okr & !anchor) | (static_cast<uint32_t>(code) > cmax)));
        if (valid) plane[v] = static_cast<PlaneT<kWide>>(code);
        prev = valid ? code : prev;
    };
    // walk entries (v | a << 8 | b << 16 | c << 24), 16-byte aligned per meshlet
    const uint4* wq = reinterpret_cast<const uint4*>(a.walk_scratch + L.wp_base);
    // two quads in flight: the walk is read from L2
    {
        uint4 qn = n_walk ? __ldcg(wq) : make_uint4(0u, 0u, 0u, 0u);
        uint4 qm = n_walk > 4u ? __ldcg(wq + 1) : qn;
        for (uint32_t i = 0; i < n_walk; i += 4u) {
            const uint4 q = qn;
            qn = qm;
            if (i + 8u < n_walk) qm = __ldcg(wq + (i >> 2) + 2u);
            step(q.x, true, i == 0u);
            step(q.y, i + 1u < n_walk, false);
            step(q.z, i + 2u < n_walk, false);
            step(q.w, i + 3u < n_walk, false);
        }
    }
    if (longc) {  // rare: the lane's axis again, from its substream starts
        fast = false;
        cdd = S.cdd;
        cp = S.cp;
        prev = 0;
        fail = false;
        for (uint32_t i = 0; i < n_walk; i += 4u) {
            const uint4 q = __ldcg(wq + (i >> 2));
            step(q.x, true, i == 0u);
            step(q.y, i + 1u < n_walk, false);
            step(q.z, i + 2u < n_walk, false);
            step(q.w, i + 3u < n_walk, false);
        }
    }
    S.cp = cp;
    S.bad = S.bad || fail;
}

// One round of warp d: its active lanes find where their axis' two
// substreams start -- the delta substreams dx dy dz come first, then px py
// pz, so axis d skips the three delta substreams and the d parallelogram
// substreams before its own (substream lengths are not stored, only their
// code counts) -- decode axis d of their meshlets, then the warp writes that
// coordinate of every vertex.  The three warps skip independently: waiting
// for one another's skips measured slower than repeating them.
template <bool kShared, bool kWide, bool kPair>
__device__ __forceinline__ void vert_round(const DecodeArgs& a, const GroupLane& L, uint32_t d, bool act,
                                           uint32_t rmask, const uint32_t* w, uint32_t rbase, uint8_t* planes,
                                           uint32_t code_off, int lane) {
    VertLane S;
    S.bad = false;
    S.cp = S.cdd = 0u;
    S.anc = 0;
    S.td = S.tp = 0u;
    if (act) {
        uint32_t tk[6];
        uint32_t pos = vert_header<kShared>(L, d, w, rbase, S, tk);
        const uint32_t n_kind0 = L.d.walk & 0xFFFFu;
        const uint32_t n_delta = n_kind0 ? n_kind0 - 1u : 0u;  // the anchor has no delta
        const uint32_t n_para = (L.d.walk >> 16) - n_kind0;
        const uint32_t end = L.d.end_bit;
        bool ok = !S.bad;
        S.cdd = pos;
#pragma unroll
        for (uint32_t e = 0; e < 3u; e++) {
            S.cdd = e == d ? pos : S.cdd;
            if (ok) ok = skip_codes<kShared>(w, rbase, pos, tk[e], n_delta, end);
        }
        for (uint32_t e = 0; e < d; e++)
            if (ok) ok = skip_codes<kShared>(w, rbase, pos, e == 0u ? tk[3] : tk[4], n_para, end);
        S.cp = pos;
        S.bad = !ok;
        if (ok) {  // the side table: this axis' substream starts after the anchor
            const uint32_t base = L.d.anchor_bit;
            uint16_t* so = a.descs[L.m].sub_offs;
            const uint32_t rp = min(S.cp - base, 0xFFFFu), rd = min(S.cdd - base, 0xFFFFu);
            if (d != 0u) so[d - 1u] = static_cast<uint16_t>(rd);  // dy, dz (dx follows the tags)
            so[2u + d] = static_cast<uint16_t>(rp);                // px, py, pz
        }
    }
    PlaneT<kWide>* plane = reinterpret_cast<PlaneT<kWide>*>(planes + code_off);
    if (act && !S.bad) vert_axis<kShared, kWide>(a, L, d, w, rbase, plane, S);
    __syncwarp();
    emit_axis<kWide, kPair>(a, L, rmask, planes, code_off, d, lane);
    if (act) {
        // pz, the last substream, must end where the next meshlet starts (:507)
        const MeshParams* P = L.P;
        const bool last_of_mesh = L.m - P->meshlet_begin + 1u == P->n_meshlets;
        if (d == 2u && !S.bad && (last_of_mesh ? S.cp > L.d.end_bit : S.cp != L.d.end_bit)) S.bad = true;
        if (S.bad) report(a.status, kErrCorrupt, L.m);
    }
}

// Axis d of group g's 32 meshlets by warp d of the CTA (warps 0..2; a
// fourth warp, d = 3, only joins the CTA's barriers and the stage pass); the
// group's residual bits are staged once and read by all three axis warps.
// False when a stage copy did not arrive in time (reported).
template <bool kWide, bool kPair>
__device__ __forceinline__ bool vert_group(const DecodeArgs& a, uint32_t g, uint32_t d, int lane, uint32_t* stage,
                                           uint8_t* planes, uint64_t* bar, uint32_t& phase, uint32_t vstage,
                                           uint32_t code_bytes) {
    GroupLane L;
    load_group_lane(a, g, lane, L);
    const uint32_t n_local = L.d.counts0 & 0xFFFFu;
    bool ok = L.valid;
    if (ok && !placement_ok(a, L)) {
        if (d == 0u) report(a.status, kErrCorrupt, L.m);
        ok = false;
    }
    // this lane's residual bits: anchor .. end, 16-byte aligned
    const unsigned long long src16 = (L.blob_off + (L.d.anchor_bit >> 3)) & ~15ull;
    const unsigned long long end16 = (L.blob_off + ((L.d.end_bit + 7u) >> 3) + 15ull) & ~15ull;
    const uint32_t ssz = ok ? static_cast<uint32_t>(end16 - src16) : 0u;
    // its stage region: an odd number of 16-byte units, for the reason
    // the code planes have odd word counts (lanes read at about the same
    // offsets at the same time)
    const uint32_t sreg = ssz + ((ssz & 16u) ? 0u : 16u);
    // A lane's code plane is an odd number of words: the walk visits local
    // ids in about the same order in every meshlet, so the lanes read and
    // write at about the same offsets at the same time, and odd strides
    // put those offsets in different banks (16-byte strides used 8).
    const uint32_t csz = 4u * (((n_local * static_cast<uint32_t>(sizeof(PlaneT<kWide>)) + 3u) >> 2) | 1u);
    // the three warps see the same descriptors, so they form the same rounds
    uint32_t todo = __ballot_sync(kFull, ok);
    while (todo) {
        const int first = __ffs(todo) - 1;
        const bool in = (todo >> lane) & 1u;
        uint32_t cc = in ? csz : 0u, cs = in ? sreg : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t1 = __shfl_up_sync(kFull, cc, o);
            const uint32_t t2 = __shfl_up_sync(kFull, cs, o);
            if (lane >= o) {
                cc += t1;
                cs += t2;
            }
        }
        const bool fit = in && cc <= code_bytes && cs <= vstage;
        uint32_t rmask = __ballot_sync(kFull, fit);
        const bool staged = rmask != 0u;
        if (!staged) {  // one meshlet whose residuals exceed the stage: global reads
            rmask = 1u << first;
            cc = in ? csz : 0u;
        }
        todo &= ~rmask;
        const bool act = (rmask >> lane) & 1u;
        const uint32_t code_off = act ? cc - csz : 0u;
        if (staged) {
            // bytes the copies deliver (the regions' padding is not copied)
            const uint32_t total = __reduce_add_sync(kFull, act ? ssz : 0u);
            const uint32_t dst_off = act ? cs - sreg : 0u;
            if (d == 0u) {
                if (lane == 0) mbar_expect(bar, total);
                __syncwarp();
                if (act && ssz)
                    bulk_copy(reinterpret_cast<uint8_t*>(stage) + dst_off, a.arena + src16, ssz, bar);
            }
            const bool timed_out = !mbar_wait(bar, phase, a.wait_clocks);
            if (__syncthreads_or(timed_out)) {
                if (threadIdx.x == 0) report(a.status, kErrTimeout, L.m);
                mbar_wait(bar, phase, 1ll << 31);  // let the copies land before the CTA exits
                return false;
            }
            phase ^= 1u;
            {  // the round's stage in bit order, once for the three warps
                const uint32_t words = __shfl_sync(kFull, cs, 31 - __clz(rmask)) >> 2;
                for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) stage[i] = bswap32(stage[i]);
                __syncthreads();
            }
            const uint32_t rbase = static_cast<uint32_t>(L.blob_off * 8ull - src16 * 8ull + dst_off * 8ull);
            if (d < 3u) vert_round<true, kWide, kPair>(a, L, d, act, rmask, stage, rbase, planes, code_off, lane);
        } else if (d < 3u) {
            vert_round<false, kWide, kPair>(a, L, d, act, rmask,
                                     reinterpret_cast<const uint32_t*>(a.arena + L.blob_off), 0u, planes,
                                     code_off, lane);
        }
        __syncthreads();  // the next round overwrites the stage
    }
    return true;
}

// A CTA decodes one group of 32 meshlets with three warps, warp d = axis d.
template <bool kWide>
__global__ void __launch_bounds__(96, 5) vert_kernel(DecodeArgs a, uint32_t stage_bytes, uint32_t code_bytes,
                                                  int persistent) {
    extern __shared__ __align__(128) uint8_t smem[];
    __shared__ uint32_t s_group;
    const uint32_t d = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const bool failed = *reinterpret_cast<volatile unsigned long long*>(&a.status->err) != 0ull;
    if (__syncthreads_or(failed)) return;  // CTA-uniform: every barrier below is reached by all threads
    const uint32_t vstage = vert_stage_bytes(stage_bytes);
    uint32_t* stage = reinterpret_cast<uint32_t*>(smem);
    uint8_t* planes = smem + align16(vstage + 32u) + d * vert_axis_bytes(code_bytes);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + align16(vstage + 32u) + 3u * vert_axis_bytes(code_bytes));
    if (threadIdx.x == 0) mbar_init(bar);
    __syncthreads();
    uint32_t phase = 0u;
    const uint32_t n_groups = (a.total_meshlets + 31u) / 32u;
    uint32_t f = blockIdx.x;  // position in the group order
    if (persistent) {
        if (threadIdx.x == 0) s_group = atomicAdd(&a.status->work_vert, 1u);
        __syncthreads();
        f = s_group;
    }
    while (f < n_groups) {
        if (!vert_group<kWide, true>(a, group_at(f, n_groups), d, lane, stage, planes, bar, phase, vstage, code_bytes))
            return;
        if (!persistent) break;
        __syncthreads();  // every thread has read s_group
        if (threadIdx.x == 0) s_group = atomicAdd(&a.status->work_vert, 1u);
        __syncthreads();
        f = s_group;
    }
}

// ---------------------------------------------------------------------------
// 4. one kernel for both phases
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Entry i of the completion list: word pad[0] of meshlet 32 i's record
// (i < the number of groups, so the record exists; the scan zeroes it), set
// to group + 1 when the group's connectivity is written.
__device__ __forceinline__ uint32_t* done_entry(const DecodeArgs& a, uint32_t i) { return &a.descs[32u * i].pad[0]; }


// The next group of the vertex phase: the next completion-list entry,
// waited for (bounded: DecodeArgs::wait_clocks, about a second by default).  n_groups when the list
// is used up, the decode has failed, or the wait ran out (reported).
__device__ uint32_t next_done_group(const DecodeArgs& a, uint32_t n_groups) {
    const uint32_t i = atomicAdd(&a.status->work_vert, 1u);
    if (i >= n_groups) return n_groups;
    const uint32_t* e = done_entry(a, i);
    const long long t0 = clock64();
    for (;;) {
        const uint32_t v = ld_acquire_u32(e);
        if (v != 0u) return v - 1u < n_groups ? v - 1u : n_groups;
        if (*reinterpret_cast<volatile unsigned long long*>(&a.status->err) != 0ull) return n_groups;
        if (clock64() - t0 > a.wait_clocks) {
            report(a.status, kErrTimeout, 32u * i);
            return n_groups;
        }
        __nanosleep(256);
    }
}

// Connectivity and vertices in one persistent launch.  Each CTA's two warp
// pairs take connectivity groups (costliest first) until none is left; a
// finished group is appended to the completion list.  Then the CTA turns to
// the vertex phase (its shared memory becomes the stage and the code planes)
// and takes groups from the list in completion order, so the vertex work of
// the groups that finish early runs while the costliest connectivity groups
// are still decoding.  A CTA in the vertex phase waits only for groups that
// running CTAs have taken (every group is taken before any CTA leaves the
// connectivity phase, and that phase waits for nothing), so every wait ends.
// kMinBlocks: CTAs per SM the registers are budgeted for (4: 128 registers
// a thread; 5: 96, which suits large launches).
template <bool kWide, int kMinBlocks>
__global__ void __launch_bounds__(128, kMinBlocks) flow_kernel(DecodeArgs a, uint32_t stage_bytes,
                                                               uint32_t code_bytes) {
    extern __shared__ __align__(128) uint8_t smem[];
    __shared__ uint32_t s_claim[2];
    __shared__ uint32_t s_group;
    __shared__ uint4 mtf_masks[17];
    __shared__ uint32_t s_redo[2];
    if (threadIdx.x < 17u) mtf_masks[threadIdx.x] = threadIdx.x < 16u ? mtf_mask_row(threadIdx.x) : make_uint4(0u, 0u, 0u, 0u);
    // launched as the scan's programmatic dependent: nothing the scan or the
    // status reset writes is read before the scan grid has completed (a
    // no-op after an ordinary launch)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const bool failed = *reinterpret_cast<volatile unsigned long long*>(&a.status->err) != 0ull;
    if (__syncthreads_or(failed)) return;
    const uint32_t n_groups = (a.total_meshlets + 31u) / 32u;
    {
        const uint32_t pair = warp >> 1;
        const bool parser = (warp & 1u) == 0u;
        uint8_t* base = smem + pair * conn_pair_bytes();
        // each pair's first group by position, as the connectivity kernel
        // hands them out (the CTAs dispatched first, one per SM, take two);
        // later groups are taken from the counter
        const uint32_t n_first = min(n_groups, 2u * gridDim.x);
        uint32_t f = blockIdx.x * 2u + pair;
        for (;;) {
            if (f >= n_first) {  // pair-uniform
                if (parser && lane == 0) s_claim[pair] = n_first + atomicAdd(&a.status->work_conn, 1u);
                claim_bar(pair);
                f = s_claim[pair];
            }
            if (f >= n_groups) break;
            const uint32_t g = group_at(f, n_groups);
            conn_group<2>(a, g, pair, parser, lane, base, mtf_masks, s_redo + pair);
            __threadfence();  // this thread's outputs, before the list entry
            claim_bar(pair);  // both warps are done with the group
            if (!parser && lane == 0) st_release_u32(done_entry(a, atomicAdd(&a.status->done_tail, 1u)), g + 1u);
            f = n_first;
        }
    }
    __syncthreads();  // both pairs are through: the memory becomes the vertex layout
    const uint32_t vstage = vert_stage_bytes(stage_bytes);
    uint32_t* stage = reinterpret_cast<uint32_t*>(smem);
    uint8_t* planes = smem + align16(vstage + 32u) + min(warp, 2u) * vert_axis_bytes(code_bytes);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + align16(vstage + 32u) + 3u * vert_axis_bytes(code_bytes));
    if (threadIdx.x == 0) mbar_init(bar);
    __syncthreads();
    uint32_t phase = 0u;
    for (;;) {
        if (threadIdx.x == 0) s_group = next_done_group(a, n_groups);
        __syncthreads();
        const uint32_t g = s_group;
        if (g >= n_groups) return;
        if (!vert_group<kWide, false>(a, g, warp, lane, stage, planes, bar, phase, vstage, code_bytes)) return;
        __syncthreads();  // every thread has read s_group
    }
}

// ---------------------------------------------------------------------------
// launch plumbing
// ---------------------------------------------------------------------------
template <class K>
cudaError_t opt_in_smem(K kernel, size_t smem, size_t* configured) {
    int dev = 0;
    cudaGetDevice(&dev);
    dev = dev < 0 || dev >= 64 ? 0 : dev;
    if (configured[dev] < smem) {
        cudaError_t e =
            cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        // the whole unified L1 as shared memory: both kernels read global
        // data through L2 only, and the default split leaves room for one
        // CTA fewer per SM than the shared-memory size allows
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        configured[dev] = smem;
    }
    return cudaSuccess;
}

// Resident CTAs per SM of one kernel instantiation, cached per device and
// shared-memory size (the occupancy query costs microseconds per launch).
struct OccCache {
    size_t smem[64] = {0};
    int per_sm[64] = {0};
};

template <class K>
uint32_t grid_for(K kernel, int threads, size_t smem, const LaunchCfg& cfg, uint32_t n_groups, int W,
                  OccCache& cache) {
    uint32_t grid = (n_groups + W - 1) / W;
    if (cfg.persistent) {
        int per_sm = cfg.ctas_per_sm;
        if (per_sm <= 0) {
            int dev = 0;
            cudaGetDevice(&dev);
            dev = dev < 0 || dev >= 64 ? 0 : dev;
            if (cache.per_sm[dev] > 0 && cache.smem[dev] == smem) {
                per_sm = cache.per_sm[dev];
            } else {
                per_sm = 1;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
                if (per_sm < 1) per_sm = 1;
                cache.per_sm[dev] = per_sm;
                cache.smem[dev] = smem;
            }
        }
        const uint32_t cap = static_cast<uint32_t>(per_sm * device_sm_count());
        if (grid > cap) grid = cap;
    }
    return grid;
}

// Connectivity pairs per CTA for a launch shape (warps_per_cta 4 -> 2 pairs).
__host__ __device__ constexpr int conn_pairs(int warps_per_cta) { return warps_per_cta >= 4 ? 2 : 1; }

template <int G>
cudaError_t launch_conn(const DecodeArgs& a, const LaunchCfg& cfg, cudaStream_t s) {
    (void)cfg;
    static size_t configured[64] = {0};
    const size_t smem = static_cast<size_t>(G) * conn_pair_bytes();
    cudaError_t e = opt_in_smem(conn_kernel<G>, smem, configured);
    if (e != cudaSuccess) return e;
    const uint32_t g1 = std::min(a.conn_g1, (a.total_meshlets + 31u) / 32u);
    const uint32_t n_groups = g1 - std::min(a.conn_g0, g1);
    const uint32_t grid = (n_groups + G - 1) / G;
    if (grid == 0) return cudaSuccess;
    conn_kernel<G><<<grid, G * 64, smem, s>>>(a);
    return cudaGetLastError();
}

template <bool kWide>
cudaError_t launch_vert(const DecodeArgs& a, const LaunchCfg& cfg, cudaStream_t s) {
    static size_t configured[64] = {0};
    static OccCache occ;
    const size_t smem = vert_cta_bytes(cfg.stage_bytes, cfg.code_bytes);
    cudaError_t e = opt_in_smem(vert_kernel<kWide>, smem, configured);
    if (e != cudaSuccess) return e;
    const uint32_t n_groups = (a.total_meshlets + 31u) / 32u;
    const uint32_t grid = grid_for(vert_kernel<kWide>, 96, smem, cfg, n_groups, 1, occ);
    if (grid == 0) return cudaSuccess;
    vert_kernel<kWide><<<grid, 96, smem, s>>>(a, cfg.stage_bytes, cfg.code_bytes, cfg.persistent);
    note_launch(static_cast<uint32_t>(smem), grid);
    return cudaGetLastError();
}

// Shared memory of a fused CTA: the two pairs' connectivity memory, then
// the vertex layout in the same bytes.
size_t flow_cta_bytes(const LaunchCfg& cfg) {
    return std::max<size_t>(2u * conn_pair_bytes(), vert_cta_bytes(cfg.stage_bytes, cfg.code_bytes));
}

template <bool kWide, int kMinBlocks>
cudaError_t launch_flow(const DecodeArgs& a, const LaunchCfg& cfg, cudaStream_t s, bool after_scan) {
    static size_t configured[64] = {0};
    static OccCache occ;
    const size_t smem = flow_cta_bytes(cfg);
    cudaError_t e = opt_in_smem(flow_kernel<kWide, kMinBlocks>, smem, configured);
    if (e != cudaSuccess) return e;
    const uint32_t n_groups = (a.total_meshlets + 31u) / 32u;
    // one CTA per group (up to the resident count): the vertex phase runs
    // one group per CTA at a time, and pairs that find no connectivity
    // group left go straight to it
    const uint32_t grid = grid_for(flow_kernel<kWide, kMinBlocks>, 128, smem, cfg, n_groups, 1, occ);
    if (grid == 0) return cudaSuccess;
    if (after_scan) {  // the scan kernel directly before it on the stream
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3(grid);
        lc.blockDim = dim3(128);
        lc.dynamicSmemBytes = smem;
        lc.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        lc.attrs = attr;
        lc.numAttrs = 1;
        e = cudaLaunchKernelEx(&lc, flow_kernel<kWide, kMinBlocks>, a, cfg.stage_bytes, cfg.code_bytes);
    } else {
        flow_kernel<kWide, kMinBlocks><<<grid, 128, smem, s>>>(a, cfg.stage_bytes, cfg.code_bytes);
        e = cudaGetLastError();
    }
    note_launch(static_cast<uint32_t>(smem), grid);
    return e;
}

// Groups from which the fused kernel is budgeted for five CTAs per SM.
// Measured on one GB300: up to about 700 groups four CTAs of 128 registers
// are faster (1449^2 heightfield, 666 groups: 164 against 174 us); from
// about 1,300 groups five CTAs of 96 registers are (2897^2 heightfield,
// 2,700 groups: 432 against 460 us; 4,096 mixed meshes: 3.84 against 4.19 ms).
constexpr uint32_t kFlowFiveGroups = 1024u;

cudaError_t launch_flow_any(const DecodeArgs& a, const LaunchCfg& cfg, cudaStream_t s, bool after_scan) {
    const bool five = (a.total_meshlets + 31u) / 32u >= kFlowFiveGroups;
    if (a.wide_codes)
        return five ? launch_flow<true, 5>(a, cfg, s, after_scan) : launch_flow<true, 4>(a, cfg, s, after_scan);
    return five ? launch_flow<false, 5>(a, cfg, s, after_scan) : launch_flow<false, 4>(a, cfg, s, after_scan);
}

// ev[k] is recorded when ev and ev[k] are non-null
void record(void* const* ev, int k, cudaStream_t s) {
    if (ev && ev[k]) cudaEventRecord(static_cast<cudaEvent_t>(ev[k]), s);
}

template <int W>
cudaError_t launch_pair(const DecodeArgs& a, const LaunchCfg& cfg, cudaStream_t s, void* const* ev) {
    cudaError_t e = launch_conn<conn_pairs(W)>(a, cfg, s);
    if (e != cudaSuccess) return e;
    record(ev, 2, s);
    return a.wide_codes ? launch_vert<true>(a, cfg, s) : launch_vert<false>(a, cfg, s);
}

}  // namespace

namespace {
thread_local uint32_t t_launch_smem = 0, t_launch_grid = 0;
}  // namespace

void note_launch(uint32_t smem_bytes, uint32_t grid) {
    t_launch_smem = smem_bytes;
    t_launch_grid = grid;
}

void last_launch(uint32_t* smem_bytes, uint32_t* grid) {
    *smem_bytes = t_launch_smem;
    *grid = t_launch_grid;
}

size_t conn_smem_bytes(const LaunchCfg& cfg) {
    return static_cast<size_t>(conn_pairs(cfg.warps_per_cta)) * conn_pair_bytes();
}

size_t vert_smem_bytes(const LaunchCfg& cfg) { return vert_cta_bytes(cfg.stage_bytes, cfg.code_bytes); }

int device_sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cached[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = n > 0 ? n : 1;
    }
    return cached[dev];
}

__global__ void side_table_kernel(const MeshletDesc* __restrict__ descs, uint32_t n,
                                  unsigned long long* __restrict__ resid_bit, uint16_t* __restrict__ sub_offs) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    resid_bit[m] = __ldcg(&descs[m].anchor_bit);
#pragma unroll
    for (int k = 0; k < 5; k++) sub_offs[5ull * m + k] = __ldcg(&descs[m].sub_offs[k]);
}

int check_config(const LaunchCfg& cfg, bool wide) {
    if (cfg.warps_per_cta != 1 && cfg.warps_per_cta != 2 && cfg.warps_per_cta != 4) return STRIDE_ERR_ARG;
    if (cfg.persistent < 0 || cfg.persistent > 3 || (cfg.persistent == 2 && cfg.warps_per_cta != 4) ||
        (cfg.persistent == 3 && cfg.warps_per_cta > 2))
        return STRIDE_ERR_ARG;
    if (cfg.persistent == 3) return group_smem_bytes(cfg) <= 227u * 1024u ? STRIDE_OK : STRIDE_ERR_ARG;
    // one meshlet of kMaxLocal vertices, its plane padded to an odd word count
    if (cfg.code_bytes < kMaxLocal * (wide ? 4u : 2u) + 4u || cfg.stage_bytes < 256u) return STRIDE_ERR_ARG;
    if (conn_smem_bytes(cfg) > 227u * 1024u || vert_smem_bytes(cfg) > 227u * 1024u) return STRIDE_ERR_ARG;
    if (cfg.persistent == 2 && flow_cta_bytes(cfg) > 227u * 1024u) return STRIDE_ERR_ARG;
    return STRIDE_OK;
}

// Groups from which the default launch shape is the two-kernel one, below
// kFlowFiveGroups.  Measured on one GB300 (step, L2 flushed, every output
// bit-identical), fused against two kernels: 513^2 heightfield (83 groups)
// 0.111 / 0.115 ms, level-8 icosphere (210) 0.137 / 0.121, 1025^2 (331)
// 0.147 / 0.125, 1449^2 (666) 0.177 / 0.173, 2049^2 (1,347) 0.222 / 0.278,
// 2897^2 (2,700) 0.407 / 0.475.  Between these bounds the vertex kernel's
// three-warp CTAs (no idle warp, two meshlets per L2 round trip in the
// output pass) outrun the fused kernel's vertex phase; above them the
// fused kernel's overlap of the two phases wins, below them its single
// launch.
constexpr uint32_t kTwoKernelGroups = 128u;

LaunchCfg default_config(uint32_t total_meshlets) {
    LaunchCfg cfg;
    const uint32_t groups = (total_meshlets + 31u) / 32u;
    cfg.persistent = (groups >= kTwoKernelGroups && groups < kFlowFiveGroups) ? 1 : 2;
    return cfg;
}

namespace {
// The scan kernel over scan blocks [b0, b1), with the blocks that fill the
// dequantisation tables when `tables`.
int launch_scan(const DecodeArgs& a, cudaStream_t s, uint32_t b0, uint32_t b1, bool tables) {
    const uint32_t nb = b1 - b0;
    const uint32_t lut_bx = (a.lut_max + 255u) / 256u;
    const unsigned long long grid = nb + (tables ? static_cast<unsigned long long>(a.n_lut_meshes) * lut_bx : 0ull);
    if (grid > 0x7FFFFFFFull) return STRIDE_ERR_UNSUPPORTED;
    if (grid) {
        scan_kernel<<<static_cast<uint32_t>(grid), kScanThreads, 0, s>>>(a, b0, nb, lut_bx);
        if (cudaGetLastError() != cudaSuccess) return STRIDE_ERR_CUDA;
    }
    return STRIDE_OK;
}
}  // namespace

int enqueue_decode(const DecodeArgs& a, const LaunchCfg& cfg, void* stream, void* const* ev) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (check_config(cfg, a.wide_codes)) return STRIDE_ERR_ARG;
    if (cudaMemsetAsync(a.status, 0, sizeof(Status), s) != cudaSuccess) return STRIDE_ERR_CUDA;
    record(ev, 0, s);
    const int rc = launch_scan(a, s, 0u, scan_blocks(a.total_meshlets), true);
    if (rc) return rc;
    record(ev, 1, s);
    if (a.total_meshlets != 0) {
        cudaError_t e;
        if (cfg.persistent == 3) {  // one warp per group: no connectivity/vertex split
            e = launch_group(a, cfg, s);
            record(ev, 2, s);
        } else if (cfg.persistent == 2) {  // one kernel: the connectivity/vertex split is not timed
            // without timing events between them, the fused kernel is the
            // scan's programmatic dependent
            e = launch_flow_any(a, cfg, s, ev == nullptr);
            record(ev, 2, s);
        } else {
            switch (cfg.warps_per_cta) {
                case 1: e = launch_pair<1>(a, cfg, s, ev); break;
                case 2: e = launch_pair<2>(a, cfg, s, ev); break;
                default: e = launch_pair<4>(a, cfg, s, ev); break;
            }
        }
        if (e != cudaSuccess) return STRIDE_ERR_CUDA;
    } else if (ev) {
        record(ev, 2, s);
    }
    record(ev, 3, s);
    return STRIDE_OK;
}

int enqueue_parts_begin(const DecodeArgs& a, const LaunchCfg& cfg, void* stream) {
    if (cfg.persistent >= 2) return STRIDE_ERR_ARG;
    if (check_config(cfg, a.wide_codes)) return STRIDE_ERR_ARG;
    return cudaMemsetAsync(a.status, 0, sizeof(Status), static_cast<cudaStream_t>(stream)) == cudaSuccess
               ? STRIDE_OK
               : STRIDE_ERR_CUDA;
}

int enqueue_part(const DecodeArgs& a, const LaunchCfg& cfg, void* stream, uint32_t g0, uint32_t g1, bool first,
                 void* bytes_in, void* scan_done, void* conn_done) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (bytes_in && cudaStreamWaitEvent(s, static_cast<cudaEvent_t>(bytes_in), 0) != cudaSuccess)
        return STRIDE_ERR_CUDA;
    // the part's windows are its scan blocks
    const uint32_t nb = scan_blocks(a.total_meshlets);
    const uint32_t b0 = std::min(g0 / 8u, nb), b1 = std::max(b0, std::min((g1 + 7u) / 8u, nb));
    const int rc = launch_scan(a, s, b0, b1, first);
    if (rc) return rc;
    if (scan_done && cudaEventRecord(static_cast<cudaEvent_t>(scan_done), s) != cudaSuccess) return STRIDE_ERR_CUDA;
    DecodeArgs ap = a;
    ap.conn_g0 = g0;
    ap.conn_g1 = g1;
    cudaError_t e;
    switch (cfg.warps_per_cta) {
        case 1: e = launch_conn<conn_pairs(1)>(ap, cfg, s); break;
        case 2: e = launch_conn<conn_pairs(2)>(ap, cfg, s); break;
        default: e = launch_conn<conn_pairs(4)>(ap, cfg, s); break;
    }
    if (e != cudaSuccess) return STRIDE_ERR_CUDA;
    if (conn_done && cudaEventRecord(static_cast<cudaEvent_t>(conn_done), s) != cudaSuccess) return STRIDE_ERR_CUDA;
    return STRIDE_OK;
}

int enqueue_parts_end(const DecodeArgs& a, const LaunchCfg& cfg, void* stream, void* vert_done) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (a.total_meshlets != 0) {
        const cudaError_t e = a.wide_codes ? launch_vert<true>(a, cfg, s) : launch_vert<false>(a, cfg, s);
        if (e != cudaSuccess) return STRIDE_ERR_CUDA;
    }
    if (vert_done && cudaEventRecord(static_cast<cudaEvent_t>(vert_done), s) != cudaSuccess) return STRIDE_ERR_CUDA;
    return STRIDE_OK;
}

// ---------------------------------------------------------------------------
// Meshlet-native outputs: ranges, bounds, frustum culling
// ---------------------------------------------------------------------------
__device__ __forceinline__ void meshlet_rows(const MeshletDesc* descs, const BlockPrefix* bp, uint32_t m,
                                             unsigned long long& v0, unsigned long long& t0, uint32_t& nv,
                                             uint32_t& nt) {
    const BlockPrefix& p = bp[m / kScanThreads];
    const uint32_t c = __ldcg(&descs[m].counts0);
    v0 = __ldcg(&p.v) + __ldcg(&descs[m].v_pref);
    t0 = __ldcg(&p.t) + __ldcg(&descs[m].t_pref);
    nv = c & 0xFFFFu;
    nt = c >> 16;
}

__global__ void meshlet_ranges_kernel(const MeshletDesc* __restrict__ descs, const BlockPrefix* __restrict__ bp,
                                      uint32_t n, unsigned long long* __restrict__ v_first,
                                      unsigned long long* __restrict__ t_first) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    unsigned long long v0, t0;
    uint32_t nv, nt;
    meshlet_rows(descs, bp, m, v0, t0, nv, nt);
    v_first[m] = v0;
    t_first[m] = t0;
    if (m + 1u == n) {
        v_first[n] = v0 + nv;
        t_first[n] = t0 + nt;
    }
}

// One warp per meshlet: min / max of each coordinate over its rows of pos.
__global__ void meshlet_bounds_kernel(const MeshletDesc* __restrict__ descs, const BlockPrefix* __restrict__ bp,
                                      uint32_t n, const float* __restrict__ pos, float* __restrict__ bounds) {
    const uint32_t m = blockIdx.x * (blockDim.x / 32u) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (m >= n) return;  // warp-uniform
    unsigned long long v0, t0;
    uint32_t nv, nt;
    meshlet_rows(descs, bp, m, v0, t0, nv, nt);
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    const float* base = pos + 3ull * v0;
    for (uint32_t i = lane; i < 3u * nv; i += 32u) {  // the meshlet's floats, coalesced
        const float x = __ldcg(base + i);
        const uint32_t d = i % 3u;  // base is a row start
        lo[0] = d == 0u ? fminf(lo[0], x) : lo[0];
        lo[1] = d == 1u ? fminf(lo[1], x) : lo[1];
        lo[2] = d == 2u ? fminf(lo[2], x) : lo[2];
        hi[0] = d == 0u ? fmaxf(hi[0], x) : hi[0];
        hi[1] = d == 1u ? fmaxf(hi[1], x) : hi[1];
        hi[2] = d == 2u ? fmaxf(hi[2], x) : hi[2];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            lo[d] = fminf(lo[d], __shfl_xor_sync(kFull, lo[d], o));
            hi[d] = fmaxf(hi[d], __shfl_xor_sync(kFull, hi[d], o));
        }
    }
    if (lane < 6) bounds[6ull * m + lane] = lane < 3 ? lo[lane] : hi[lane - 3];
}

// A box is culled when it lies wholly on the outer side of one plane: its
// corner furthest along the plane normal (the p-vertex) has
// a x + b y + c z + d < 0.  Evaluated left to right without contraction.
// An empty meshlet's box (min > max) is culled.
__global__ void cull_kernel(const float* __restrict__ bounds, uint32_t n, Planes pl, uint32_t* __restrict__ visible,
                            uint32_t* __restrict__ count) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    bool vis = false;
    if (m < n) {
        const float* b = bounds + 6ull * m;
        const float x0 = b[0], y0 = b[1], z0 = b[2], x1 = b[3], y1 = b[4], z1 = b[5];
        vis = x0 <= x1 && y0 <= y1 && z0 <= z1;
#pragma unroll
        for (int k = 0; k < 6; k++) {
            const float a = pl.p[4 * k], bb = pl.p[4 * k + 1], c = pl.p[4 * k + 2], d = pl.p[4 * k + 3];
            const float px = a >= 0.f ? x1 : x0, py = bb >= 0.f ? y1 : y0, pz = c >= 0.f ? z1 : z0;
            const float s = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a, px), __fmul_rn(bb, py)), __fmul_rn(c, pz)), d);
            vis = vis && !(s < 0.f);
        }
    }
    const uint32_t word = __ballot_sync(kFull, vis);
    if ((threadIdx.x & 31) == 0 && m < n) {  // lane 0 holds the warp's first meshlet: word m / 32 exists
        visible[m / 32u] = word;
        if (word) atomicAdd(count, static_cast<uint32_t>(__popc(word)));
    }
}

int enqueue_meshlet_ranges(const MeshletDesc* descs, const BlockPrefix* bp, uint32_t n, unsigned long long* v_first,
                           unsigned long long* t_first, void* stream) {
    if (n == 0u) return STRIDE_OK;
    meshlet_ranges_kernel<<<(n + 255u) / 256u, 256, 0, static_cast<cudaStream_t>(stream)>>>(descs, bp, n, v_first,
                                                                                              t_first);
    return cudaGetLastError() == cudaSuccess ? STRIDE_OK : STRIDE_ERR_CUDA;
}

int enqueue_meshlet_bounds(const MeshletDesc* descs, const BlockPrefix* bp, uint32_t n, const float* pos,
                           float* bounds, void* stream) {
    if (n == 0u) return STRIDE_OK;
    meshlet_bounds_kernel<<<(n + 7u) / 8u, 256, 0, static_cast<cudaStream_t>(stream)>>>(descs, bp, n, pos, bounds);
    return cudaGetLastError() == cudaSuccess ? STRIDE_OK : STRIDE_ERR_CUDA;
}

int enqueue_cull(const float* bounds, uint32_t n, const Planes& planes, uint32_t* visible, uint32_t* count,
                 void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(count, 0, sizeof(uint32_t), s) != cudaSuccess) return STRIDE_ERR_CUDA;
    if (n == 0u) return STRIDE_OK;
    cull_kernel<<<(n + 255u) / 256u, 256, 0, s>>>(bounds, n, planes, visible, count);
    return cudaGetLastError() == cudaSuccess ? STRIDE_OK : STRIDE_ERR_CUDA;
}

int enqueue_side_table(const MeshletDesc* descs, uint32_t n, unsigned long long* resid_bit, uint16_t* sub_offs,
                       void* stream) {
    if (n == 0u) return STRIDE_OK;
    side_table_kernel<<<(n + 255u) / 256u, 256, 0, static_cast<cudaStream_t>(stream)>>>(descs, n, resid_bit,
                                                                                          sub_offs);
    return cudaGetLastError() == cudaSuccess ? STRIDE_OK : STRIDE_ERR_CUDA;
}

}  // namespace stride
