// Device helpers shared by the STRIDE decode kernels: MSB-first bit access,
// Rice / Exp-Golomb codeword readers (utils/bit_codec.py:199-254), the
// per-lane byte rings and bulk-copy staging, output rings, group
// bookkeeping (meshlet records, placement checks, group order), and the
// warp-cooperative coordinate emission with exact dequantisation.
//
// Everything here has internal linkage: each kernel translation unit gets
// its own copy.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <type_traits>

#include "stride_common.cuh"

namespace stride {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// Bit access: MSB-first stream read as big-endian 32-bit words.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0u, 0x0123u); }

// Global data is read through L2 only (ld.global.cg here, and every plain
// global load of this file is compiled with -dlcm=cg): the serving engine
// rewrites arena ranges (streams, mesh tables, dequantisation tables) for a
// new launch while launches on other streams may still run on the same SMs,
// so nothing may be served from an SM's L1 or read-only cache.
//
// ldw returns word i in bit order (the stream's first bit as the MSB).  The
// vertex kernel's stage is put in bit order once when it lands, so reads
// from it need no byte swap; global words are swapped as they are read.
template <bool kShared>
__device__ __forceinline__ uint32_t ldw(const uint32_t* w, uint32_t i) {
    if constexpr (kShared) {
        return w[i];
    } else {
        return bswap32(__ldcg(w + i));
    }
}

// 32 bits starting at bit `rel` of the word array.
template <bool kShared>
__device__ __forceinline__ uint32_t peek32(const uint32_t* w, uint32_t rel) {
    const uint32_t i = rel >> 5;
    const uint32_t hi = ldw<kShared>(w, i);
    const uint32_t lo = ldw<kShared>(w, i + 1);
    return __funnelshift_l(lo, hi, rel & 31u);
}

__device__ __forceinline__ void report(Status* st, int code, uint32_t meshlet) {
    const unsigned long long v = (static_cast<unsigned long long>(static_cast<unsigned>(code)) << 32) | meshlet;
    atomicCAS(&st->err, 0ull, v);
}

// One Rice(k) / Exp-Golomb(k) codeword (utils/bit_codec.py:226-250).
// tk bit 7 selects Exp-Golomb (a tag other than 1, paradelta_v5_dup.py:563-567),
// bits 0..5 hold k.  `limit` is the meshlet's end bit.
template <bool kShared>
__device__ __forceinline__ int read_code(const uint32_t* w, uint32_t rbase, uint32_t& pos,
                                         uint32_t tk, uint32_t limit, uint32_t& u) {
    const bool eg = (tk & 0x80u) != 0u;
    const uint32_t k = tk & 0x3Fu;
    uint32_t x = peek32<kShared>(w, pos + rbase);
    uint32_t z;
    if (x != 0u) {
        z = __clz(x);
    } else {  // unary prefix of 32 or more zeros
        z = 32u;
        for (;;) {
            if (pos + z >= limit) return kErrCorrupt;
            const uint32_t y = peek32<kShared>(w, pos + z + rbase);
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
    if (nb) {
        if (z + 1u + nb <= 32u) {
            val = (x << (z + 1u)) >> (32u - nb);
        } else {
            val = peek32<kShared>(w, p1 + rbase) >> (32u - nb);
        }
    }
    const unsigned long long base = eg ? ((1ull << z) - 1ull) : static_cast<unsigned long long>(z);
    const unsigned long long uu = (base << k) + val;
    if (uu >> 32) return kErrUnsupported;
    pos = p1 + nb;
    if (pos > limit) return kErrCorrupt;
    u = static_cast<uint32_t>(uu);
    return 0;
}

__device__ __forceinline__ int32_t unzigzag(uint32_t u) {
    return static_cast<int32_t>((u >> 1) ^ (0u - (u & 1u)));
}

__device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int src) {
    return __shfl_sync(kFull, v, src);
}

// Sequential reader of one lane's bits through a three-word register
// window: peeking costs one funnel shift, and the shared/global load that
// refills the window is issued a word ahead of its use, off the chain that
// carries the bit position.  Reads reach at most 95 bits past `pos`.
template <bool kShared>
struct BitWin {
    const uint32_t* w;
    uint32_t rbase, pos, w0, w1, w2;
    __device__ __forceinline__ void seek(uint32_t p) {
        pos = p;
        const uint32_t i = (p + rbase) >> 5;
        w0 = ldw<kShared>(w, i);
        w1 = ldw<kShared>(w, i + 1u);
        w2 = ldw<kShared>(w, i + 2u);
    }
    __device__ __forceinline__ uint32_t peek() const { return __funnelshift_l(w1, w0, (pos + rbase) & 31u); }
    // len <= 32: crosses at most one word boundary
    __device__ __forceinline__ void advance(uint32_t len) {
        const uint32_t np = pos + len;
        const uint32_t i = (np + rbase) >> 5;
        const bool cross = i != ((pos + rbase) >> 5);
        pos = np;
        if (cross) {
            w0 = w1;
            w1 = w2;
            w2 = ldw<kShared>(w, i + 2u);
        }
    }
};

// ---------------------------------------------------------------------------
// Bulk-copy staging (TMA bulk, no tensor map) and its mbarrier.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    unsigned long long gsrc;
    asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(gsrc) : "l"(src));
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(gsrc), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0u;
}

// Non-blocking check of the phase.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0u;
}

// Bounded wait (`limit` SM clocks, DecodeArgs::wait_clocks); false on
// timeout.  The first check does not block and the clock is read before
// every (blocking) try, so a limit of 0 gives up as soon as the phase is
// found incomplete.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, long long limit) {
    if (mbar_test_wait(bar, phase)) return true;
    const long long t0 = clock64();
    for (;;) {
        if (clock64() - t0 > limit) return false;
        if (mbar_try_wait(bar, phase)) return true;
    }
}

// ---------------------------------------------------------------------------
// Per-lane byte rings of the connectivity parser.  Each lane streams its own
// meshlet through a 64-word ring in shared memory, 32 words (128 bytes) per
// chunk, fetched with 16-byte cp.async copies (L2 only) a chunk ahead of the
// bit cursor.  Word j of the lane's data (counted from its 16-byte aligned
// first byte) sits at ring[(j + rot) & 63]; the per-lane rotation (a
// multiple of four words) spreads lanes that read the same relative word
// over different banks.
// ---------------------------------------------------------------------------
constexpr uint32_t kLaneRingWords = 64u;
constexpr uint32_t kLaneChunkWords = 32u;

__device__ __forceinline__ void cp_async16(uint32_t* dst, const uint8_t* src, uint32_t src_bytes) {
    unsigned long long gsrc;
    asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(gsrc) : "l"(src));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(gsrc), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Chunk c of a lane's data: bytes [128c, 128c + 128) from `src` (16-byte
// aligned); 16-byte units at or past `avail` are zero-filled without a read.
__device__ __forceinline__ void ring_fetch(uint32_t* ring, const uint8_t* src, uint32_t avail, uint32_t rot,
                                           uint32_t c) {
#pragma unroll
    for (uint32_t u = 0; u < kLaneChunkWords / 4u; u++) {
        const uint32_t off = c * (4u * kLaneChunkWords) + 16u * u;
        const bool in = off < avail;
        cp_async16(ring + ((c * kLaneChunkWords + 4u * u + rot) & (kLaneRingWords - 1u)), in ? src + off : src,
                   in ? 16u : 0u);
    }
}


// Output rings.  Each lane collects its triangles (packed local ids) and its
// walk entries in a 32-slot row of shared memory; every kFlushEvery token
// iterations the warp writes whole 4-entry quads out with 16-byte stores
// (a quad of triangles is 48 bytes starting at a triangle index divisible by
// four), and at the end of the meshlet the unaligned head and tail go out as
// single words.  A row is 36 words so that quads stay 16-byte aligned.
constexpr uint32_t kRing = 32;
constexpr uint32_t kRingRow = 36;
constexpr uint32_t kFlushEvery = kRing - 4;  // a pending partial quad (<= 3) + new entries fit

// Triangles [tf, tcnt) of one lane (local indices; the first triangle has
// global index t_base, with ph = t_base & 3 and slot (ph + local) mod kN;
// kN, the ring's entries, is a power of two).
template <uint32_t kN = kRing>
__device__ __forceinline__ void flush_tris(uint32_t* idx, unsigned long long t_base, const uint32_t* ring,
                                           uint32_t& tf, uint32_t tcnt, uint32_t vloc, bool final) {
    auto id = [vloc](uint32_t packed, uint32_t k) { return vloc + ((packed >> (8u * k)) & 0xFFu); };
    const uint32_t ph = static_cast<uint32_t>(t_base) & 3u;
    const uint32_t h = tf + ((4u - ((ph + tf) & 3u)) & 3u);  // first quad-aligned local index >= tf
    const uint32_t he = min(h, tcnt);
    const uint32_t r = (ph + tcnt) & 3u;
    const uint32_t qe = tcnt >= r ? tcnt - r : 0u;            // end of the last whole quad (0: none)
    uint32_t* out = idx + 3ull * t_base;
    for (uint32_t l = tf; l < he; l++) {  // head: up to 3 triangles
        const uint32_t p = ring[(ph + l) & (kN - 1u)];
        out[3u * l] = id(p, 0);
        out[3u * l + 1u] = id(p, 1);
        out[3u * l + 2u] = id(p, 2);
    }
    for (uint32_t l = h; l < qe; l += 4u) {
        const uint4 q = *reinterpret_cast<const uint4*>(ring + ((ph + l) & (kN - 1u)));
        uint4* o = reinterpret_cast<uint4*>(out + 3u * l);
        o[0] = make_uint4(id(q.x, 0), id(q.x, 1), id(q.x, 2), id(q.y, 0));
        o[1] = make_uint4(id(q.y, 1), id(q.y, 2), id(q.z, 0), id(q.z, 1));
        o[2] = make_uint4(id(q.z, 2), id(q.w, 0), id(q.w, 1), id(q.w, 2));
    }
    const uint32_t done = max(he, qe);
    if (final) {
        for (uint32_t l = done; l < tcnt; l++) {  // tail: up to 3 triangles
            const uint32_t p = ring[(ph + l) & (kN - 1u)];
            out[3u * l] = id(p, 0);
            out[3u * l + 1u] = id(p, 1);
            out[3u * l + 2u] = id(p, 2);
        }
        tf = tcnt;
    } else {
        tf = done;
    }
}

// Walk entries [wf, wcnt) of one lane; the lane's walk region starts 16-byte
// aligned, so quads start at local indices divisible by four.
template <uint32_t kN = kRing>
__device__ __forceinline__ void flush_walk(uint32_t* out, const uint32_t* ring, uint32_t& wf, uint32_t wcnt,
                                           bool final) {
    const uint32_t qe = wcnt & ~3u;
    for (uint32_t l = wf; l < qe; l += 4u)
        *reinterpret_cast<uint4*>(out + l) = *reinterpret_cast<const uint4*>(ring + (l & (kN - 1u)));
    if (final) {
        for (uint32_t l = max(wf, qe); l < wcnt; l++) out[l] = ring[l & (kN - 1u)];
        wf = wcnt;
    } else {
        wf = max(wf, qe);
    }
}

__host__ __device__ constexpr uint32_t align16(uint32_t x) { return (x + 15u) & ~15u; }

struct GroupLane {
    uint32_t m;
    bool valid;
    MeshletDesc d;
    uint32_t mi;
    const MeshParams* P;
    unsigned long long v_base, t_base, wp_base;
    unsigned long long blob_off;
};

// Order in which the decode kernels take groups.  The scan sorts each
// 256-meshlet window ascending by token count, so a window's groups (eight)
// grow costlier with their index; taking every window's last group first and
// every window's first group last approximates costliest-first: the cheap
// groups land on the CTAs dispatched last (the extra CTA some SMs get) and at
// the end of the vertex kernel's work queue.  Entry f -> group; a bijection
// of [0, n_groups).
__device__ __forceinline__ uint32_t group_at(uint32_t f, uint32_t n_groups) {
    constexpr uint32_t kPer = kScanThreads / 32u;  // groups per window
    const uint32_t nw = (n_groups + kPer - 1u) / kPer;
    const uint32_t q = n_groups - kPer * (nw - 1u);  // groups in the last window, 1..kPer
    const uint32_t head = (kPer - q) * (nw - 1u);     // entries of the levels the last window lacks
    uint32_t l, w;
    if (f < head) {
        l = kPer - 1u - f / (nw - 1u);
        w = f % (nw - 1u);
    } else {
        const uint32_t r = f - head;
        l = q - 1u - r / nw;
        w = r % nw;
    }
    return kPer * w + l;
}

__device__ __forceinline__ void load_group_lane(const DecodeArgs& a, uint32_t g, int lane, GroupLane& L) {
    const uint32_t slot = g * 32u + lane;
    L.valid = slot < a.total_meshlets;
    L.m = L.valid ? __ldcg(&a.descs[slot].slot_meshlet) : slot;
    if (L.valid) {
        const uint4* src = reinterpret_cast<const uint4*>(a.descs + L.m);
        uint4* dst = reinterpret_cast<uint4*>(&L.d);
        dst[0] = __ldcg(src);
        dst[1] = __ldcg(src + 1);
        dst[2] = __ldcg(src + 2);
        dst[3] = __ldcg(src + 3);
        const BlockPrefix& bp = a.blk_prefix[L.m / kScanThreads];
        L.v_base = bp.v + L.d.v_pref;
        L.t_base = bp.t + L.d.t_pref;
        L.wp_base = bp.wp + L.d.wp_pref;
    } else {
        memset(&L.d, 0, sizeof(L.d));
        L.v_base = L.t_base = L.wp_base = 0ull;
    }
    L.mi = (L.valid && a.meshlet_mesh) ? __ldcg(a.meshlet_mesh + L.m) : 0u;
    L.P = a.meshes + L.mi;
    L.blob_off = L.valid ? L.P->blob_off : 0ull;
}

// The meshlet's output ranges lie inside its mesh's (header n_v_total, n_t)
// and the mesh's last meshlet ends exactly there; checked before anything is
// written, so a stream whose counts disagree with its header is rejected
// instead of writing into a neighbour's output.
__device__ __forceinline__ bool placement_ok(const DecodeArgs& a, const GroupLane& L) {
    const uint32_t n_local = L.d.counts0 & 0xFFFFu;
    const uint32_t n_tris = L.d.counts0 >> 16;
    const unsigned long long vo = L.P->v_offset, to = L.P->t_offset, nv = L.P->n_v, nt = L.P->n_t;
    bool ok = L.v_base >= vo && L.v_base + n_local <= vo + nv && L.t_base >= to && L.t_base + n_tris <= to + nt;
    if (ok && L.m - L.P->meshlet_begin + 1u == L.P->n_meshlets)
        ok = L.v_base + n_local == vo + nv && L.t_base + n_tris == to + nt;
    return ok && L.wp_base + ((n_local + 3u) & ~3u) <= a.walk_cap;
}

// One axis of a meshlet's integer codes in shared memory: 16 bits per vertex
// for codes of up to 16 bits, 32 above.
template <bool kWide>
using PlaneT = typename std::conditional<kWide, int32_t, uint16_t>::type;

// Exact float64 evaluation for the codes whose float-float result is too
// close to a float32 rounding boundary (well under 1 in 1000): out of line,
// so the common path stays short and branch-free.
__device__ __noinline__ float dequant_slow(const MeshParams* P, uint32_t axis, uint32_t q) {
    return stride_dequant_exact(&P->dq[axis], q);
}

// Residual of one axis: Rice/EG codeword at `pos` with a straight-line fast
// path (prefix and value inside one 32-bit window); the general reader runs
// inline behind the only branch, taken for codewords longer than 32 bits.
// Returns false on a malformed codeword; `pos` never passes `limit`, so a
// corrupt stream cannot steer reads outside the meshlet.
template <bool kShared>
__device__ __forceinline__ bool residual(const uint32_t* w, uint32_t rbase, uint32_t& pos, uint32_t tk,
                                         uint32_t limit, int32_t& r) {
    const uint32_t x = peek32<kShared>(w, pos + rbase);
    const uint32_t z = __clz(x);
    const uint32_t k = tk & 0x3Fu;
    const bool eg = (tk & 0x80u) != 0u;
    const uint32_t nb = (eg ? z : 0u) + k;
    const uint32_t len = z + 1u + nb;
    const uint32_t t = __funnelshift_lc(0u, x, z + 1u);      // bits after the terminator
    const uint32_t val = __funnelshift_rc(t, 0u, 32u - nb);  // the top nb of them
    const uint32_t base = eg ? ((1u << (z & 31u)) - 1u) : z;
    uint32_t u = (base << k) + val;
    uint32_t np = pos + len;
    bool ok = true;
    if (len > 32u) {  // long prefix or long value: rare
        np = pos;
        ok = read_code<kShared>(w, rbase, np, tk, limit, u) == 0;
    }
    ok = ok && np <= limit;
    pos = min(np, limit);
    r = unzigzag(u);
    return ok;
}

// Skip n codewords (substream boundaries are not stored in the stream).
// Rice(0) codewords (the common case: smooth residuals) are skipped by
// counting one bits, about twenty per step; others up to four per step,
// those that lie wholly inside the 32-bit window (a bit scan per codeword,
// about 80 cycles each measured on one warp); a codeword longer than the
// window goes to the general reader.  (An 8-bit table of whole codewords
// per step measured slower than both on mixed warps.)
template <bool kShared>
__device__ __forceinline__ bool skip_codes(const uint32_t* w, uint32_t rbase, uint32_t& pos, uint32_t tk,
                                           uint32_t n, uint32_t limit) {
    const uint32_t k = tk & 0x3Fu;
    const bool eg = (tk & 0x80u) != 0u;
    bool ok = true;
    BitWin<kShared> b;
    b.w = w;
    b.rbase = rbase;
    b.seek(pos);
    if (!eg && k == 0u) {
        // Rice(0) codewords are unary: each ends at a one bit, so skipping n
        // of them is finding the n-th one bit -- a population count per 32
        // bits, then a five-step halving search inside the last window.
        while (n > 0u) {
            const uint32_t x = b.peek();
            const uint32_t c = __popc(x);
            if (c < n) {
                b.advance(32u);
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
                b.advance(at + 1u);  // through the n-th one
                n = 0u;
            }
            if (b.pos > limit) {  // only a corrupt stream runs past its meshlet
                ok = false;
                b.seek(limit);
                break;
            }
        }
        pos = b.pos;
        return ok;
    }
    while (n > 0u) {
        const uint32_t x = b.peek();
        uint32_t used = 0u, cnt = 0u;
#pragma unroll
        for (int s = 0; s < 4; s++) {
            const uint32_t xx = __funnelshift_lc(0u, x, used);  // the window past the codewords taken
            const uint32_t z = __clz(xx);                       // 32 when nothing is left
            const uint32_t len = z + 1u + (eg ? z : 0u) + k;
            const bool fits = (used + len <= 32u) & (cnt < n);
            used += fits ? len : 0u;
            cnt += fits ? 1u : 0u;
        }
        if (cnt) {
            b.advance(used);
            n -= cnt;
        } else {  // prefix or value beyond the window: general reader
            uint32_t u, np = b.pos;
            ok = ok & (read_code<kShared>(w, rbase, np, tk, limit, u) == 0);
            b.seek(min(np, limit));
            n--;
        }
        if (b.pos > limit) {  // only a corrupt stream runs past its meshlet
            ok = false;
            b.seek(limit);
        }
    }
    pos = b.pos;
    return ok;
}

// The same codeword read without a branch, for codewords that fit the
// 32-bit window (prefix, terminator and value); a longer one sets `longc`
// and leaves the result undefined.  The walk uses this form so that the
// compiler can overlap consecutive walk entries (a branch per entry keeps
// them apart: 5% of the fused kernel on the 2049^2 heightfield).
template <bool kShared>
__device__ __forceinline__ bool residual_fast(const uint32_t* w, uint32_t rbase, uint32_t& pos, uint32_t tk,
                                              uint32_t limit, int32_t& r, bool& longc) {
    const uint32_t x = peek32<kShared>(w, pos + rbase);
    const uint32_t z = __clz(x);
    const uint32_t k = tk & 0x3Fu;
    const bool eg = (tk & 0x80u) != 0u;
    const uint32_t nb = (eg ? z : 0u) + k;
    const uint32_t len = z + 1u + nb;
    const uint32_t t = __funnelshift_lc(0u, x, z + 1u);
    const uint32_t val = __funnelshift_rc(t, 0u, 32u - nb);
    const uint32_t base = eg ? ((1u << (z & 31u)) - 1u) : z;
    const uint32_t u = (base << k) + val;
    const uint32_t np = pos + len;
    longc = longc | (len > 32u);
    const bool ok = np <= limit;
    pos = min(np, limit);
    r = unzigzag(u);
    return ok;
}

// Axis d of every vertex of the round's meshlets -> positions (and codes),
// the warp working through one meshlet at a time (n_local <= kMaxLocal, so
// a meshlet's table reads all go out before its first store: one L2 round
// trip per meshlet).  The mesh's constants
// (table base, or float-float dequantisation coefficients) stay in registers
// while consecutive meshlets belong to the same mesh.
// With kPair, two consecutive meshlets of the same mesh with at most 128
// vertices each share one L2 round trip (all eight table reads of a lane in
// flight before the stores): the vertex kernel alone runs 5-10% faster
// (2049^2 heightfield 142 -> 132 us, 513^2 57 -> 51 us); the fused kernel,
// whose registers are budgeted tighter, measured no gain.
template <bool kWide, bool kPair = false>
__device__ void emit_axis(const DecodeArgs& a, const GroupLane& L, uint32_t rmask, const uint8_t* planes,
                          uint32_t code_off, uint32_t d, int lane) {
    uint32_t cached = 0xFFFFFFFFu;
    const MeshParams* Pj = a.meshes;
    stride_dequant_axis c;
    c.a_hi = c.a_lo = c.b_hi = c.b_lo = c.err = 0.f;
    bool zero_bits = false, has_lut = false;
    const float* lut = nullptr;
    uint32_t qmax = 0u;
    for (uint32_t mm = rmask; mm; mm &= mm - 1u) {
        const int j = __ffs(mm) - 1;
        const uint32_t nv = __shfl_sync(kFull, L.d.counts0, j) & 0xFFFFu;
        const unsigned long long vb = shfl64(L.v_base, j);
        const uint32_t off = __shfl_sync(kFull, code_off, j);
        const uint32_t mj = __shfl_sync(kFull, L.mi, j);
        if (mj != cached) {  // warp-uniform
            cached = mj;
            Pj = a.meshes + mj;
            has_lut = __ldcg(&Pj->has_lut) != 0;
            if (has_lut) {
                const uint32_t g0 = __ldcg(&Pj->g_bits[0]), g1 = __ldcg(&Pj->g_bits[1]);
                lut = a.lut + __ldcg(&Pj->lut_off) + (d >= 1u ? 1u << g0 : 0u) + (d >= 2u ? 1u << g1 : 0u);
                qmax = (1u << __ldcg(&Pj->g_bits[d])) - 1u;  // a corrupt stream's codes may lie outside
            } else {
                c.a_hi = __ldcg(&Pj->dq[d].a_hi);
                c.a_lo = __ldcg(&Pj->dq[d].a_lo);
                c.b_hi = __ldcg(&Pj->dq[d].b_hi);
                c.b_lo = __ldcg(&Pj->dq[d].b_lo);
                c.err = __ldcg(&Pj->dq[d].err);
                zero_bits = __ldcg(&Pj->dq[d].zero_bits) != 0;
            }
        }
        if constexpr (kPair) {
            if (has_lut && ((mm & (mm - 1u)) != 0u) && nv <= 128u) {  // warp-uniform: a second meshlet follows
                const uint32_t m2 = mm & (mm - 1u);
                const int j2 = __ffs(m2) - 1;
                const uint32_t nv2 = __shfl_sync(kFull, L.d.counts0, j2) & 0xFFFFu;
                const uint32_t mj2 = __shfl_sync(kFull, L.mi, j2);
                if (mj2 == cached && nv2 <= 128u) {
                    const unsigned long long vb2 = shfl64(L.v_base, j2);
                    const uint32_t off2 = __shfl_sync(kFull, code_off, j2);
                    const PlaneT<kWide>* p1 = reinterpret_cast<const PlaneT<kWide>*>(planes + off);
                    const PlaneT<kWide>* p2 = reinterpret_cast<const PlaneT<kWide>*>(planes + off2);
                    float y1[4], y2[4];
#pragma unroll
                    for (uint32_t k = 0; k < 4u; k++) {
                        const uint32_t v = lane + 32u * k;
                        y1[k] = v < nv ? __ldcg(lut + min(static_cast<uint32_t>(p1[v]), qmax)) : 0.f;
                        y2[k] = v < nv2 ? __ldcg(lut + min(static_cast<uint32_t>(p2[v]), qmax)) : 0.f;
                    }
                    float* d1 = a.pos + 3ull * vb + d;
                    float* d2 = a.pos + 3ull * vb2 + d;
#pragma unroll
                    for (uint32_t k = 0; k < 4u; k++) {
                        const uint32_t v = lane + 32u * k;
                        if (v < nv) d1[3u * v] = y1[k];
                        if (v < nv2) d2[3u * v] = y2[k];
                    }
                    if (a.codes) {
                        int32_t* c1 = a.codes + 3ull * vb + d;
                        int32_t* c2 = a.codes + 3ull * vb2 + d;
                        for (uint32_t v = lane; v < nv; v += 32u) c1[3u * v] = static_cast<int32_t>(p1[v]);
                        for (uint32_t v = lane; v < nv2; v += 32u) c2[3u * v] = static_cast<int32_t>(p2[v]);
                    }
                    mm = m2;  // the loop's step clears the second meshlet's bit
                    continue;
                }
            }
        }
        const PlaneT<kWide>* pj = reinterpret_cast<const PlaneT<kWide>*>(planes + off);
        float* dst = a.pos + 3ull * vb + d;
        if (has_lut) {  // every table read of the meshlet (<= 256 vertices) in flight at once
            const uint32_t ns = (nv + 31u) >> 5;  // slots the meshlet fills (warp-uniform)
            float y[kMaxLocal / 32];
#pragma unroll
            for (uint32_t k = 0; k < kMaxLocal / 32u; k++) {
                const uint32_t v = lane + 32u * k;
                y[k] = (k < ns && v < nv) ? __ldcg(lut + min(static_cast<uint32_t>(pj[v]), qmax)) : 0.f;
            }
#pragma unroll
            for (uint32_t k = 0; k < kMaxLocal / 32u; k++) {
                const uint32_t v = lane + 32u * k;
                if (k < ns && v < nv) dst[3u * v] = y[k];
            }
        } else {
            for (uint32_t v = lane; v < nv; v += 32u) {
                const uint32_t q = static_cast<uint32_t>(pj[v]);
                float y;
                const bool fast = stride_dequant_fast(&c, q, &y) != 0;
                if (!fast || zero_bits) y = dequant_slow(Pj, d, q);
                dst[3u * v] = y;
            }
        }
        if (a.codes) {
            int32_t* cdst = a.codes + 3ull * vb + d;
            for (uint32_t v = lane; v < nv; v += 32u) cdst[3u * v] = static_cast<int32_t>(pj[v]);
        }
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// FIFO: byte i of (f0, f1, f2, f3) is depth i, depth 0 the newest entry;
// `len` entries are valid.  Deque index fi (0 = oldest) is depth len-1-fi.
// ---------------------------------------------------------------------------
struct MtfFifo {
    uint32_t f0 = 0, f1 = 0, f2 = 0, f3 = 0, len = 0;

    __device__ __forceinline__ uint32_t at(uint32_t s) const {
        const bool h = (s & 8u) != 0u;
        return __byte_perm(h ? f2 : f0, h ? f3 : f1, s & 7u) & 0xFFu;
    }
    // Remove depth p, move depths 0 .. p-1 one deeper and put v (< 256) at
    // depth 0, given the masks of depths <= p (mtf_mask_row(p)): word w
    // takes its shifted value at those depths.
    __device__ __forceinline__ void mtf_masked(uint32_t v, uint4 m) {
        const uint32_t s0 = __byte_perm(f0, v, 0x2104u);
        const uint32_t s1 = __funnelshift_l(f0, f1, 8u);
        const uint32_t s2 = __funnelshift_l(f1, f2, 8u);
        const uint32_t s3 = __funnelshift_l(f2, f3, 8u);
        f0 = (s0 & m.x) | (f0 & ~m.x);
        f1 = (s1 & m.y) | (f1 & ~m.y);
        f2 = (s2 & m.z) | (f2 & ~m.z);
        f3 = (s3 & m.w) | (f3 & ~m.w);
    }
    // exact zero-byte flags of f ^ vv at the bytes marked 0x80 in m
    __device__ __forceinline__ static uint32_t match(uint32_t f, uint32_t vv, uint32_t m) {
        const uint32_t x = f ^ vv;
        const uint32_t t = (x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu;
        return ~(t | x) & m;
    }
    // v among the 16 bytes (valid entries or filler): an exact test, no depth
    __device__ __forceinline__ bool holds(uint32_t v) const {
        const uint32_t vv = __byte_perm(v, 0u, 0u);
        const uint32_t k = 0x01010101u, h = 0x80808080u;
        const uint32_t x0 = f0 ^ vv, x1 = f1 ^ vv, x2 = f2 ^ vv, x3 = f3 ^ vv;
        // a zero byte of x sets its top bit in (x - k) & ~x (borrows never
        // reach past the first zero byte)
        return ((((x0 - k) & ~x0) | ((x1 - k) & ~x1) | ((x2 - k) & ~x2) | ((x3 - k) & ~x3)) & h) != 0u;
    }
    // depth of v among the valid entries, or 16
    __device__ __forceinline__ uint32_t find(uint32_t v) const {
        const uint32_t vv = __byte_perm(v, 0u, 0u);
        const int32_t b = static_cast<int32_t>(8u * len);
        const uint32_t k = 0x80808080u;
        const uint32_t t0 = match(f0, vv, __funnelshift_lc(0xFFFFFFFFu, 0u, static_cast<uint32_t>(b)) & k);
        const uint32_t t1 = match(f1, vv, __funnelshift_lc(0xFFFFFFFFu, 0u, static_cast<uint32_t>(max(b - 32, 0))) & k);
        const uint32_t t2 = match(f2, vv, __funnelshift_lc(0xFFFFFFFFu, 0u, static_cast<uint32_t>(max(b - 64, 0))) & k);
        const uint32_t t3 = match(f3, vv, __funnelshift_lc(0xFFFFFFFFu, 0u, static_cast<uint32_t>(max(b - 96, 0))) & k);
        const uint32_t t = t0 | t1 | t2 | t3;  // the entries are distinct: at most one byte is set
        const uint32_t j = ((t >> 7) * 0x00010203u) >> 24;
        const uint32_t i = ((t1 | t3) != 0u ? 1u : 0u) | ((t2 | t3) != 0u ? 2u : 0u);
        return t ? 4u * i + j : 16u;
    }
};

// Masks of the FIFO's move-to-front (depths 0..p of the 16-byte register, as
// four words), one 16-byte row per p in shared memory: the row is loaded
// off the FIFO's dependency chain, where computing it would cost nine
// instructions per token.
__device__ __forceinline__ uint4 mtf_mask_row(uint32_t p) {
    const int32_t b = static_cast<int32_t>(8u * p + 8u);
    uint4 m;
    m.x = __funnelshift_lc(0xFFFFFFFFu, 0u, static_cast<uint32_t>(b));
    m.y = __funnelshift_lc(0xFFFFFFFFu, 0u, static_cast<uint32_t>(max(b - 32, 0)));
    m.z = __funnelshift_lc(0xFFFFFFFFu, 0u, static_cast<uint32_t>(max(b - 64, 0)));
    m.w = __funnelshift_lc(0xFFFFFFFFu, 0u, static_cast<uint32_t>(max(b - 96, 0)));
    return m;
}

}  // namespace
}  // namespace stride
