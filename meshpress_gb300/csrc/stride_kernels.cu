// STRIDE (DPR4 v3) decode kernels for sm_103a.
//
// Two launches per decode:
//
//  1. parse_kernel -- one thread per meshlet.  Reads the meshlet's offset
//     table entry and 48-bit header, walks its strip connectivity (token
//     widths only; first-occurrence counting gives n_delta / n_para), skips
//     the six residual substreams to find their start bits (the side table
//     that the reference GPU bench reads from encoder metadata instead,
//     bench_cpp/stride_dup_decode_bench.cu:21-43), validates everything
//     against the offset table, and runs a device-wide exclusive scan of
//     n_local / n_tris: a block scan plus a last-block scan of block sums.
//
//  2. decode_kernel -- a warp decodes 32 consecutive meshlets.  One bulk
//     copy (cp.async.bulk + mbarrier) stages the group's payload bytes in
//     shared memory.  Each lane then replays one meshlet: strip walk with the
//     16-entry move-to-tail FIFO held in four registers, first-occurrence
//     walk, IRLP prediction in int32 and residual decode from the staged
//     bits (the serial work of decode_dup, encoder/paradelta_v5_dup.py:
//     507-600, spread over 32 meshlets instead of one lane of a warp).
//     Triangles go through a per-lane ring in shared memory and integer codes
//     through per-lane shared storage; both are written out warp-cooperatively
//     with 128-bit stores, positions after exact dequantisation
//     (stride_dequant.h).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "stride_common.cuh"
#include "stride_gb300.h"

namespace stride {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// Bit access: MSB-first stream read as big-endian 32-bit words.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0u, 0x0123u); }

template <bool kShared>
__device__ __forceinline__ uint32_t ldw(const uint32_t* w, uint32_t i) {
    if constexpr (kShared) {
        return w[i];
    } else {
        return __ldg(w + i);
    }
}

// 32 bits starting at bit `rel` of the word array.
template <bool kShared>
__device__ __forceinline__ uint32_t peek32(const uint32_t* w, uint32_t rel) {
    const uint32_t i = rel >> 5;
    const uint32_t hi = bswap32(ldw<kShared>(w, i));
    const uint32_t lo = bswap32(ldw<kShared>(w, i + 1));
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

// ---------------------------------------------------------------------------
// Parse kernel
// ---------------------------------------------------------------------------
__device__ int parse_meshlet(const uint8_t* __restrict__ arena, const MeshParams& P, uint32_t lm,
                             MeshletDesc& d, uint32_t* seen /* stride kScanThreads */) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(arena + P.blob_off);
    const uint32_t nbits = static_cast<uint32_t>(P.nbits);
    const uint32_t tbit = kHeaderBytes * 8u;
    const uint32_t off = peek32<false>(w, tbit + 32u * lm);
    const uint32_t next = (lm + 1u < P.n_meshlets) ? peek32<false>(w, tbit + 32u * (lm + 1u)) : nbits;
    if ((lm == 0u && off != P.body_bit) || off < P.body_bit || next > nbits || next < off + 48u ||
        off + 48u < off)
        return kErrOffset;
    uint32_t pos = off;
    const uint32_t h0 = peek32<false>(w, pos);
    const uint32_t n_local = h0 >> 16;
    const uint32_t n_tris = h0 & 0xFFFFu;
    const uint32_t n_strips = peek32<false>(w, pos + 32u) >> 16;
    pos += 48u;
    if (n_local > static_cast<uint32_t>(kMaxLocal) || n_tris > static_cast<uint32_t>(kMaxTris))
        return kErrUnsupported;
    if (n_strips > n_tris) return kErrCorrupt;  // every strip emits >= 1 triangle
    const uint32_t ib = max(1u, 32u - __clz(n_local));
#pragma unroll
    for (int i = 0; i < 8; i++) seen[i * kScanThreads] = 0u;
    uint32_t nseen = 0u, k0 = 0u, k1 = 0u, tris = 0u;
    for (uint32_t s = 0; s < n_strips; s++) {
        if (pos + 16u > next) return kErrCorrupt;
        const uint32_t len = peek32<false>(w, pos) >> 16;
        pos += 16u;
        const uint32_t body = len > 1u ? len - 1u : 0u;
        tris += 1u + body;
        if (tris > n_tris) return kErrCorrupt;
        const uint32_t ntok = 3u + body;
        for (uint32_t j = 0; j < ntok; j++) {
            uint32_t x = peek32<false>(w, pos);
            if (j >= 3u) {
                x <<= 1;
                pos += 1u;
            }
            if (x >> 31) {
                const uint32_t v = (x << 1) >> (32u - ib);
                pos += 1u + ib;
                if (v >= n_local) return kErrCorrupt;
                uint32_t& sw = seen[(v >> 5) * kScanThreads];
                const uint32_t bit = 1u << (v & 31u);
                if (!(sw & bit)) {
                    sw |= bit;
                    nseen++;
                    if (j < 3u) k0++; else k1++;
                }
            } else {
                const uint32_t fi = (x << 1) >> 27;
                pos += 6u;
                if (fi >= min(nseen, static_cast<uint32_t>(kFifo))) return kErrCorrupt;
            }
            if (pos > next) return kErrCorrupt;
        }
    }
    if (tris != n_tris) return kErrCorrupt;
    d.anchor_bit = pos;
    pos += P.anchor_bits;
    uint32_t tk[6];
#pragma unroll
    for (int i = 0; i < 6; i++) {
        const uint32_t t = peek32<false>(w, pos) >> 16;
        pos += 16u;
        const uint32_t k = t & 0xFFu;
        if (k > static_cast<uint32_t>(kMaxResidK)) return kErrUnsupported;
        tk[i] = ((t >> 8) == 1u ? 0u : 0x80u) | k;
    }
    if (pos > next) return kErrCorrupt;
    const uint32_t n_delta = k0 ? k0 - 1u : 0u;
    const uint32_t n_para = k1;
#pragma unroll 1
    for (int s = 0; s < 6; s++) {
        d.res_bit[s] = pos;
        const uint32_t n = s < 3 ? n_delta : n_para;
        for (uint32_t i = 0; i < n; i++) {
            uint32_t u;
            const int e = read_code<false>(w, 0u, pos, tk[s], next, u);
            if (e) return e;
        }
    }
    if ((lm + 1u < P.n_meshlets) ? (pos != next) : (pos > next)) return kErrCorrupt;
    d.conn_bit = off + 48u;
    d.counts0 = n_local | (n_tris << 16);
    d.counts1 = n_strips | (n_delta << 16);
    d.counts2 = n_para;
    d.tk_delta = tk[0] | (tk[1] << 8) | (tk[2] << 16);
    d.tk_para = tk[3] | (tk[4] << 8) | (tk[5] << 16);
    d.end_bit = pos;
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

__global__ void __launch_bounds__(kScanThreads) parse_kernel(DecodeArgs a) {
    __shared__ uint32_t seen[8 * kScanThreads];
    __shared__ unsigned long long wsum[kScanThreads / 32];
    __shared__ int is_last;
    const uint32_t tid = threadIdx.x;
    const uint32_t m = blockIdx.x * kScanThreads + tid;
    uint32_t nl = 0u, nt = 0u;
    MeshletDesc d;
    bool ok = false;
    if (m < a.total_meshlets) {
        const uint32_t mi = a.meshlet_mesh ? __ldg(a.meshlet_mesh + m) : 0u;
        const MeshParams& P = a.meshes[mi];
        const int e = parse_meshlet(a.arena, P, m - P.meshlet_begin, d, seen + tid);
        if (e) {
            report(a.status, e, m);
        } else {
            ok = true;
            nl = d.counts0 & 0xFFFFu;
            nt = d.counts0 >> 16;
        }
    }
    const unsigned long long x = (static_cast<unsigned long long>(nt) << 32) | nl;
    unsigned long long total;
    const unsigned long long ex = block_scan(x, wsum, total);
    if (ok) {
        d.v_pref = static_cast<uint32_t>(ex);
        d.t_pref = static_cast<uint32_t>(ex >> 32);
        uint4* dst = reinterpret_cast<uint4*>(a.descs + m);
        const uint4* src = reinterpret_cast<const uint4*>(&d);
        dst[0] = src[0];
        dst[1] = src[1];
        dst[2] = src[2];
        dst[3] = src[3];
    }
    if (tid == 0) a.blk_sums[blockIdx.x] = make_uint2(static_cast<uint32_t>(total), static_cast<uint32_t>(total >> 32));
    // The last block to finish turns the block sums into block prefixes.
    __threadfence();
    __syncthreads();
    if (tid == 0) is_last = atomicAdd(&a.status->ticket, 1u) == gridDim.x - 1u;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    unsigned long long cv = 0ull, ct = 0ull;
    for (uint32_t base = 0; base < gridDim.x; base += kScanThreads) {
        const uint32_t i = base + tid;
        const uint2 s = i < gridDim.x ? __ldcg(a.blk_sums + i) : make_uint2(0u, 0u);
        unsigned long long tv, tt;
        const unsigned long long ev = block_scan(s.x, wsum, tv);
        const unsigned long long et = block_scan(s.y, wsum, tt);
        if (i < gridDim.x) a.blk_prefix[i] = make_ulonglong2(cv + ev, ct + et);
        cv += tv;
        ct += tt;
    }
}

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

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    unsigned long long gsrc;
    asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(gsrc) : "l"(src));
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
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

// Bounded wait (about a second of SM clocks); false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, phase)) {
        if (clock64() - t0 > (1ll << 31)) return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Warp-cooperative output: n consecutive 32-bit words at dst, 16-byte
// vector stores for the aligned body.
// ---------------------------------------------------------------------------
template <class F>
__device__ __forceinline__ void warp_store_words(uint32_t* dst, uint32_t n, F f, int lane) {
    uint32_t head = static_cast<uint32_t>((16u - (reinterpret_cast<uintptr_t>(dst) & 15u)) & 15u) >> 2;
    if (head > n) head = n;
    if (static_cast<uint32_t>(lane) < head) dst[lane] = f(static_cast<uint32_t>(lane));
    const uint32_t rem = n - head;
    const uint32_t nvec = rem >> 2;
    uint4* v = reinterpret_cast<uint4*>(dst + head);
    for (uint32_t i = lane; i < nvec; i += 32u) {
        const uint32_t b = head + 4u * i;
        v[i] = make_uint4(f(b), f(b + 1u), f(b + 2u), f(b + 3u));
    }
    const uint32_t t0 = head + 4u * nvec;
    if (static_cast<uint32_t>(lane) < n - t0) dst[t0 + lane] = f(t0 + lane);
}

__device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int src) {
    return __shfl_sync(kFull, v, src);
}

// ---------------------------------------------------------------------------
// Integer code storage: 8 bytes per vertex (16-bit codes) or 16 (wider).
// ---------------------------------------------------------------------------
template <bool kWide>
struct Codes {
    static constexpr uint32_t kBytes = kWide ? 16u : 8u;
    __device__ static __forceinline__ void store(uint8_t* base, uint32_t v, int32_t x, int32_t y, int32_t z) {
        if constexpr (kWide) {
            reinterpret_cast<int4*>(base)[v] = make_int4(x, y, z, 0);
        } else {
            reinterpret_cast<uint2*>(base)[v] =
                make_uint2(static_cast<uint32_t>(x) | (static_cast<uint32_t>(y) << 16), static_cast<uint32_t>(z));
        }
    }
    __device__ static __forceinline__ void load(const uint8_t* base, uint32_t v, int32_t& x, int32_t& y,
                                                int32_t& z) {
        if constexpr (kWide) {
            const int4 c = reinterpret_cast<const int4*>(base)[v];
            x = c.x;
            y = c.y;
            z = c.z;
        } else {
            const uint2 c = reinterpret_cast<const uint2*>(base)[v];
            x = static_cast<int32_t>(c.x & 0xFFFFu);
            y = static_cast<int32_t>(c.x >> 16);
            z = static_cast<int32_t>(c.y);
        }
    }
    __device__ static __forceinline__ uint32_t component(const uint8_t* base, uint32_t v, uint32_t k) {
        if constexpr (kWide) {
            return reinterpret_cast<const uint32_t*>(base)[4u * v + k];
        } else {
            const uint32_t* p = reinterpret_cast<const uint32_t*>(base) + 2u * v;
            return k == 2u ? p[1] : ((p[0] >> (16u * k)) & 0xFFFFu);
        }
    }
};

// ---------------------------------------------------------------------------
// 16-entry move-to-tail FIFO (_read_vert, encoder/paradelta_codec.py:330-340)
// in four registers: byte 15 is the newest entry, the valid entries are bytes
// [16 - len, 16), so the deque index fi (0 = oldest) is byte 16 - len + fi.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t low_bytes_mask(uint32_t p, uint32_t word) {
    // bytes [0, p) of the 16-byte value, restricted to 32-bit word `word`
    const int sh = min(max(static_cast<int>(p) - static_cast<int>(4u * word), 0), 4) * 8;
    return static_cast<uint32_t>((1ull << sh) - 1ull);
}

struct Fifo {
    uint32_t f0 = 0, f1 = 0, f2 = 0, f3 = 0, len = 0;
    __device__ __forceinline__ uint32_t at(uint32_t p) const {
        const uint32_t w = (p & 8u) ? ((p & 4u) ? f3 : f2) : ((p & 4u) ? f1 : f0);
        return (w >> ((p & 3u) * 8u)) & 0xFFu;
    }
    // byte position of v among the valid entries, or 16
    __device__ __forceinline__ uint32_t find(uint32_t v) const {
        const uint32_t vv = v * 0x01010101u;
        const uint32_t lo = 16u - len;
        const uint32_t e0 = __vcmpeq4(f0, vv) & ~low_bytes_mask(lo, 0);
        const uint32_t e1 = __vcmpeq4(f1, vv) & ~low_bytes_mask(lo, 1);
        const uint32_t e2 = __vcmpeq4(f2, vv) & ~low_bytes_mask(lo, 2);
        const uint32_t e3 = __vcmpeq4(f3, vv) & ~low_bytes_mask(lo, 3);
        if (e0) return (__ffs(e0) - 1) >> 3;
        if (e1) return 4u + ((__ffs(e1) - 1) >> 3);
        if (e2) return 8u + ((__ffs(e2) - 1) >> 3);
        if (e3) return 12u + ((__ffs(e3) - 1) >> 3);
        return 16u;
    }
    // remove the byte at p, shift the newer bytes down, append v as newest
    __device__ __forceinline__ void remove_append(uint32_t p, uint32_t v) {
        const uint32_t s0 = __funnelshift_r(f0, f1, 8);
        const uint32_t s1 = __funnelshift_r(f1, f2, 8);
        const uint32_t s2 = __funnelshift_r(f2, f3, 8);
        const uint32_t s3 = (f3 >> 8) | (v << 24);
        const uint32_t k0 = low_bytes_mask(p, 0), k1 = low_bytes_mask(p, 1);
        const uint32_t k2 = low_bytes_mask(p, 2), k3 = low_bytes_mask(p, 3);
        f0 = (f0 & k0) | (s0 & ~k0);
        f1 = (f1 & k1) | (s1 & ~k1);
        f2 = (f2 & k2) | (s2 & ~k2);
        f3 = (f3 & k3) | (s3 & ~k3);
    }
};

struct WarpSmem {
    uint32_t* stage;
    uint8_t* codes;
    uint32_t* ring;
    uint32_t* seen;
    float* dqc;  // 3 axes x 8 floats: a_hi a_lo b_hi b_lo err konst zero_bits pad
    uint64_t* bar;
};

__device__ __forceinline__ float dequant_value(const float* c, const MeshParams* P, uint32_t axis, uint32_t q) {
    if (__float_as_uint(c[6])) return c[5];
    stride_dequant_axis t;
    t.a_hi = c[0];
    t.a_lo = c[1];
    t.b_hi = c[2];
    t.b_lo = c[3];
    t.err = c[4];
    float y;
    if (stride_dequant_fast(&t, q, &y)) return y;
    return stride_dequant_exact(&P->dq[axis], q);
}

__device__ __forceinline__ void flush_tris(const WarpSmem& S, uint32_t& rcnt, unsigned long long& t_next,
                                           uint32_t vloc, uint32_t* __restrict__ idx_out, int lane) {
    __syncwarp();
    for (int j = 0; j < 32; j++) {
        const uint32_t c = __shfl_sync(kFull, rcnt, j);
        if (c == 0u) continue;
        const unsigned long long tb = shfl64(t_next, j);
        const uint32_t vb = __shfl_sync(kFull, vloc, j);
        const uint32_t* rj = S.ring + j * kRingStride;
        warp_store_words(
            idx_out + 3ull * tb, 3u * c,
            [&](uint32_t i) {
                const uint32_t t = i / 3u;
                const uint32_t k = i - 3u * t;
                return vb + ((rj[t] >> (8u * k)) & 0xFFu);
            },
            lane);
    }
    t_next += rcnt;
    rcnt = 0u;
    __syncwarp();
}

template <bool kShared>
__device__ __forceinline__ int read_axis(const uint32_t* w, uint32_t rbase, bool para, uint32_t& cd, uint32_t& cp,
                                         uint32_t tkd, uint32_t tkp, uint32_t limit, int32_t& r) {
    uint32_t p = para ? cp : cd;
    uint32_t u = 0u;
    const int e = read_code<kShared>(w, rbase, p, para ? tkp : tkd, limit, u);
    if (para) cp = p; else cd = p;
    r = unzigzag(u);
    return e;
}

// Decode the meshlets of the lanes in `act` (one per lane) from the word
// array `w` (staged shared memory or the global stream).
template <bool kShared, bool kWide>
__device__ void decode_lanes(const DecodeArgs& a, const WarpSmem& S, const MeshletDesc& d, const MeshParams* P,
                             uint32_t mi, bool act, uint32_t m, uint32_t round_mask, uint32_t round_code_bytes,
                             uint32_t code_off, const uint32_t* w, uint32_t rbase,
                             unsigned long long v_base, unsigned long long t_base, int lane) {
    using C = Codes<kWide>;
    // clear first-occurrence bits and the integer codes of this round
#pragma unroll
    for (int i = 0; i < 8; i++) S.seen[i * 32 + lane] = 0u;
    for (uint32_t i = lane; i < round_code_bytes / 8u; i += 32u) reinterpret_cast<uint2*>(S.codes)[i] = make_uint2(0u, 0u);
    __syncwarp();

    uint8_t* my_codes = S.codes + code_off;
    const uint32_t n_local = d.counts0 & 0xFFFFu;
    const uint32_t n_strips = d.counts1 & 0xFFFFu;
    const uint32_t ib = max(1u, 32u - __clz(n_local));
    const uint32_t limit = d.end_bit;
    int32_t pn0 = 0, pn1 = 0, pn2 = 0, pn3 = 0, pn4 = 0, pn5 = 0, pn6 = 0, pn7 = 0, pn8 = 0;
    int32_t pk0 = 0, pk1 = 0, pk2 = 0, ph0 = 0, ph1 = 0, ph2 = 0;
    uint32_t cm0 = 0, cm1 = 0, cm2 = 0, gb0 = 0, gb1 = 0, gb2 = 0;
    unsigned long long v_off = 0ull;
    if (act) {
        pn0 = P->pred_n[0]; pn1 = P->pred_n[1]; pn2 = P->pred_n[2];
        pn3 = P->pred_n[3]; pn4 = P->pred_n[4]; pn5 = P->pred_n[5];
        pn6 = P->pred_n[6]; pn7 = P->pred_n[7]; pn8 = P->pred_n[8];
        pk0 = P->pred_k[0]; pk1 = P->pred_k[1]; pk2 = P->pred_k[2];
        ph0 = P->pred_half[0]; ph1 = P->pred_half[1]; ph2 = P->pred_half[2];
        cm0 = P->code_max[0]; cm1 = P->code_max[1]; cm2 = P->code_max[2];
        gb0 = P->g_bits[0]; gb1 = P->g_bits[1]; gb2 = P->g_bits[2];
        v_off = P->v_offset;
    }
    const uint32_t tkd = d.tk_delta, tkp = d.tk_para;
    uint32_t c0 = d.res_bit[0], c1 = d.res_bit[1], c2 = d.res_bit[2];
    uint32_t c3 = d.res_bit[3], c4 = d.res_bit[4], c5 = d.res_bit[5];
    // anchor: raw codes of g_bits each (paradelta_v5_dup.py:545-546)
    int32_t ax = 0, ay = 0, az = 0;
    if (act) {
        uint32_t p = d.anchor_bit;
        if (gb0) { ax = static_cast<int32_t>(peek32<kShared>(w, p + rbase) >> (32u - gb0)); p += gb0; }
        if (gb1) { ay = static_cast<int32_t>(peek32<kShared>(w, p + rbase) >> (32u - gb1)); p += gb1; }
        if (gb2) { az = static_cast<int32_t>(peek32<kShared>(w, p + rbase) >> (32u - gb2)); }
    }

    uint32_t cpos = d.conn_bit;
    uint32_t strips_left = n_strips;
    uint32_t tok_left = 0u, tok_idx = 0u;
    uint32_t p0 = 0u, p1 = 0u, p2 = 0u;
    Fifo fifo;
    bool have_anchor = false;
    int32_t prx = 0, pry = 0, prz = 0;
    uint32_t rcnt = 0u;
    unsigned long long t_next = t_base;
    const uint32_t vloc = static_cast<uint32_t>(v_base - v_off);
    bool running = act && n_strips > 0u;
    bool bad = false;
    uint32_t* my_ring = S.ring + lane * kRingStride;

    while (__any_sync(kFull, running)) {
        if (running) {
            if (tok_left == 0u) {  // strip header (paradelta_v5_dup.py:519)
                const uint32_t len = peek32<kShared>(w, cpos + rbase) >> 16;
                cpos += 16u;
                tok_left = 3u + (len > 1u ? len - 1u : 0u);
                tok_idx = 0u;
                strips_left--;
            }
            uint32_t x = peek32<kShared>(w, cpos + rbase);
            const bool body = tok_idx >= 3u;
            const uint32_t ec = body ? (x >> 31) : 0u;
            if (body) {
                x <<= 1;
                cpos += 1u;
            }
            const bool raw = (x >> 31) != 0u;
            const uint32_t rid = min((x << 1) >> (32u - ib), 255u);
            const uint32_t fi = (x << 1) >> 27;
            cpos += raw ? 1u + ib : 6u;
            const uint32_t v = raw ? rid : fifo.at((16u - fifo.len + fi) & 15u);
            const uint32_t at = fifo.find(v);
            const uint32_t rm = at < 16u ? at : (fifo.len == 16u ? 0u : 15u - fifo.len);
            fifo.remove_append(rm, v);
            fifo.len = min(fifo.len + (at == 16u ? 1u : 0u), 16u);
            uint32_t c_ref = 0u;
            if (body) {  // edge code: 0 -> (p1, p2, p0), 1 -> (p0, p2, p1)  (:530-535)
                const uint32_t na = ec ? p0 : p1;
                c_ref = ec ? p1 : p0;
                p0 = na;
                p1 = p2;
                p2 = v;
            } else {
                p0 = tok_idx == 0u ? v : p0;
                p1 = tok_idx == 1u ? v : p1;
                p2 = tok_idx == 2u ? v : p2;
            }
            if (body || tok_idx == 2u) {
                my_ring[rcnt] = p0 | (p1 << 8) | (p2 << 16);
                rcnt++;
            }
            tok_idx++;
            tok_left--;
            if (tok_left == 0u && strips_left == 0u) running = false;
            // first occurrence -> next vertex of the walk (:523-541, :581-600)
            uint32_t& sw = S.seen[(v >> 5) * 32u + lane];
            const uint32_t bit = 1u << (v & 31u);
            if (!(sw & bit)) {
                sw |= bit;
                int32_t cx, cy, cz;
                if (!body && !have_anchor) {
                    cx = ax;
                    cy = ay;
                    cz = az;
                    have_anchor = true;
                } else {
                    int32_t qx = prx, qy = pry, qz = prz;
                    if (body) {  // IRLP (:91-104) over (a, b, c) = (p0, p1, c_ref)
                        int32_t axx, ayy, azz, bx, by, bz, cxx, cyy, czz;
                        C::load(my_codes, p0, axx, ayy, azz);
                        C::load(my_codes, p1, bx, by, bz);
                        C::load(my_codes, c_ref, cxx, cyy, czz);
                        qx = (pn0 * axx + pn1 * bx + pn2 * cxx + ph0) >> pk0;
                        qy = (pn3 * ayy + pn4 * by + pn5 * cyy + ph1) >> pk1;
                        qz = (pn6 * azz + pn7 * bz + pn8 * czz + ph2) >> pk2;
                    }
                    int32_t rx, ry, rz;
                    int e = read_axis<kShared>(w, rbase, body, c0, c3, tkd & 0xFFu, tkp & 0xFFu, limit, rx);
                    e |= read_axis<kShared>(w, rbase, body, c1, c4, (tkd >> 8) & 0xFFu, (tkp >> 8) & 0xFFu, limit, ry);
                    e |= read_axis<kShared>(w, rbase, body, c2, c5, (tkd >> 16) & 0xFFu, (tkp >> 16) & 0xFFu, limit, rz);
                    const long long lx = static_cast<long long>(qx) + rx;
                    const long long ly = static_cast<long long>(qy) + ry;
                    const long long lz = static_cast<long long>(qz) + rz;
                    if (e || lx < 0 || ly < 0 || lz < 0 || lx > cm0 || ly > cm1 || lz > cm2) bad = true;
                    cx = static_cast<int32_t>(lx < 0 ? 0 : (lx > cm0 ? cm0 : lx));
                    cy = static_cast<int32_t>(ly < 0 ? 0 : (ly > cm1 ? cm1 : ly));
                    cz = static_cast<int32_t>(lz < 0 ? 0 : (lz > cm2 ? cm2 : lz));
                }
                C::store(my_codes, v, cx, cy, cz);
                prx = cx;
                pry = cy;
                prz = cz;
            }
        }
        if (__any_sync(kFull, rcnt == static_cast<uint32_t>(kRing))) flush_tris(S, rcnt, t_next, vloc, a.idx, lane);
    }
    flush_tris(S, rcnt, t_next, vloc, a.idx, lane);
    if (bad) report(a.status, kErrCorrupt, m);

    // positions (and optionally codes), one meshlet at a time, whole warp
    uint32_t cached = 0xFFFFFFFFu;
    for (int j = 0; j < 32; j++) {
        if (!((round_mask >> j) & 1u)) continue;
        const uint32_t n = __shfl_sync(kFull, n_local, j);
        const unsigned long long vb = shfl64(v_base, j);
        const uint32_t off = __shfl_sync(kFull, code_off, j);
        const uint32_t mj = __shfl_sync(kFull, mi, j);
        const MeshParams* Pj = a.meshes + mj;
        if (mj != cached) {
            __syncwarp();
            if (lane < 24) {
                const uint32_t ax_ = lane >> 3, f = lane & 7u;
                const stride_dequant_axis& q = Pj->dq[ax_];
                float val;
                switch (f) {
                    case 0: val = q.a_hi; break;
                    case 1: val = q.a_lo; break;
                    case 2: val = q.b_hi; break;
                    case 3: val = q.b_lo; break;
                    case 4: val = q.err; break;
                    case 5: val = q.konst; break;
                    case 6: val = __uint_as_float(static_cast<uint32_t>(q.zero_bits)); break;
                    default: val = 0.f; break;
                }
                S.dqc[lane] = val;
            }
            __syncwarp();
            cached = mj;
        }
        const uint8_t* cj = S.codes + off;
        warp_store_words(
            reinterpret_cast<uint32_t*>(a.pos + 3ull * vb), 3u * n,
            [&](uint32_t i) {
                const uint32_t vv = i / 3u;
                const uint32_t k = i - 3u * vv;
                return __float_as_uint(dequant_value(S.dqc + 8u * k, Pj, k, C::component(cj, vv, k)));
            },
            lane);
        if (a.codes) {
            warp_store_words(
                reinterpret_cast<uint32_t*>(a.codes + 3ull * vb), 3u * n,
                [&](uint32_t i) {
                    const uint32_t vv = i / 3u;
                    return C::component(cj, vv, i - 3u * vv);
                },
                lane);
        }
    }
    __syncwarp();
}

__host__ __device__ constexpr uint32_t align16(uint32_t x) { return (x + 15u) & ~15u; }

__host__ __device__ inline uint32_t warp_smem_bytes(uint32_t stage_bytes, uint32_t code_bytes) {
    return align16(stage_bytes + 32u) + align16(code_bytes) + align16(kRingStride * 32u * 4u) + 8u * 32u * 4u +
           3u * 8u * 4u + 16u;
}

template <bool kWide>
__device__ bool process_group(const DecodeArgs& a, const WarpSmem& S, uint32_t g, uint32_t stage_bytes,
                              uint32_t code_bytes, uint32_t& phase, int lane) {
    using C = Codes<kWide>;
    const uint32_t m = g * 32u + lane;
    const bool valid = m < a.total_meshlets;
    MeshletDesc d;
    if (valid) {
        const uint4* src = reinterpret_cast<const uint4*>(a.descs + m);
        uint4* dst = reinterpret_cast<uint4*>(&d);
        dst[0] = __ldg(src);
        dst[1] = __ldg(src + 1);
        dst[2] = __ldg(src + 2);
        dst[3] = __ldg(src + 3);
    } else {
        memset(&d, 0, sizeof(d));
    }
    const uint32_t mi = (valid && a.meshlet_mesh) ? __ldg(a.meshlet_mesh + m) : 0u;
    const MeshParams* P = a.meshes + mi;
    const uint32_t n_local = d.counts0 & 0xFFFFu;
    const uint32_t n_tris = d.counts0 >> 16;
    unsigned long long v_base = 0ull, t_base = 0ull;
    bool ok = false;
    unsigned long long blob_off = 0ull;
    if (valid) {
        const ulonglong2 bp = a.blk_prefix[m / kScanThreads];
        v_base = bp.x + d.v_pref;
        t_base = bp.y + d.t_pref;
        const unsigned long long vo = P->v_offset, to = P->t_offset, nv = P->n_v, nt = P->n_t;
        ok = v_base >= vo && v_base + n_local <= vo + nv && t_base >= to && t_base + n_tris <= to + nt;
        if (ok && m - P->meshlet_begin + 1u == P->n_meshlets)
            ok = v_base + n_local == vo + nv && t_base + n_tris == to + nt;
        if (!ok) report(a.status, kErrCorrupt, m);
        blob_off = P->blob_off;
    }
    const unsigned long long start_b = blob_off + ((d.conn_bit - 48u) >> 3);
    const unsigned long long end16 = (blob_off + ((d.end_bit + 7u) >> 3) + 15ull) & ~15ull;
    const uint32_t csz = n_local * C::kBytes;
    uint32_t todo = __ballot_sync(kFull, ok);
    while (todo) {
        const int first = __ffs(todo) - 1;
        const bool in = (todo >> lane) & 1u;
        uint32_t cum = in ? csz : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, cum, o);
            if (lane >= o) cum += t;
        }
        const unsigned long long s0 = shfl64(start_b, first) & ~15ull;
        const bool fit = in && cum <= code_bytes && (end16 - s0) <= stage_bytes;
        uint32_t rmask = __ballot_sync(kFull, fit);
        const bool staged = rmask != 0u;
        if (!staged) rmask = 1u << first;  // a meshlet larger than the stage: read it from global memory
        todo &= ~rmask;
        const bool act = (rmask >> lane) & 1u;
        const uint32_t last = 31 - __clz(rmask);
        const uint32_t round_bytes = __shfl_sync(kFull, cum, last);
        const uint32_t code_off = act ? cum - csz : 0u;
        if (staged) {
            const unsigned long long e_last = shfl64(end16, last);
            const uint32_t bytes = static_cast<uint32_t>(e_last - s0);
            __syncwarp();
            if (lane == 0) bulk_load(S.stage, a.arena + s0, bytes, S.bar);
            if (!mbar_wait(S.bar, phase)) {
                if (lane == 0) report(a.status, kErrTimeout, m);
                mbar_wait(S.bar, phase);  // give the copy in flight one more bounded wait
                return false;
            }
            phase ^= 1u;
            const uint32_t rbase = static_cast<uint32_t>(blob_off * 8ull - s0 * 8ull);
            decode_lanes<true, kWide>(a, S, d, P, mi, act, m, rmask, round_bytes, code_off, S.stage, rbase, v_base,
                                      t_base, lane);
        } else {
            const uint32_t* gw = reinterpret_cast<const uint32_t*>(a.arena + blob_off);
            decode_lanes<false, kWide>(a, S, d, P, mi, act, m, rmask, round_bytes, code_off, gw, 0u, v_base,
                                       t_base, lane);
        }
    }
    return true;
}

template <int W, bool kWide>
__global__ void __launch_bounds__(W * 32) decode_kernel(DecodeArgs a, uint32_t stage_bytes, uint32_t code_bytes,
                                                        int persistent) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    if (*reinterpret_cast<volatile unsigned long long*>(&a.status->err) != 0ull) return;
    const uint32_t per_warp = warp_smem_bytes(stage_bytes, code_bytes);
    uint8_t* base = smem + warp * per_warp;
    WarpSmem S;
    S.stage = reinterpret_cast<uint32_t*>(base);
    S.codes = base + align16(stage_bytes + 32u);
    S.ring = reinterpret_cast<uint32_t*>(S.codes + align16(code_bytes));
    S.seen = S.ring + align16(kRingStride * 32u * 4u) / 4u;
    S.dqc = reinterpret_cast<float*>(S.seen + 8 * 32);
    S.bar = reinterpret_cast<uint64_t*>(S.dqc + 24);
    if (lane == 0) mbar_init(S.bar);
    __syncwarp();
    uint32_t phase = 0u;
    const uint32_t n_groups = (a.total_meshlets + 31u) / 32u;
    uint32_t g;
    if (persistent) {
        uint32_t t = 0u;
        if (lane == 0) t = atomicAdd(&a.status->work, 1u);
        g = __shfl_sync(kFull, t, 0);
    } else {
        g = blockIdx.x * W + warp;
    }
    while (g < n_groups) {
        if (!process_group<kWide>(a, S, g, stage_bytes, code_bytes, phase, lane)) return;
        if (!persistent) break;
        uint32_t t = 0u;
        if (lane == 0) t = atomicAdd(&a.status->work, 1u);
        g = __shfl_sync(kFull, t, 0);
    }
}

template <int W, bool kWide>
cudaError_t launch_decode_t(const DecodeArgs& a, const LaunchCfg& cfg, cudaStream_t s) {
    const size_t smem = static_cast<size_t>(W) * warp_smem_bytes(cfg.stage_bytes, cfg.code_bytes);
    // opt in to large dynamic shared memory once per (device, kernel)
    static size_t configured[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    dev = dev < 0 || dev >= 64 ? 0 : dev;
    if (configured[dev] < smem) {
        cudaError_t e = cudaFuncSetAttribute(decode_kernel<W, kWide>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        configured[dev] = smem;
    }
    const uint32_t n_groups = (a.total_meshlets + 31u) / 32u;
    uint32_t grid = (n_groups + W - 1) / W;
    if (cfg.persistent) {
        const int per_sm = cfg.ctas_per_sm > 0 ? cfg.ctas_per_sm : 4;
        const uint32_t cap = static_cast<uint32_t>(per_sm * device_sm_count());
        if (grid > cap) grid = cap;
    }
    if (grid == 0) return cudaSuccess;
    decode_kernel<W, kWide><<<grid, W * 32, smem, s>>>(a, cfg.stage_bytes, cfg.code_bytes, cfg.persistent);
    return cudaGetLastError();
}

template <bool kWide>
cudaError_t launch_decode_w(const DecodeArgs& a, const LaunchCfg& cfg, cudaStream_t s) {
    switch (cfg.warps_per_cta) {
        case 1: return launch_decode_t<1, kWide>(a, cfg, s);
        case 2: return launch_decode_t<2, kWide>(a, cfg, s);
        case 4: return launch_decode_t<4, kWide>(a, cfg, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

size_t decode_smem_bytes(const LaunchCfg& cfg, bool /*wide*/) {
    return static_cast<size_t>(cfg.warps_per_cta) * warp_smem_bytes(cfg.stage_bytes, cfg.code_bytes);
}

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

int check_config(const LaunchCfg& cfg, bool wide) {
    if (cfg.warps_per_cta != 1 && cfg.warps_per_cta != 2 && cfg.warps_per_cta != 4) return STRIDE_ERR_ARG;
    if (cfg.code_bytes < kMaxLocal * (wide ? 16u : 8u) || cfg.stage_bytes < 1024u) return STRIDE_ERR_ARG;
    if (decode_smem_bytes(cfg, wide) > 227u * 1024u) return STRIDE_ERR_ARG;
    return STRIDE_OK;
}

int enqueue_decode(const DecodeArgs& a, const LaunchCfg& cfg, void* stream, void* const* ev) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (check_config(cfg, a.wide_codes)) return STRIDE_ERR_ARG;
    if (cudaMemsetAsync(a.status, 0, sizeof(Status), s) != cudaSuccess) return STRIDE_ERR_CUDA;
    if (ev) cudaEventRecord(static_cast<cudaEvent_t>(ev[0]), s);
    if (a.total_meshlets != 0) {
        const uint32_t nb = parse_blocks(a.total_meshlets);
        parse_kernel<<<nb, kScanThreads, 0, s>>>(a);
        if (cudaGetLastError() != cudaSuccess) return STRIDE_ERR_CUDA;
    }
    if (ev) cudaEventRecord(static_cast<cudaEvent_t>(ev[1]), s);
    if (a.total_meshlets != 0) {
        const cudaError_t e = a.wide_codes ? launch_decode_w<true>(a, cfg, s) : launch_decode_w<false>(a, cfg, s);
        if (e != cudaSuccess) return STRIDE_ERR_CUDA;
    }
    if (ev) cudaEventRecord(static_cast<cudaEvent_t>(ev[2]), s);
    return STRIDE_OK;
}

}  // namespace stride
