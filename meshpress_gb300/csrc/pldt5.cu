// PLDT v5 decoding on the GPU: the format the reference's CuPy decoder
// ParaDeltaV5GpuDecoder reads (utils/paradelta_v5_cuda.py:515-718), decoded
// bit-exactly like its CPU decoder decode_paradelta_v5
// (encoder/paradelta_v5.py:286-462; the CuPy kernel computes in float32).
//
// Split as in the reference: the host parses the global header and the
// boundary table (parse_globals_v5, :515-577) and reads every meshlet's
// four-field header from the offset table (the reference's sizes kernel and
// cumulative sums, :640-660); the device decodes the meshlets, one thread
// each, into float64 normalised rows, and a second kernel turns the rows
// into float32 world positions.
//
// Rows: the boundary vertices, then every meshlet's interior vertices in
// meshlet order.  A meshlet's triangles go to its rows of the index output
// as global row numbers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <new>
#include <stdexcept>
#include <vector>

#include "stride_common.cuh"
#include "stride_device.cuh"
#include "stride_gb300.h"
#include "stride_internal.h"

namespace stride {
namespace {

constexpr uint32_t kP5Magic = 0x504C4454u;  // MAGIC (encoder/paradelta_codec.py:101)
constexpr uint32_t kP5Version = 5u;         // VERSION_V5 (encoder/paradelta_v5.py:27)
constexpr uint32_t kP5HeaderBits = 32 + 8 + 8 + 32 * 11 + 8 * 3 + 32 * 4 + 32 * 3;
constexpr int kP5MaxLocal = 256;  // local ids are bytes in the walk scratch
constexpr int kP5MaxK = 24;       // largest Rice / Exp-Golomb parameter accepted (the encoder writes <= 11)
constexpr int kP5MaxWidth = 32;   // largest fixed-width residual accepted

struct P5Args {
    const uint8_t* blob;       // stream bytes (64 zero bytes after the end)
    unsigned long long nbits;  // valid bits of the stream
    const uint32_t* start;     // meshlet m starts at start[m]; start[n] = stream end
    const uint32_t* row_base;  // first row of meshlet m's interior vertices
    const uint32_t* tri_base;  // first triangle of meshlet m
    const uint32_t* ref_base;  // first boundary reference of meshlet m
    uint32_t n_meshlets, n_boundary;
    double* rows;              // normalised positions (n_rows x 3)
    uint32_t* refs;            // boundary references of every meshlet
    uint32_t* walk;            // first-reach order per interior row: v | a << 8 | b << 16 | c << 24
    uint32_t* idx;             // output triangles (n_t x 3)
    double w0, w1, w2, delta;
    Status* status;
};

__device__ __forceinline__ void p5_report(Status* st, int code, uint32_t m) {
    const unsigned long long v = (static_cast<unsigned long long>(static_cast<unsigned>(code)) << 32) | m;
    atomicCAS(&st->err, 0ull, v);
}

// MSB-first reads from global memory (through L2, as every global read of
// the library) through a three-word register window: a read costs a funnel
// shift, and the word load that refills the window is issued a word ahead
// of its use.  The stream is read as big-endian 32-bit words (its device
// copy is 256-byte aligned and followed by 64 zero bytes, so the window
// never reads past the padding); a read never passes `limit`.
struct P5Bits {
    const uint32_t* w;
    unsigned long long pos, limit, wi;  // wi: word index of w0
    uint32_t w0, w1, w2;
    bool bad;
    __device__ __forceinline__ static uint32_t ld(const uint32_t* w, unsigned long long i) {
        return bswap32(__ldcg(w + i));
    }
    __device__ __forceinline__ void seek(unsigned long long p) {
        pos = p;
        wi = p >> 5;
        w0 = ld(w, wi);
        w1 = ld(w, wi + 1ull);
        w2 = ld(w, wi + 2ull);
    }
    __device__ __forceinline__ uint32_t peek() const {
        return __funnelshift_l(w1, w0, static_cast<uint32_t>(pos & 31ull));
    }
    // n <= 32: crosses at most one word boundary
    __device__ __forceinline__ void skip(uint32_t n) {
        pos += n;
        const unsigned long long ni = pos >> 5;
        if (ni != wi) {
            wi = ni;
            w0 = w1;
            w1 = w2;
            w2 = ld(w, wi + 2ull);
        }
    }
    __device__ __forceinline__ uint32_t bits(int n) {  // n <= 32
        if (n <= 0) return 0u;
        if (pos + static_cast<unsigned>(n) > limit) {
            bad = true;
            return 0u;
        }
        const uint32_t v = peek() >> (32 - n);
        skip(static_cast<uint32_t>(n));
        return v;
    }
    // zeros before the next one bit, and the one bit (BitReader unary prefix;
    // any length up to the end of the stream)
    __device__ __forceinline__ uint32_t unary() {
        uint32_t q = 0u;
        for (;;) {
            if (pos >= limit) {
                bad = true;
                return 0u;
            }
            const uint32_t x = peek();
            if (x) {
                const uint32_t z = static_cast<uint32_t>(__clz(x));
                q += z;
                skip(z + 1u);
                if (pos > limit) bad = true;
                return q;
            }
            q += 32u;
            skip(32u);
        }
    }
    // Rice(k) (BitReader.read_rice); q < 2^32 and k <= 24 fit 64 bits
    __device__ __forceinline__ unsigned long long rice(int k) {
        const uint32_t q = unary();
        const uint32_t low = bits(k);
        return (static_cast<unsigned long long>(q) << k) | low;
    }
    // Exp-Golomb(k) (BitReader.read_exp_golomb); a prefix above 32 bits (a
    // value of at least 2^32, never a residual of a valid stream) is rejected
    __device__ __forceinline__ unsigned long long eg(int k) {
        const uint32_t lb = unary();
        if (lb > 32u) {
            bad = true;
            return 0ull;
        }
        const uint32_t off = bits(static_cast<int>(lb));
        const unsigned long long s = ((1ull << lb) - 1ull) + off;
        const uint32_t low = bits(k);
        return (s << k) | low;
    }
};

// n <= 32 bits at an arbitrary position (fixed-width codes), 0 past `limit`
__device__ __forceinline__ uint32_t p5_bits_at(const uint32_t* w, unsigned long long pos, int n,
                                               unsigned long long limit, bool& bad) {
    if (n <= 0) return 0u;
    if (pos + static_cast<unsigned>(n) > limit) {
        bad = true;
        return 0u;
    }
    const unsigned long long i = pos >> 5;
    const uint32_t x = __funnelshift_l(P5Bits::ld(w, i + 1ull), P5Bits::ld(w, i), static_cast<uint32_t>(pos & 31ull));
    return x >> (32 - n);
}

__device__ __forceinline__ long long unzig(unsigned long long u) {
    return static_cast<long long>((u >> 1) ^ (0ull - (u & 1ull)));
}

// One axis' residual substream: tag 0 fixed width (random access), 1 Rice,
// 2 Exp-Golomb (paradelta_v5.py:405-424); tags 1 and 2 read through their
// own window.
struct P5Axis {
    int tag, k, bw;
    long long mn;
    unsigned long long base;  // first code (tag 0)
    P5Bits r;                 // the next code (tags 1, 2)
};


// One codeword of a Rice (eg false) or Exp-Golomb substream through its
// window: a straight-line read when prefix, terminator and value fit the
// 32-bit window, the general reader otherwise (rare; a branch taken by
// single lanes).  u is the codeword's value.
__device__ __forceinline__ unsigned long long p5_codeword(P5Bits& r, bool eg, int k) {
    const uint32_t x = r.peek();
    const uint32_t z = static_cast<uint32_t>(__clz(x));
    const uint32_t nb = (eg ? z : 0u) + static_cast<uint32_t>(k);
    const uint32_t len = z + 1u + nb;
    if (len > 32u || r.pos + len > r.limit) return eg ? r.eg(k) : r.rice(k);
    const uint32_t t = __funnelshift_lc(0u, x, z + 1u);      // bits after the terminator
    const uint32_t val = nb ? (t >> (32u - nb)) : 0u;        // the top nb of them
    const unsigned long long base = eg ? ((1ull << z) - 1ull) : static_cast<unsigned long long>(z);
    r.skip(len);
    return (base << k) + val;
}

constexpr int kP5Threads = 64;     // meshlets (lanes) per block
constexpr int kP5RefCache = 128;   // a lane's first boundary references kept in shared memory

// One lane per meshlet, 32 meshlets per warp, every phase a loop that the
// whole warp runs to its longest lane's count (no branch per token: the
// lanes stay together), as in the DPR4 kernels:
//  1. the meshlet header and its boundary references (:350-361), the first
//     kP5RefCache of them into shared memory;
//  2. connectivity, one token per iteration (strip header, roots, strip
//     bodies; the FIFO as a move-to-front register), triangles written as
//     rows, first-reach order of the interior vertices (:371-400);
//  3. the three residual substreams' starts (:403-424);
//  4. the float64 reconstruction in walk order (:426-445).
// Validity is checked lazily: running extremes and counts compared once per
// meshlet, ids clamped below n_local and writes bounded by the header's
// counts until then, so a corrupt lane runs on harmlessly and is reported.
__global__ void __launch_bounds__(kP5Threads) p5_decode_kernel(P5Args a) {
    __shared__ uint4 masks[17];
    __shared__ uint32_t seen_all[8 * kP5Threads];           // word i of lane t at [i * kP5Threads + t]
    __shared__ uint32_t ref_all[kP5RefCache * kP5Threads];  // reference l of lane t at [l * kP5Threads + t]
    if (threadIdx.x < 17u) masks[threadIdx.x] = threadIdx.x < 16u ? mtf_mask_row(threadIdx.x) : make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    const uint32_t m = blockIdx.x * kP5Threads + threadIdx.x;
    bool act = m < a.n_meshlets;
    const uint32_t mm = act ? m : 0u;
    const unsigned long long s0 = a.start[mm], s1 = a.start[mm + 1u];
    const bool last = mm + 1u == a.n_meshlets;
    const uint32_t* words = reinterpret_cast<const uint32_t*>(a.blob);
    P5Bits b;
    b.w = words;
    b.limit = a.nbits;
    b.bad = false;
    b.seek(act ? s0 : 0ull);
    uint32_t n_bnd = b.bits(16), n_int = b.bits(16), n_tris = b.bits(16), n_strips = b.bits(16);
    uint32_t n_local = n_bnd + n_int;
    bool bad = b.bad;
    if (act && n_local > static_cast<uint32_t>(kP5MaxLocal)) {
        p5_report(a.status, kErrUnsupported, m);
        act = false;
    }
    bad = bad || n_strips > n_tris;  // every strip emits a triangle
    if (!act || bad) n_bnd = n_int = n_tris = n_strips = n_local = 0u;
    const uint32_t rb = act ? a.ref_base[m] : 0u;
    const uint32_t row0 = act ? a.row_base[m] : 0u;
    uint32_t* tri = a.idx + 3ull * (act ? a.tri_base[m] : 0u);
    uint32_t* refc = ref_all + threadIdx.x;
    // 1. boundary references; the decoder reads them as rows of the boundary
    // table (a stream whose references point past it is rejected)
    if (n_bnd > 0u) {
        unsigned long long prev = b.bits(32);
        bad = bad || prev >= a.n_boundary;
        a.refs[rb] = static_cast<uint32_t>(prev);
        refc[0] = static_cast<uint32_t>(prev);
        const int k = n_bnd > 1u ? static_cast<int>(b.bits(8)) : 0;
        bad = bad || k > kP5MaxK;
        for (uint32_t i = 1; i < n_bnd && !bad; i++) {
            prev = prev + p5_codeword(b, false, k) + 1ull;
            bad = bad || b.bad || prev >= a.n_boundary;
            a.refs[rb + i] = static_cast<uint32_t>(prev);
            if (i < static_cast<uint32_t>(kP5RefCache)) refc[i * kP5Threads] = static_cast<uint32_t>(prev);
        }
    }
    auto row_of = [&](uint32_t l) -> uint32_t {
        if (l >= n_bnd) return row0 + (l - n_bnd);
        return l < static_cast<uint32_t>(kP5RefCache) ? refc[l * kP5Threads] : __ldcg(a.refs + rb + l);
    };
    // 2. connectivity
    uint32_t* seen = seen_all + threadIdx.x;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint32_t lo = 32u * i;
        seen[i * kP5Threads] = n_bnd >= lo + 32u ? 0xFFFFFFFFu : (n_bnd > lo ? (1u << (n_bnd - lo)) - 1u : 0u);
    }
    const uint32_t idx_bits = max(1u, 32u - __clz(n_local));  // max(1, ceil(log2(n_local + 1)))
    const uint32_t rsh = 32u - idx_bits, vmax = n_local ? n_local - 1u : 0u;
    MtfFifo f;
    uint32_t sl = n_strips, tl = 0u, tx = 0u, P = 0u, n_t = 0u, n_emit = 0u, ridmax = 0u;
    int32_t smin = 0;
    bool live = act && !bad && sl > 0u;
    const uint32_t iters = __reduce_max_sync(0xFFFFFFFFu, live ? n_tris + 2u * n_strips : 0u);
    for (uint32_t it = 0; it < iters; it++) {
        const uint32_t x0 = b.peek();
        const bool hdr = tl == 0u;                     // strip header (:376)
        const uint32_t sb = max(x0 >> 16, 1u) - 1u;   // body tokens of the strip
        tl = hdr ? sb + 3u : tl;
        sl -= hdr ? 1u : 0u;
        const uint32_t tix = hdr ? 0u : tx;
        uint32_t x = hdr ? (x0 << 16) : x0;
        uint32_t used = hdr ? 16u : 0u;
        const bool body = tix == 3u;
        const uint32_t ec = x >> 31;  // edge bit of a strip-body token
        x = body ? (x << 1) : x;
        used += body ? 1u : 0u;
        const bool raw = static_cast<int32_t>(x) < 0;  // _read_vert's flag
        const uint32_t y = x << 1;
        const uint32_t rid = y >> rsh;
        const uint32_t fi = y >> 27;
        used += raw ? 1u + idx_bits : 6u;
        // IndexError on a FIFO index past the entries or an id past n_local
        const int32_t sd = static_cast<int32_t>(f.len) - 1 - static_cast<int32_t>(fi);
        smin = min(smin, (raw | !live) ? 0 : sd);
        ridmax = max(ridmax, (raw & live) ? rid + 1u : 0u);
        const uint32_t sdep = static_cast<uint32_t>(sd) & 15u;
        const uint32_t v = raw ? (rid & 0xFFu) : f.at(sdep);
        const uint32_t at = raw ? f.find(v) : sdep;
        const bool fresh = at == 16u;
        f.mtf_masked(v, masks[live ? (fresh ? min(f.len, 15u) : at) : 16u]);  // row 16: no change
        f.len += (live & fresh & (f.len < 16u)) ? 1u : 0u;
        if (live) {
            const uint32_t u = min(v, vmax);
            // edge 0 -> (p1, p2 | p0), 1 -> (p0, p2 | p1) (:386-391); a root
            // token puts u at its position
            const uint32_t sel = body ? (ec ? 0x7420u : 0x7421u) : (0x7210u + ((4u - tix) << (4u * tix)));
            const uint32_t cref = ec ? ((P >> 8) & 0xFFu) : (P & 0xFFu);
            const uint32_t Pn = __byte_perm(P, u, sel);
            if ((body | (tix == 2u)) && n_t < n_tris) {
                tri[3u * n_t] = row_of(Pn & 0xFFu);
                tri[3u * n_t + 1u] = row_of((Pn >> 8) & 0xFFu);
                tri[3u * n_t + 2u] = row_of((Pn >> 16) & 0xFFu);
            }
            n_t += (body | (tix == 2u)) ? 1u : 0u;
            // first reach of an interior vertex (boundary bits are preset)
            uint32_t* sp = seen + (u >> 5) * kP5Threads;
            const uint32_t sw = *sp;
            const uint32_t bit = 1u << (u & 31u);
            if ((sw & bit) == 0u) {
                *sp = sw | bit;
                if (n_emit < n_int)
                    a.walk[row0 + n_emit] = body ? (u | ((Pn & 0xFFFFu) << 8) | (cref << 24)) : u * 0x01010101u;
                n_emit++;
            }
            P = Pn;
        }
        tl--;
        tx = min(tix + 1u, 3u);
        b.skip(live ? used : 0u);
        live = live & ((tl | sl) != 0u) & (b.pos <= b.limit);
    }
    bad = bad || live || b.pos > b.limit || smin < 0 || ridmax > n_local || n_t != n_tris || n_emit > n_int;
    // 3. residual substreams: tag, then fixed width (tag 0: minimum and width,
    // random access) or Rice / Exp-Golomb (tags 1, 2: k); each axis' start
    P5Axis ax[3];
    const bool vx = act && !bad && n_int > 0u;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        ax[d].tag = vx ? static_cast<int>(b.bits(8)) : 1;
        ax[d].k = 0;
        ax[d].bw = 0;
        ax[d].mn = 0;
        ax[d].base = 0ull;
        ax[d].r.w = words;
        ax[d].r.limit = a.nbits;
        ax[d].r.bad = false;
        if (ax[d].tag == 0) {
            const uint32_t mn_u = b.bits(16);
            ax[d].mn = (mn_u & 0x8000u) ? static_cast<long long>(mn_u) - 0x10000 : mn_u;
            ax[d].bw = static_cast<int>(b.bits(8));
            bad = bad || ax[d].bw > kP5MaxWidth;
            ax[d].base = b.pos;
            const unsigned long long e = b.pos + static_cast<unsigned long long>(n_int) * static_cast<unsigned>(ax[d].bw);
            bad = bad || e > b.limit;
            if (vx && !bad) b.seek(e);
        } else if (ax[d].tag == 1 || ax[d].tag == 2) {
            ax[d].k = vx ? static_cast<int>(b.bits(8)) : 0;
            bad = bad || ax[d].k > kP5MaxK;
            ax[d].r.seek(vx ? b.pos : 0ull);
        } else {
            bad = true;  // ValueError("bad tag")
        }
        // the substream's codewords, skipped (every lane of the warp takes
        // part in the count)
        const bool skipping = vx && !bad && (ax[d].tag == 1 || ax[d].tag == 2);
        const uint32_t n = __reduce_max_sync(0xFFFFFFFFu, skipping ? n_int : 0u);
        for (uint32_t i = 0; i < n; i++)
            if (skipping && i < n_int) (void)p5_codeword(b, ax[d].tag == 2, ax[d].k);
        bad = bad || b.bad;
    }
    // meshlets lie back to back, as the CPU decoder reads them
    if (act) {
        bad = bad || (last ? b.pos > a.nbits : b.pos != s1);
        if (bad) p5_report(a.status, kErrCorrupt, m);
    }
    // 4. reconstruction in float64, in the reference's operation order, no
    // contraction (:426-445).  A strip-body vertex is predicted from the
    // previous triangle, whose interior vertices were reconstructed a step
    // or two before: the last four interior rows stay in registers, so those
    // references do not wait for a store to come back from L2.
    const bool rec = act && !bad && n_int > 0u;
    double fb[3] = {0.0, 0.0, 0.0};
    if (rec && n_bnd > 0u) {
        for (int d = 0; d < 3; d++) {
            double s = __ldcg(a.rows + 3ull * row_of(0u) + d);
#pragma unroll 4
            for (uint32_t i = 1; i < n_bnd; i++) s = __dadd_rn(s, __ldcg(a.rows + 3ull * row_of(i) + d));
            fb[d] = __ddiv_rn(s, static_cast<double>(n_bnd));
        }
    }
    uint32_t cid[4] = {0xFFFFu, 0xFFFFu, 0xFFFFu, 0xFFFFu};  // local ids of the cached rows (newest first)
    double cx[4][3];
#pragma unroll
    for (int j = 0; j < 4; j++) cx[j][0] = cx[j][1] = cx[j][2] = 0.0;
    // coordinate d of local vertex l: a cached row or the rows array
    auto coord = [&](uint32_t l, unsigned long long o, int d) -> double {
        double r = 0.0;
        bool hit = false;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const bool h = cid[j] == l;
            r = h ? cx[j][d] : r;
            hit = hit || h;
        }
        return hit ? r : __ldcg(a.rows + o + d);
    };
    const uint32_t ne = __reduce_max_sync(0xFFFFFFFFu, rec ? n_emit : 0u);
    uint32_t e_next = (rec && n_emit > 0u) ? __ldcg(a.walk + row0) : 0u;
    for (uint32_t i = 0; i < ne; i++) {
        if (!rec || i >= n_emit) continue;
        const uint32_t e = e_next;
        if (i + 1u < n_emit) e_next = __ldcg(a.walk + row0 + i + 1u);  // the next entry, a step ahead
        const uint32_t v = e & 0xFFu, ra = (e >> 8) & 0xFFu, rbv = (e >> 16) & 0xFFu, rc = e >> 24;
        const bool para = ra != v;  // roots are stored as (v, v, v, v)
        const unsigned long long out = 3ull * row_of(v);
        const unsigned long long oa = 3ull * row_of(ra), ob = 3ull * row_of(rbv), oc = 3ull * row_of(rc);
        double nr[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            long long code;
            if (ax[d].tag == 0) {
                code = ax[d].mn + static_cast<long long>(p5_bits_at(words, ax[d].base + static_cast<unsigned long long>(i) *
                                                                               static_cast<unsigned>(ax[d].bw),
                                                                    ax[d].bw, a.nbits, bad));
            } else {
                code = unzig(p5_codeword(ax[d].r, ax[d].tag == 2, ax[d].k));
            }
            double pred = fb[d];
            if (para) {
                const double t0 = __dmul_rn(a.w0, coord(ra, oa, d));
                const double t1 = __dmul_rn(a.w1, coord(rbv, ob, d));
                const double t2 = __dmul_rn(a.w2, coord(rc, oc, d));
                pred = __dadd_rn(__dadd_rn(t0, t1), t2);
            }
            nr[d] = __dadd_rn(pred, __dmul_rn(static_cast<double>(code), a.delta));
            a.rows[out + d] = nr[d];
        }
#pragma unroll
        for (int j = 3; j > 0; j--) {
            cid[j] = cid[j - 1];
            cx[j][0] = cx[j - 1][0];
            cx[j][1] = cx[j - 1][1];
            cx[j][2] = cx[j - 1][2];
        }
        cid[0] = v;
        cx[0][0] = nr[0];
        cx[0][1] = nr[1];
        cx[0][2] = nr[2];
    }
}

// rows -> f32(row * scale + center)
__global__ void p5_world_kernel(const double* __restrict__ rows, unsigned long long n, double scale, double c0,
                                double c1, double c2, float* __restrict__ pos) {
    const unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
    if (i >= 3ull * n) return;
    const int d = static_cast<int>(i % 3ull);
    const double c = d == 0 ? c0 : (d == 1 ? c1 : c2);
    pos[i] = __double2float_rn(__dadd_rn(__dmul_rn(rows[i], scale), c));
}

// ---- host side ------------------------------------------------------------
struct HostBits {
    const uint8_t* p;
    unsigned long long nbits, pos;
    bool bad;
    uint64_t read(int n) {  // n <= 64
        if (n <= 0) return 0;
        if (pos + static_cast<unsigned>(n) > nbits) {
            bad = true;
            pos = nbits;
            return 0;
        }
        uint64_t v = 0;
        for (int i = 0; i < n; i++, pos++) v = (v << 1) | ((p[pos >> 3] >> (7 - (pos & 7))) & 1u);
        return v;
    }
    uint64_t rice(int k) {  // q < 2^32 (the stream length) and k <= 24 fit 64 bits
        uint64_t q = 0;
        for (;;) {
            if (pos >= nbits) {
                bad = true;
                return 0;
            }
            const unsigned bit = (p[pos >> 3] >> (7 - (pos & 7))) & 1u;
            pos++;
            if (bit) break;
            q++;
        }
        if (k > kP5MaxK) {
            bad = true;
            return 0;
        }
        return (q << k) | read(k);
    }
    float f32() {
        const uint32_t u = static_cast<uint32_t>(read(32));
        float f;
        std::memcpy(&f, &u, 4);
        return f;
    }
};

}  // namespace
}  // namespace stride

using namespace stride;

struct pldt5_handle {
    pldt5_info_t info;
    size_t len = 0;
    uint8_t* d_blob = nullptr;
    uint32_t* d_meta = nullptr;  // start (n + 1) | row_base (n) | tri_base (n) | ref_base (n)
    uint32_t* d_refs = nullptr;
    uint32_t* d_walk = nullptr;
    double* d_rows = nullptr;
    Status* d_status = nullptr;
    Status* h_status = nullptr;
    cudaEvent_t done = nullptr;
    bool launched = false;
    double w[3], delta, scale, center[3];
};

static void pldt5_free(pldt5_handle* h) {
    cudaFree(h->d_blob);
    cudaFree(h->d_meta);
    cudaFree(h->d_refs);
    cudaFree(h->d_walk);
    cudaFree(h->d_rows);
    cudaFree(h->d_status);
    if (h->h_status) cudaFreeHost(h->h_status);
    if (h->done) cudaEventDestroy(h->done);
    delete h;
}

// Host parse shared by pldt5_open and pldt5_inspect: header, boundary rows
// (float64), every meshlet's start bit and output placement.  STRIDE_OK or
// a STRIDE_ERR_* with the message set.
struct P5Host {
    pldt5_info_t info;
    float per_coord_err;
    std::vector<double> rows0;    // boundary rows, n_boundary x 3
    std::vector<uint32_t> meta;   // start (M + 1) | row_base (M) | tri_base (M) | ref_base (M)
    uint64_t refs = 0;
};

static int p5_host_parse_sized(const uint8_t* data, size_t len, P5Host& H);

// The host parse with its host allocations' failures turned into an error
// code (no exception may cross the C ABI).
static int p5_host_parse(const uint8_t* data, size_t len, P5Host& H) {
    try {
        return p5_host_parse_sized(data, len, H);
    } catch (const std::bad_alloc&) {
        return fail(STRIDE_ERR_NOMEM, "host memory for the PLDT v5 tables");
    } catch (const std::length_error&) {
        return fail(STRIDE_ERR_NOMEM, "host memory for the PLDT v5 tables");
    }
}

static int p5_host_parse_sized(const uint8_t* data, size_t len, P5Host& H) {
    pldt5_info_t& info = H.info;
    HostBits r{data, 8ull * len, 0, false};
    if (8ull * len < kP5HeaderBits) return fail(STRIDE_ERR_TRUNCATED, "PLDT v5 header past the end");
    std::memset(&info, 0, sizeof(info));
    const uint32_t magic = static_cast<uint32_t>(r.read(32));
    if (magic != kP5Magic) return fail(STRIDE_ERR_MAGIC, "bad magic 0x%08X (PLDT v5 expected)", magic);
    const uint32_t version = static_cast<uint32_t>(r.read(8));
    if (version != kP5Version) return fail(STRIDE_ERR_VERSION, "expected v5, got v%u", version);
    (void)r.read(8);  // code width: a shared-memory hint of the reference kernel
    for (int d = 0; d < 3; d++) info.center[d] = r.f32();
    info.scale = r.f32();
    const float per_coord_err = r.f32();
    H.per_coord_err = per_coord_err;
    float g_min[3], g_range[3];
    for (int d = 0; d < 3; d++) g_min[d] = r.f32();
    for (int d = 0; d < 3; d++) g_range[d] = r.f32();
    for (int d = 0; d < 3; d++) info.g_bits[d] = static_cast<uint32_t>(r.read(8));
    (void)r.read(32);  // n_v and n_t of the source mesh: the decoder counts its own
    (void)r.read(32);
    info.n_boundary = static_cast<uint32_t>(r.read(32));
    info.n_meshlets = static_cast<uint32_t>(r.read(32));
    for (int d = 0; d < 3; d++) info.lin3_w[d] = r.f32();
    for (int d = 0; d < 3; d++)
        if (info.g_bits[d] > 32) return fail(STRIDE_ERR_UNSUPPORTED, "g_bits %u above 32", info.g_bits[d]);
    // boundary table (parse_globals_v5, :538-560), positions in float64 like
    // the CPU decoder (:322-336)
    const uint64_t nb = info.n_boundary;
    // every row after the first takes at least one bit per axis (a Rice
    // codeword's terminator): the header's count is bounded by the bits
    // left before anything is sized from it
    if (nb > (8ull * len - r.pos) / 3ull + 1ull) return fail(STRIDE_ERR_TRUNCATED, "boundary table past the end");
    std::vector<double>& rows0 = H.rows0;
    rows0.assign(3 * nb, 0.0);
    {
        std::vector<int64_t> code(3 * nb, 0);
        for (int d = 0; d < 3 && nb > 0; d++) {
            code[d] = static_cast<int64_t>(r.read(static_cast<int>(info.g_bits[d])));
            if (nb > 1) {
                const int k = static_cast<int>(r.read(8));
                for (uint64_t i = 1; i < nb && !r.bad; i++) {
                    const uint64_t u = r.rice(k);
                    code[3 * i + d] = code[3 * (i - 1) + d] + static_cast<int64_t>((u >> 1) ^ (0ull - (u & 1ull)));
                }
            }
        }
        if (r.bad) return fail(STRIDE_ERR_TRUNCATED, "boundary table past the end or malformed");
        for (uint64_t i = 0; i < nb; i++)
            for (int d = 0; d < 3; d++) {
                const uint64_t mx = (1ull << info.g_bits[d]) - 1ull;
                if (mx == 0) {
                    rows0[3 * i + d] = static_cast<double>(g_min[d]);
                } else {
                    const double q = static_cast<double>(code[3 * i + d]) / static_cast<double>(mx);
                    rows0[3 * i + d] = static_cast<double>(g_min[d]) + q * static_cast<double>(g_range[d]);
                }
            }
    }
    // offset table, then every meshlet's header (the reference's sizes pass)
    r.pos += (0ull - r.pos) & 7ull;
    const uint64_t M = info.n_meshlets;
    if (r.pos + 32ull * M > r.nbits) return fail(STRIDE_ERR_TRUNCATED, "offset table past the end");
    std::vector<uint32_t>& meta = H.meta;
    meta.assign(4 * M + 1, 0u);
    uint32_t* start = meta.data();
    uint32_t* row_base = start + M + 1;
    uint32_t* tri_base = row_base + M;
    uint32_t* ref_base = tri_base + M;
    for (uint64_t m = 0; m < M; m++) start[m] = static_cast<uint32_t>(r.read(32));
    const uint64_t body = r.pos;
    start[M] = static_cast<uint32_t>(std::min<uint64_t>(8ull * len, 0xFFFFFFFFull));
    if (8ull * len > 0xFFFFFFFFull) return fail(STRIDE_ERR_UNSUPPORTED, "stream above 512 MiB");
    uint64_t rows = nb, tris = 0, refs = 0;
    for (uint64_t m = 0; m < M; m++) {
        // the CPU decoder reads meshlets back to back from the end of the table
        if ((m == 0 && start[0] != body) || start[m] < body || start[m] + 64ull > 8ull * len ||
            (m > 0 && start[m] <= start[m - 1]))
            return fail(STRIDE_ERR_OFFSET, "meshlet %llu offset out of order or range", (unsigned long long)m);
        HostBits hb{data, 8ull * len, start[m], false};
        const uint32_t n_bnd = static_cast<uint32_t>(hb.read(16));
        const uint32_t n_int = static_cast<uint32_t>(hb.read(16));
        const uint32_t n_tris = static_cast<uint32_t>(hb.read(16));
        if (n_bnd + n_int > static_cast<uint32_t>(kP5MaxLocal))
            return fail(STRIDE_ERR_UNSUPPORTED, "meshlet %llu has %u local vertices (at most 256)",
                        (unsigned long long)m, n_bnd + n_int);
        row_base[m] = static_cast<uint32_t>(rows);
        tri_base[m] = static_cast<uint32_t>(tris);
        ref_base[m] = static_cast<uint32_t>(refs);
        rows += n_int;
        tris += n_tris;
        refs += n_bnd;
        if (rows > 0xFFFFFFFFull || tris > 0x55555555ull || refs > 0xFFFFFFFFull)
            return fail(STRIDE_ERR_UNSUPPORTED, "more than 2^32 rows, indices or boundary references");
    }
    info.n_v = rows;
    info.n_t = tris;
    info.nbytes = len;
    H.refs = refs;
    return STRIDE_OK;
}

extern "C" {

int pldt5_open(const uint8_t* data, size_t len, pldt5_handle** out) {
    if (!out || (!data && len)) return fail(STRIDE_ERR_ARG, "null argument");
    *out = nullptr;
    P5Host H;
    const int prc = p5_host_parse(data, len, H);
    if (prc) return prc;
    const pldt5_info_t& info = H.info;
    const uint64_t nb = info.n_boundary, rows = info.n_v, refs = H.refs;
    const float per_coord_err = H.per_coord_err;
    const std::vector<double>& rows0 = H.rows0;
    const std::vector<uint32_t>& meta = H.meta;

    pldt5_handle* h = new pldt5_handle();
    h->info = info;
    h->len = len;
    for (int d = 0; d < 3; d++) {
        h->w[d] = static_cast<double>(info.lin3_w[d]);
        h->center[d] = static_cast<double>(info.center[d]);
    }
    h->scale = static_cast<double>(info.scale);
    h->delta = 2.0 * static_cast<double>(per_coord_err);
    cudaError_t e;
    const size_t blob = blob_alloc_bytes(len);
    if ((e = cudaMalloc(&h->d_blob, blob)) != cudaSuccess ||
        (e = cudaMalloc(&h->d_meta, 4 * meta.size())) != cudaSuccess ||
        (e = cudaMalloc(&h->d_refs, 4 * std::max<uint64_t>(refs, 1))) != cudaSuccess ||
        (e = cudaMalloc(&h->d_walk, 4 * std::max<uint64_t>(rows, 1))) != cudaSuccess ||
        (e = cudaMalloc(&h->d_rows, 24 * std::max<uint64_t>(rows, 1))) != cudaSuccess ||
        (e = cudaMalloc(&h->d_status, sizeof(Status))) != cudaSuccess ||
        (e = cudaHostAlloc(reinterpret_cast<void**>(&h->h_status), sizeof(Status), cudaHostAllocDefault)) !=
            cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming)) != cudaSuccess) {
        pldt5_free(h);
        return cuda_fail(e, "pldt5_open");
    }
    if ((e = cudaMemset(h->d_blob, 0, blob)) != cudaSuccess ||
        (len && (e = cudaMemcpy(h->d_blob, data, len, cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (e = cudaMemcpy(h->d_meta, meta.data(), 4 * meta.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (nb && (e = cudaMemcpy(h->d_rows, rows0.data(), 24 * nb, cudaMemcpyHostToDevice)) != cudaSuccess)) {
        pldt5_free(h);
        return cuda_fail(e, "pldt5_open upload");
    }
    *out = h;
    return STRIDE_OK;
}

int pldt5_inspect(const uint8_t* data, size_t len, pldt5_info_t* info) {
    if (!info || (!data && len)) return fail(STRIDE_ERR_ARG, "null argument");
    P5Host H;
    const int rc = p5_host_parse(data, len, H);
    if (rc) return rc;
    *info = H.info;
    return STRIDE_OK;
}

int pldt5_info(const pldt5_handle* h, pldt5_info_t* info) {
    if (!h || !info) return fail(STRIDE_ERR_ARG, "null argument");
    *info = h->info;
    return STRIDE_OK;
}

int pldt5_decode(pldt5_handle* h, void* stream, uint32_t* d_idx, float* d_pos) {
    if (!h || (!d_idx && h->info.n_t) || (!d_pos && h->info.n_v)) return fail(STRIDE_ERR_ARG, "null argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint64_t M = h->info.n_meshlets, nb = h->info.n_boundary, rows = h->info.n_v;
    cudaError_t e;
    if ((e = cudaMemsetAsync(h->d_status, 0, sizeof(Status), s)) != cudaSuccess ||
        (rows > nb && (e = cudaMemsetAsync(h->d_rows + 3 * nb, 0, 24 * (rows - nb), s)) != cudaSuccess))
        return cuda_fail(e, "pldt5_decode");
    if (M) {
        P5Args a;
        a.blob = h->d_blob;
        a.nbits = 8ull * h->len;
        a.start = h->d_meta;
        a.row_base = h->d_meta + M + 1;
        a.tri_base = a.row_base + M;
        a.ref_base = a.tri_base + M;
        a.n_meshlets = static_cast<uint32_t>(M);
        a.n_boundary = static_cast<uint32_t>(nb);
        a.rows = h->d_rows;
        a.refs = h->d_refs;
        a.walk = h->d_walk;
        a.idx = d_idx;
        a.w0 = h->w[0];
        a.w1 = h->w[1];
        a.w2 = h->w[2];
        a.delta = h->delta;
        a.status = h->d_status;
        // one lane per meshlet (kP5Threads per block)
        p5_decode_kernel<<<static_cast<uint32_t>((M + kP5Threads - 1) / kP5Threads), kP5Threads, 0, s>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "p5_decode_kernel");
    }
    if (rows) {
        p5_world_kernel<<<static_cast<uint32_t>((3 * rows + 255) / 256), 256, 0, s>>>(
            h->d_rows, rows, h->scale, h->center[0], h->center[1], h->center[2], d_pos);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "p5_world_kernel");
    }
    if ((e = cudaMemcpyAsync(h->h_status, h->d_status, sizeof(Status), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaEventRecord(h->done, s)) != cudaSuccess)
        return cuda_fail(e, "pldt5_decode");
    h->launched = true;
    return STRIDE_OK;
}

int pldt5_status(pldt5_handle* h, int wait) {
    if (!h) return fail(STRIDE_ERR_ARG, "null handle");
    if (!h->launched) return STRIDE_OK;
    cudaError_t e = wait ? cudaEventSynchronize(h->done) : cudaEventQuery(h->done);
    if (e == cudaErrorNotReady) return STRIDE_ERR_BUSY;
    if (e != cudaSuccess) return cuda_fail(e, "pldt5_status");
    uint32_t bad = 0;
    const int rc = status_to_code(*h->h_status, &bad);
    if (rc) return fail(rc, "%s (meshlet %u)", status_message(rc), bad);
    return STRIDE_OK;
}

void pldt5_close(pldt5_handle* h) {
    if (!h) return;
    if (h->launched) cudaEventSynchronize(h->done);
    pldt5_free(h);
}

}  // extern "C"
