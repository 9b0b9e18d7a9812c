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

__device__ __forceinline__ long long p5_code(P5Axis& ax, uint32_t i, bool& bad) {
    if (ax.tag == 0)
        return ax.mn + static_cast<long long>(p5_bits_at(ax.r.w, ax.base + static_cast<unsigned long long>(i) *
                                                                             static_cast<unsigned>(ax.bw),
                                                         ax.bw, ax.r.limit, bad));
    const unsigned long long u = ax.tag == 1 ? ax.r.rice(ax.k) : ax.r.eg(ax.k);
    bad = bad || ax.r.bad;
    return unzig(u);
}

// One token's local id through the FIFO of the 16 most recently used ids
// (_read_vert, encoder/paradelta_codec.py:330-340): a move-to-front register
// (depth 0 the newest, so the FIFO index fi, 0 the oldest, is depth
// len - 1 - fi), an id found in it moved to the front, a new one pushed
// (the oldest leaving a full FIFO).
__device__ __forceinline__ int p5_vert(P5Bits& b, MtfFifo& f, int idx_bits, const uint4* masks, bool& bad) {
    uint32_t x, at;
    if (b.bits(1) == 0u) {
        const uint32_t fi = b.bits(5);
        if (fi >= f.len) {
            bad = true;
            return 0;
        }
        at = f.len - 1u - fi;
        x = f.at(at);
    } else {
        x = b.bits(idx_bits);
        at = x < 256u ? f.find(x) : 16u;
    }
    const bool fresh = at == 16u;
    f.mtf_masked(x & 0xFFu, masks[fresh ? min(f.len, 15u) : at]);
    f.len += (fresh && f.len < 16u) ? 1u : 0u;
    return static_cast<int>(x);
}

// Lane l < per_warp of warp w decodes meshlet w * per_warp + l: the lanes of
// a warp take different branches on almost every token, so a stream with
// few meshlets gets one per warp, spread over the SMs.
__global__ void __launch_bounds__(128) p5_decode_kernel(P5Args a, uint32_t per_warp) {
    __shared__ uint4 masks[16];
    __shared__ uint32_t seen_all[8 * 128];  // each thread's first-reach bits: word i at [i * 128 + thread]
    if (threadIdx.x < 16u) masks[threadIdx.x] = mtf_mask_row(threadIdx.x);
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (lane >= per_warp) return;
    const uint32_t m = warp * per_warp + lane;
    if (m >= a.n_meshlets) return;
    const unsigned long long s0 = a.start[m], s1 = a.start[m + 1];
    const bool last = m + 1 == a.n_meshlets;
    const uint32_t* words = reinterpret_cast<const uint32_t*>(a.blob);
    P5Bits b;
    b.w = words;
    b.limit = a.nbits;
    b.bad = false;
    b.seek(s0);
    bool bad = false;
    const int n_bnd = static_cast<int>(b.bits(16));
    const int n_int = static_cast<int>(b.bits(16));
    const int n_tris = static_cast<int>(b.bits(16));
    const int n_strips = static_cast<int>(b.bits(16));
    const int n_local = n_bnd + n_int;
    if (n_local > kP5MaxLocal) {
        p5_report(a.status, kErrUnsupported, m);
        return;
    }
    const uint32_t rb = a.ref_base[m];
    const uint32_t row0 = a.row_base[m];
    uint32_t* tri = a.idx + 3ull * a.tri_base[m];
    // boundary references (:350-361); the decoder reads them as rows of the
    // boundary table (a stream whose references point past it is rejected)
    if (n_bnd > 0) {
        unsigned long long prev = b.bits(32);
        a.refs[rb] = static_cast<uint32_t>(prev);
        bad = bad || prev >= a.n_boundary;
        if (n_bnd > 1) {
            const int k = static_cast<int>(b.bits(8));
            bad = bad || k > kP5MaxK;
            for (int i = 1; i < n_bnd && !bad && !b.bad; i++) {
                prev = prev + b.rice(k) + 1ull;
                bad = bad || prev >= a.n_boundary;
                a.refs[rb + i] = static_cast<uint32_t>(prev);
            }
        }
    }
    auto row_of = [&](int l) -> unsigned long long {
        return l < n_bnd ? __ldcg(a.refs + rb + l) : row0 + static_cast<unsigned>(l - n_bnd);
    };
    // connectivity and first-reach order (:371-400)
    uint32_t* seen = seen_all + threadIdx.x;
#pragma unroll
    for (int i = 0; i < 8; i++) seen[i * 128] = 0u;
    for (int l = 0; l < n_bnd; l++) seen[(l >> 5) * 128] |= 1u << (l & 31);
    int idx_bits = 1;
    while ((1 << idx_bits) <= n_local) idx_bits++;  // max(1, ceil(log2(n_local + 1)))
    MtfFifo f;
    int n_t = 0, n_emit = 0;
    auto reach = [&](int v, uint32_t entry) {
        uint32_t* sp = seen + (v >> 5) * 128;
        const uint32_t sw = *sp;
        const uint32_t bit = 1u << (v & 31);
        if (v >= n_bnd && !(sw & bit)) {
            if (n_emit >= n_int) {
                bad = true;
            } else {
                a.walk[row0 + n_emit] = entry;
                n_emit++;
            }
        }
        *sp = sw | bit;
    };
    auto put_tri = [&](int x, int y, int z) {
        if (n_t >= n_tris) {
            bad = true;
            return;
        }
        tri[3 * n_t] = static_cast<uint32_t>(row_of(x));
        tri[3 * n_t + 1] = static_cast<uint32_t>(row_of(y));
        tri[3 * n_t + 2] = static_cast<uint32_t>(row_of(z));
        n_t++;
    };
    for (int s = 0; s < n_strips && !bad && !b.bad; s++) {
        const int strip_len = static_cast<int>(b.bits(16));
        int v[3];
        for (int j = 0; j < 3; j++) {
            v[j] = p5_vert(b, f, idx_bits, masks, bad);
            bad = bad || v[j] >= n_local;
        }
        if (bad || b.bad) break;
        put_tri(v[0], v[1], v[2]);
        for (int j = 0; j < 3; j++) reach(v[j], static_cast<uint32_t>(v[j]) * 0x01010101u);
        int p0 = v[0], p1 = v[1], p2 = v[2];
        for (int t = 0; t + 1 < strip_len && !bad && !b.bad; t++) {
            const uint32_t edge = b.bits(1);
            const int nv = p5_vert(b, f, idx_bits, masks, bad);
            if (nv >= n_local) bad = true;
            if (bad || b.bad) break;
            int x, y, c;
            if (edge == 0u) {
                x = p1; y = p2; c = p0;
            } else {
                x = p0; y = p2; c = p1;
            }
            put_tri(x, y, nv);
            reach(nv, static_cast<uint32_t>(nv) | static_cast<uint32_t>(x) << 8 | static_cast<uint32_t>(y) << 16 |
                          static_cast<uint32_t>(c) << 24);
            p0 = x; p1 = y; p2 = nv;
        }
    }
    bad = bad || b.bad || n_t != n_tris;  // the header's count must match the strips
    // residual substreams (:403-424): find each axis' start
    P5Axis ax[3];
    if (!bad && n_int > 0) {
        for (int d = 0; d < 3 && !bad; d++) {
            ax[d].tag = static_cast<int>(b.bits(8));
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
                if (!bad) b.seek(e);
            } else if (ax[d].tag == 1 || ax[d].tag == 2) {
                ax[d].k = static_cast<int>(b.bits(8));
                bad = bad || ax[d].k > kP5MaxK;
                ax[d].r.seek(b.pos);
                for (int i = 0; i < n_int && !bad && !b.bad; i++) (void)(ax[d].tag == 1 ? b.rice(ax[d].k) : b.eg(ax[d].k));
            } else {
                bad = true;  // ValueError("bad tag")
            }
            bad = bad || b.bad;
        }
    }
    // meshlets lie back to back, as the CPU decoder reads them
    bad = bad || (last ? b.pos > a.nbits : b.pos != s1);
    if (bad) {
        p5_report(a.status, kErrCorrupt, m);
        return;
    }
    if (n_int == 0) return;
    // reconstruction in float64, in the reference's operation order, no
    // contraction (:426-445)
    double fb[3] = {0.0, 0.0, 0.0};
    if (n_bnd > 0) {
        for (int d = 0; d < 3; d++) {
            double s = a.rows[3ull * a.refs[rb] + d];
            for (int i = 1; i < n_bnd; i++) s = __dadd_rn(s, a.rows[3ull * a.refs[rb + i] + d]);
            fb[d] = __ddiv_rn(s, static_cast<double>(n_bnd));
        }
    }
    for (int i = 0; i < n_emit; i++) {
        const uint32_t e = a.walk[row0 + i];
        const int v = static_cast<int>(e & 0xFFu);
        const int ra = static_cast<int>((e >> 8) & 0xFFu);
        const int rbv = static_cast<int>((e >> 16) & 0xFFu);
        const int rc = static_cast<int>(e >> 24);
        const bool para = ra != v;  // roots are stored as (v, v, v, v)
        const unsigned long long out = 3ull * row_of(v);
        const unsigned long long oa = para ? 3ull * row_of(ra) : 0ull;
        const unsigned long long ob = para ? 3ull * row_of(rbv) : 0ull;
        const unsigned long long oc = para ? 3ull * row_of(rc) : 0ull;
        for (int d = 0; d < 3; d++) {
            const long long code = p5_code(ax[d], static_cast<uint32_t>(i), bad);
            double pred = fb[d];
            if (para) {
                const double t0 = __dmul_rn(a.w0, a.rows[oa + d]);
                const double t1 = __dmul_rn(a.w1, a.rows[ob + d]);
                const double t2 = __dmul_rn(a.w2, a.rows[oc + d]);
                pred = __dadd_rn(__dadd_rn(t0, t1), t2);
            }
            a.rows[out + d] = __dadd_rn(pred, __dmul_rn(static_cast<double>(code), a.delta));
        }
    }
    if (bad) p5_report(a.status, kErrCorrupt, m);  // cannot happen: the substreams were read once already
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
        // about sixteen busy warps per SM, at most 32 meshlets per warp
        const uint64_t target = 16ull * static_cast<uint64_t>(device_sm_count());
        const uint32_t per_warp = static_cast<uint32_t>(std::min<uint64_t>(32, std::max<uint64_t>(1, (M + target - 1) / target)));
        const uint64_t warps = (M + per_warp - 1) / per_warp;
        p5_decode_kernel<<<static_cast<uint32_t>((warps + 3) / 4), 128, 0, s>>>(a, per_warp);
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
