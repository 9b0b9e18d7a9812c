// Project STRIDE (DPR4 v3) encoder -- produces decoder inputs at scale.
//
// Writes the byte layout of the reference encoder
//   encode_dup / _write_meshlet_dup   encoder/paradelta_v5_dup.py:239-464
// from a triangle mesh, with its own meshlet partition and strip builder
// (the reference uses a learned joint partition and multi-seed strips,
// encoder/paradelta_codec.py:758-883; any valid partition decodes the same
// way).  Quantisation follows _quantize_global
// (encoder/paradelta_codec.py:149-165) and the two precision modes of
// prepare_paradelta_arrays (:769-786).  The predictor is either the
// canonical parallelogram ((1,1,-1), K=0) or a per-mesh integer-rational
// fit of this file's own (least squares, then rounding at K in 5..9 with a
// bit-cost choice), stored in the same 21-byte v3 header field.
//
// Host-only C++ (no CUDA); built into libstride_encode.so.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

constexpr uint32_t kMagic = 0x44505234u;
constexpr int kVersion = 3;
constexpr int kFifo = 16;
constexpr int kReuseBits = 5;

struct BitWriter {
    std::vector<uint8_t> buf;
    uint64_t acc = 0;
    int nacc = 0;
    void put(uint64_t v, int n) {  // n <= 32 per call
        if (n <= 0) return;
        v &= (n == 64) ? ~0ull : ((1ull << n) - 1ull);
        acc = (acc << n) | v;
        nacc += n;
        while (nacc >= 8) {
            buf.push_back(static_cast<uint8_t>(acc >> (nacc - 8)));
            nacc -= 8;
        }
        acc &= (nacc ? ((1ull << nacc) - 1ull) : 0ull);
    }
    void put_wide(uint64_t v, int n) {
        while (n > 32) {
            put(v >> (n - 32), 32);
            n -= 32;
        }
        put(v, n);
    }
    void zeros(uint64_t n) {
        while (n >= 32) { put(0, 32); n -= 32; }
        put(0, static_cast<int>(n));
    }
    uint64_t bitpos() const { return buf.size() * 8ull + static_cast<uint64_t>(nacc); }
    void rice(uint64_t u, int k) {
        zeros(u >> k);
        put(1, 1);
        put(u & ((1ull << k) - 1ull), k);
    }
    void eg(uint64_t u, int k) {
        uint64_t s = u >> k;
        int lb = 0;
        for (uint64_t x = s + 1; x > 1; x >>= 1) lb++;
        zeros(static_cast<uint64_t>(lb));
        put(1, 1);
        if (lb) put_wide(s - ((1ull << lb) - 1ull), lb);
        put(u & ((1ull << k) - 1ull), k);
    }
    std::vector<uint8_t> finish() {
        if (nacc) put(0, 8 - nacc);
        return buf;
    }
};

inline uint64_t zigzag(int64_t r) { return r >= 0 ? (static_cast<uint64_t>(r) << 1) : ((static_cast<uint64_t>(-r) << 1) - 1); }

inline int bitlen64(uint64_t x) { return x ? 64 - __builtin_clzll(x) : 0; }

uint64_t rice_bits(const std::vector<uint64_t>& u, int k) {
    uint64_t b = 0;
    for (uint64_t x : u) b += (x >> k) + 1 + k;
    return b;
}
uint64_t eg_bits(const std::vector<uint64_t>& u, int k) {
    uint64_t b = 0;
    for (uint64_t x : u) b += 2 * (bitlen64((x >> k) + 1) - 1) + 1 + k;
    return b;
}

// Per-axis (tag, k) choice, as _pick_best_k (paradelta_v5_dup.py:159-171):
// Rice k in [0, 11] vs Exp-Golomb k in [0, 7], ties to Rice; empty -> Rice 0.
void pick_tag_k(const std::vector<uint64_t>& u, int* tag, int* k) {
    if (u.empty()) { *tag = 1; *k = 0; return; }
    uint64_t br = ~0ull, be = ~0ull;
    int kr = 0, ke = 0;
    for (int kk = 0; kk <= 11; kk++) { uint64_t b = rice_bits(u, kk); if (b < br) { br = b; kr = kk; } }
    for (int kk = 0; kk <= 7; kk++) { uint64_t b = eg_bits(u, kk); if (b < be) { be = b; ke = kk; } }
    if (br <= be) { *tag = 1; *k = kr; } else { *tag = 2; *k = ke; }
}

struct Meshlet {
    std::vector<uint32_t> l2g;         // local id -> global vertex
    std::vector<uint32_t> tokens;      // packed: bit31 = strip start, bits 16..23 ec(0/1)+1 for body, low 16 = local id
    std::vector<uint16_t> strip_lens;
    uint32_t n_tris = 0;
    // walk in decode order: local id, kind (0 none / 1 para), refs a,b,c
    std::vector<uint32_t> walk_v;
    std::vector<uint8_t> walk_para;
    std::vector<uint32_t> walk_ref;
};

struct Encoder {
    const double* V;
    uint64_t nv;
    const int64_t* T;
    uint64_t nt;
    int max_verts, max_tris;
    std::vector<int32_t> adj;  // 3 per tri: neighbour across edge e = (t[e], t[e+1]) or -1
    std::vector<int32_t> lmap, lstamp;  // global vertex -> local id, valid when lstamp == meshlet mark
    uint32_t meshlet_counter = 0;

    void build_adjacency() {
        adj.assign(3 * nt, -1);
        struct E { uint64_t key; uint32_t tri; uint8_t e; };
        std::vector<E> es;
        es.reserve(3 * nt);
        for (uint64_t t = 0; t < nt; t++) {
            int64_t a = T[3 * t], b = T[3 * t + 1], c = T[3 * t + 2];
            if (a == b || b == c || a == c) continue;  // degenerate: no neighbours
            for (int e = 0; e < 3; e++) {
                uint64_t u = static_cast<uint64_t>(T[3 * t + e]);
                uint64_t w = static_cast<uint64_t>(T[3 * t + (e + 1) % 3]);
                if (u > w) std::swap(u, w);
                es.push_back({u * nv + w, static_cast<uint32_t>(t), static_cast<uint8_t>(e)});
            }
        }
        std::sort(es.begin(), es.end(), [](const E& x, const E& y) { return x.key < y.key; });
        for (size_t i = 0; i < es.size();) {
            size_t j = i;
            while (j < es.size() && es[j].key == es[i].key) j++;
            if (j - i == 2) {  // manifold edge; non-manifold edges get no adjacency
                adj[3 * es[i].tri + es[i].e] = static_cast<int32_t>(es[i + 1].tri);
                adj[3 * es[i + 1].tri + es[i + 1].e] = static_cast<int32_t>(es[i].tri);
            }
            i = j;
        }
    }

    // Greedy region growth: repeatedly add the frontier triangle that brings
    // the fewest new vertices, within max_verts / max_tris.
    std::vector<std::vector<uint32_t>> partition() {
        std::vector<int32_t> owner(nt, -1);
        std::vector<int32_t> vstamp(nv, -1);
        std::vector<std::vector<uint32_t>> out;
        std::vector<uint32_t> bucket[4];
        size_t head[4];
        uint64_t scan = 0;
        std::vector<uint32_t> carry;  // unassigned frontier of the previous meshlet
        while (true) {
            int64_t seed = -1;
            for (uint32_t t : carry)
                if (owner[t] < 0) { seed = t; break; }
            if (seed < 0) {
                while (scan < nt && owner[scan] >= 0) scan++;
                if (scan >= nt) break;
                seed = static_cast<int64_t>(scan);
            }
            int32_t cur = static_cast<int32_t>(out.size());
            std::vector<uint32_t> tris;
            uint32_t nverts = 0;
            for (int b = 0; b < 4; b++) { bucket[b].clear(); head[b] = 0; }
            auto newcount = [&](uint32_t t) {
                const int64_t a = T[3 * t], b = T[3 * t + 1], c = T[3 * t + 2];
                int n = vstamp[a] != cur;
                n += (b != a) && vstamp[b] != cur;
                n += (c != a && c != b) && vstamp[c] != cur;
                return n;
            };
            bucket[newcount(static_cast<uint32_t>(seed))].push_back(static_cast<uint32_t>(seed));
            while (tris.size() < static_cast<size_t>(max_tris)) {
                int b = 0;
                while (b < 4 && head[b] >= bucket[b].size()) b++;
                if (b == 4) break;
                uint32_t t = bucket[b][head[b]++];
                if (owner[t] >= 0) continue;
                int c = newcount(t);
                if (c < b) { bucket[c].push_back(t); continue; }
                if (nverts + c > static_cast<uint32_t>(max_verts)) continue;
                owner[t] = cur;
                tris.push_back(t);
                for (int k = 0; k < 3; k++) {
                    int64_t v = T[3 * t + k];
                    if (vstamp[v] != cur) { vstamp[v] = cur; nverts++; }
                }
                for (int e = 0; e < 3; e++) {
                    int32_t n = adj[3 * t + e];
                    if (n >= 0 && owner[n] < 0) bucket[newcount(static_cast<uint32_t>(n))].push_back(static_cast<uint32_t>(n));
                }
            }
            carry.clear();
            for (int b = 0; b < 4; b++)
                for (size_t i = head[b]; i < bucket[b].size(); i++)
                    if (owner[bucket[b][i]] < 0) carry.push_back(bucket[b][i]);
            out.push_back(std::move(tris));
        }
        return out;
    }

    // Strips inside one meshlet + FIFO tokens + decode-order walk.
    Meshlet strips(const std::vector<uint32_t>& tris, std::vector<int32_t>& tri_local) {
        Meshlet m;
        const uint32_t nT = static_cast<uint32_t>(tris.size());
        for (uint32_t i = 0; i < nT; i++) tri_local[tris[i]] = static_cast<int32_t>(i);
        auto lnb = [&](uint32_t li, int e) -> int32_t {
            int32_t n = adj[3 * tris[li] + e];
            if (n < 0) return -1;
            int32_t l = tri_local[n];
            return (l >= 0 && l < static_cast<int32_t>(nT) && tris[l] == static_cast<uint32_t>(n)) ? l : -1;
        };
        std::vector<uint8_t> visited(nT, 0);
        std::vector<uint8_t> deg(nT, 0);
        for (uint32_t i = 0; i < nT; i++)
            for (int e = 0; e < 3; e++) deg[i] += lnb(i, e) >= 0;
        auto visit = [&](uint32_t li) {
            visited[li] = 1;
            for (int e = 0; e < 3; e++) { int32_t n = lnb(li, e); if (n >= 0 && deg[n]) deg[n]--; }
        };
        // neighbour of li across the edge {u, w}; returns local tri and its third vertex
        auto across = [&](uint32_t li, int64_t u, int64_t w, int64_t* third) -> int32_t {
            const int64_t* t = &T[3 * tris[li]];
            for (int e = 0; e < 3; e++) {
                int64_t x = t[e], y = t[(e + 1) % 3];
                if ((x == u && y == w) || (x == w && y == u)) {
                    int32_t n = lnb(li, e);
                    if (n < 0 || visited[n]) return -1;
                    const int64_t* q = &T[3 * tris[n]];
                    for (int k = 0; k < 3; k++)
                        if (q[k] != u && q[k] != w) { *third = q[k]; return n; }
                    return -1;
                }
            }
            return -1;
        };
        std::vector<int64_t> order_g;  // emitted global vertex per token
        std::vector<uint32_t> tok_meta;
        uint32_t done = 0;
        while (done < nT) {
            int32_t start = -1;
            for (uint32_t i = 0; i < nT; i++)
                if (!visited[i] && (start < 0 || deg[i] < deg[start])) start = static_cast<int32_t>(i);
            const int64_t* t = &T[3 * tris[start]];
            int64_t p0 = t[0], p1 = t[1], p2 = t[2];
            // orient the root so the best next triangle shares (p1, p2)
            int32_t best = -1;
            int bestdeg = 99;
            for (int e = 0; e < 3; e++) {
                int32_t n = lnb(static_cast<uint32_t>(start), e);
                if (n >= 0 && !visited[n] && deg[n] < bestdeg) { best = e; bestdeg = deg[n]; }
            }
            if (best >= 0) {
                p1 = t[best];
                p2 = t[(best + 1) % 3];
                p0 = t[(best + 2) % 3];
            }
            visit(static_cast<uint32_t>(start));
            done++;
            uint32_t len = 1;
            order_g.push_back(p0); tok_meta.push_back(1u << 31);
            order_g.push_back(p1); tok_meta.push_back(0);
            order_g.push_back(p2); tok_meta.push_back(0);
            uint32_t curt = static_cast<uint32_t>(start);
            while (len < 65535) {
                int64_t n0v = 0, n1v = 0;
                int32_t c0 = across(curt, p1, p2, &n0v);  // ec = 0
                int32_t c1 = across(curt, p0, p2, &n1v);  // ec = 1
                if (c0 < 0 && c1 < 0) break;
                int ec;
                if (c0 >= 0 && c1 >= 0) ec = deg[c0] <= deg[c1] ? 0 : 1;
                else ec = c0 >= 0 ? 0 : 1;
                int64_t nv_ = ec == 0 ? n0v : n1v;
                int32_t nt_ = ec == 0 ? c0 : c1;
                if (ec == 0) { p0 = p1; p1 = p2; } else { p1 = p2; }
                p2 = nv_;
                order_g.push_back(nv_);
                tok_meta.push_back(static_cast<uint32_t>(ec + 1) << 16);
                visit(static_cast<uint32_t>(nt_));
                curt = static_cast<uint32_t>(nt_);
                done++;
                len++;
            }
            m.strip_lens.push_back(static_cast<uint16_t>(len));
        }
        m.n_tris = nT;
        for (uint32_t i = 0; i < nT; i++) tri_local[tris[i]] = -1;
        // local ids by first appearance; walk exactly as the decoder replays it
        const int32_t mark = static_cast<int32_t>(++meshlet_counter);
        auto local_of = [&](int64_t g) -> uint32_t {
            if (lstamp[g] == mark) return static_cast<uint32_t>(lmap[g]);
            lstamp[g] = mark;
            lmap[g] = static_cast<int32_t>(m.l2g.size());
            m.l2g.push_back(static_cast<uint32_t>(g));
            return static_cast<uint32_t>(lmap[g]);
        };
        std::vector<uint8_t> decoded;
        m.tokens.reserve(order_g.size());
        uint32_t q0 = 0, q1 = 0, q2 = 0;
        size_t i = 0;
        for (size_t s = 0; s < m.strip_lens.size(); s++) {
            uint32_t r[3];
            for (int k = 0; k < 3; k++, i++) {
                r[k] = local_of(order_g[i]);
                m.tokens.push_back((k == 0 ? (1u << 31) : 0u) | r[k]);
            }
            for (int k = 0; k < 3; k++) {
                if (r[k] >= decoded.size()) decoded.resize(r[k] + 1, 0);
                if (!decoded[r[k]]) {
                    decoded[r[k]] = 1;
                    m.walk_v.push_back(r[k]);
                    m.walk_para.push_back(0);
                    m.walk_ref.insert(m.walk_ref.end(), {0, 0, 0});
                }
            }
            q0 = r[0]; q1 = r[1]; q2 = r[2];
            for (uint32_t j = 1; j < m.strip_lens[s]; j++, i++) {
                uint32_t ec = (tok_meta[i] >> 16) - 1;
                uint32_t nvl = local_of(order_g[i]);
                m.tokens.push_back(((ec + 1) << 16) | nvl);
                uint32_t a, b, c;
                if (ec == 0) { a = q1; b = q2; c = q0; } else { a = q0; b = q2; c = q1; }
                if (nvl >= decoded.size()) decoded.resize(nvl + 1, 0);
                if (!decoded[nvl]) {
                    decoded[nvl] = 1;
                    m.walk_v.push_back(nvl);
                    m.walk_para.push_back(1);
                    m.walk_ref.insert(m.walk_ref.end(), {a, b, c});
                }
                q0 = a; q1 = b; q2 = nvl;
            }
        }
        return m;
    }
};

inline int64_t irlp(const int64_t* n, int K, int64_t a, int64_t b, int64_t c) {
    __int128 s = static_cast<__int128>(n[0]) * a + static_cast<__int128>(n[1]) * b + static_cast<__int128>(n[2]) * c;
    if (K) s = (s + (static_cast<__int128>(1) << (K - 1))) >> K;
    return static_cast<int64_t>(s);
}

// Normalisation and global quantisation (prepare_paradelta_arrays,
// encoder/paradelta_codec.py:767-786, and _quantize_global, :149-165).
struct Quant {
    double center[3] = {0, 0, 0}, scale = 1.0, pce = 0.0, gmin[3], grange[3];
    uint32_t g_bits[3] = {0, 0, 0};
    std::vector<int32_t> gcodes;  // n_v x 3
};

// 0, or -2 with g_err set when an axis needs more than 24 bits.
int quantize(const double* verts, uint64_t n_v, double precision_error, int precision_mode, Quant& Q) {
    double* center = Q.center;
    for (uint64_t i = 0; i < n_v; i++)
        for (int d = 0; d < 3; d++) center[d] += verts[3 * i + d];
    for (int d = 0; d < 3; d++) center[d] /= static_cast<double>(n_v);
    double scale = 0, bmin[3], bmax[3];
    for (int d = 0; d < 3; d++) { bmin[d] = INFINITY; bmax[d] = -INFINITY; }
    for (uint64_t i = 0; i < n_v; i++) {
        double s = 0;
        for (int d = 0; d < 3; d++) {
            double x = verts[3 * i + d];
            bmin[d] = std::min(bmin[d], x);
            bmax[d] = std::max(bmax[d], x);
            double c = x - center[d];
            s += c * c;
        }
        scale = std::max(scale, std::sqrt(s));
    }
    if (!(scale > 0)) scale = 1.0;
    Q.scale = scale;
    if (precision_mode == 0) {
        Q.pce = precision_error / scale / std::sqrt(3.0);
    } else {
        double ext = std::max(bmax[0] - bmin[0], std::max(bmax[1] - bmin[1], bmax[2] - bmin[2]));
        Q.pce = (precision_error * ext) / (2.0 * scale);
    }
    Q.gcodes.assign(3 * n_v, 0);
    for (int d = 0; d < 3; d++) {
        double lo = INFINITY, hi = -INFINITY;
        for (uint64_t i = 0; i < n_v; i++) {
            double x = (verts[3 * i + d] - center[d]) / scale;
            lo = std::min(lo, x);
            hi = std::max(hi, x);
        }
        Q.gmin[d] = lo;
        Q.grange[d] = hi - lo;
        double step = 2.0 * Q.pce;
        if (!(Q.grange[d] > 0)) { Q.g_bits[d] = 1; continue; }
        int nb = std::max(1, static_cast<int>(std::ceil(std::log2(Q.grange[d] / step + 1.0))));
        if (nb > 24) { g_err = "precision needs more than 24 bits per axis"; return -2; }
        Q.g_bits[d] = static_cast<uint32_t>(nb);
        double mx = static_cast<double>((1u << nb) - 1u);
        for (uint64_t i = 0; i < n_v; i++) {
            double x = ((verts[3 * i + d] - center[d]) / scale - Q.gmin[d]) / Q.grange[d] * mx;
            double q = std::nearbyint(x);  // round half to even, like np.round
            q = std::min(std::max(q, 0.0), mx);
            Q.gcodes[3 * i + d] = static_cast<int32_t>(q);
        }
    }
    return 0;
}

struct Result {
    std::vector<uint8_t> data;
    std::vector<uint32_t> l2g;
    std::vector<int32_t> codes;  // n_dup x 3, decode order
    uint32_t n_meshlets = 0;
    uint32_t g_bits[3] = {0, 0, 0};
    int32_t pred_n[9];
    uint32_t pred_k[3];
};

// A PLDT v5 encode: the stream and, per decoded row, its source vertex.
struct Result5 {
    std::vector<uint8_t> data;
    std::vector<uint32_t> rows;
    uint32_t n_meshlets = 0, n_boundary = 0;
};

int best_rice_k(const std::vector<uint64_t>& u, int kmax) {
    uint64_t best = ~0ull;
    int k = 0;
    for (int kk = 0; kk <= kmax; kk++) {
        const uint64_t b = rice_bits(u, kk);
        if (b < best) { best = b; k = kk; }
    }
    return k;
}

inline uint32_t f32bits(double x) {
    const float f = static_cast<float>(x);
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}

}  // namespace

extern "C" {

struct stride_encode_opts {
    int32_t max_verts;        // <= 256 for the GPU decoder
    int32_t max_tris;         // <= 256 for the GPU decoder
    double precision_error;
    int32_t precision_mode;   // 0 = world, 1 = bbox_frac
    int32_t predictor;        // 0 = canonical, 1 = fitted
};

const char* stride_encode_last_error(void) { return g_err.c_str(); }

int stride_encode(const double* verts, uint64_t n_v, const int64_t* tris, uint64_t n_t,
                  const stride_encode_opts* o, void** out) {
    try {
        if (!verts || !tris || !o || !out || n_v == 0 || n_t == 0) { g_err = "bad arguments"; return -1; }
        if (o->max_verts < 3 || o->max_verts > 65535 || o->max_tris < 1 || o->max_tris > 65535) {
            g_err = "max_verts/max_tris out of range"; return -1;
        }
        for (uint64_t i = 0; i < 3 * n_t; i++)
            if (tris[i] < 0 || static_cast<uint64_t>(tris[i]) >= n_v) { g_err = "triangle index out of range"; return -1; }
        Quant Q;
        if (quantize(verts, n_v, o->precision_error, o->precision_mode, Q)) return -2;
        Result* R = new Result();
        for (int d = 0; d < 3; d++) R->g_bits[d] = Q.g_bits[d];
        const double* center = Q.center;
        const double scale = Q.scale, pce = Q.pce;
        const double* gmin = Q.gmin;
        const double* grange = Q.grange;
        const std::vector<int32_t>& gcodes = Q.gcodes;
        // ---- partition + strips
        Encoder E{verts, n_v, tris, n_t, o->max_verts, o->max_tris, {}, {}, {}, 0};
        E.lmap.assign(n_v, -1);
        E.lstamp.assign(n_v, -1);
        E.build_adjacency();
        std::vector<std::vector<uint32_t>> parts = E.partition();
        std::vector<Meshlet> ms;
        ms.reserve(parts.size());
        std::vector<int32_t> tri_local(n_t, -1);
        for (auto& p : parts) ms.push_back(E.strips(p, tri_local));
        R->n_meshlets = static_cast<uint32_t>(ms.size());
        // ---- predictor
        int64_t pn[9] = {1, 1, -1, 1, 1, -1, 1, 1, -1};
        int pk[3] = {0, 0, 0};
        if (o->predictor == 1) {
            // per-axis least squares of v ~ w0 a + w1 b + w2 c over para vertices
            double A[3][9] = {}, Bv[3][3] = {};
            std::vector<int64_t> sa, sb, sc, sv;
            uint64_t cnt = 0;
            for (auto& m : ms) {
                for (size_t w = 0; w < m.walk_v.size(); w++) {
                    if (!m.walk_para[w]) continue;
                    cnt++;
                    if (sv.size() < 3u * 400000u) {
                        for (int d = 0; d < 3; d++) {
                            sa.push_back(gcodes[3 * m.l2g[m.walk_ref[3 * w]] + d]);
                            sb.push_back(gcodes[3 * m.l2g[m.walk_ref[3 * w + 1]] + d]);
                            sc.push_back(gcodes[3 * m.l2g[m.walk_ref[3 * w + 2]] + d]);
                            sv.push_back(gcodes[3 * m.l2g[m.walk_v[w]] + d]);
                        }
                    }
                }
            }
            size_t ns = sv.size() / 3;
            for (int d = 0; d < 3 && ns >= 16; d++) {
                for (size_t i = 0; i < ns; i++) {
                    double x[3] = {static_cast<double>(sa[3 * i + d]), static_cast<double>(sb[3 * i + d]),
                                   static_cast<double>(sc[3 * i + d])};
                    double y = static_cast<double>(sv[3 * i + d]);
                    for (int r = 0; r < 3; r++) {
                        for (int c = 0; c < 3; c++) A[d][3 * r + c] += x[r] * x[c];
                        Bv[d][r] += x[r] * y;
                    }
                }
                // solve 3x3 (Cramer) with a ridge toward canonical weights
                double M[9], rhs[3];
                for (int i = 0; i < 9; i++) M[i] = A[d][i];
                const double canon[3] = {1, 1, -1};
                double ridge = 1e-9 * (M[0] + M[4] + M[8]) + 1e-12;
                for (int i = 0; i < 3; i++) { M[4 * i] += ridge; rhs[i] = Bv[d][i] + ridge * canon[i]; }
                auto det3 = [](const double* m) {
                    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                           m[2] * (m[3] * m[7] - m[4] * m[6]);
                };
                double D = det3(M);
                double w[3] = {1, 1, -1};
                if (std::fabs(D) > 0) {
                    for (int c = 0; c < 3; c++) {
                        double Mc[9];
                        std::memcpy(Mc, M, sizeof(Mc));
                        for (int r = 0; r < 3; r++) Mc[3 * r + c] = rhs[r];
                        w[c] = det3(Mc) / D;
                    }
                }
                auto cost = [&](const int64_t* n3, int K) {
                    uint64_t bits = 0;
                    for (size_t i = 0; i < ns; i++) {
                        int64_t p = irlp(n3, K, sa[3 * i + d], sb[3 * i + d], sc[3 * i + d]);
                        bits += 2 * bitlen64(zigzag(sv[3 * i + d] - p)) + 1;
                    }
                    return bits;
                };
                int64_t bestn[3] = {1, 1, -1};
                int bestK = 0;
                uint64_t bestc = cost(bestn, 0);
                for (int K = 5; K <= 9; K++) {
                    int64_t n3[3];
                    bool ok = true;
                    for (int j = 0; j < 3; j++) {
                        double v = std::nearbyint(w[j] * static_cast<double>(1 << K));
                        if (!(std::fabs(v) < 32767)) ok = false;
                        n3[j] = static_cast<int64_t>(v);
                    }
                    if (!ok) continue;
                    uint64_t c = cost(n3, K);
                    if (c < bestc) { bestc = c; bestK = K; std::memcpy(bestn, n3, sizeof(n3)); }
                }
                for (int j = 0; j < 3; j++) pn[3 * d + j] = bestn[j];
                pk[d] = bestK;
            }
            (void)cnt;
        }
        for (int i = 0; i < 9; i++) R->pred_n[i] = static_cast<int32_t>(pn[i]);
        for (int d = 0; d < 3; d++) R->pred_k[d] = static_cast<uint32_t>(pk[d]);
        // ---- meshlet bodies (_write_meshlet_dup, paradelta_v5_dup.py:239-313)
        BitWriter body;
        std::vector<uint64_t> offs;
        offs.reserve(ms.size());
        uint64_t total_local = 0, max_abs = 0;
        std::vector<uint64_t> streams[6];
        for (auto& m : ms) {
            offs.push_back(body.bitpos());
            const uint32_t n_local = static_cast<uint32_t>(m.l2g.size());
            total_local += n_local;
            int idx_bits = std::max(1, bitlen64(n_local));
            body.put(n_local, 16);
            body.put(m.n_tris, 16);
            body.put(m.strip_lens.size(), 16);
            int fifo[kFifo];
            int flen = 0;
            size_t ti = 0;
            for (size_t s = 0; s < m.strip_lens.size(); s++) {
                body.put(m.strip_lens[s], 16);
                uint32_t ntok = 3 + (m.strip_lens[s] - 1u);
                for (uint32_t j = 0; j < ntok; j++, ti++) {
                    uint32_t tk = m.tokens[ti];
                    int v = static_cast<int>(tk & 0xFFFFu);
                    if (j >= 3) body.put((tk >> 16) & 0xFF ? ((tk >> 16) & 0xFF) - 1 : 0, 1);
                    int at = -1;
                    for (int q = 0; q < flen; q++) if (fifo[q] == v) { at = q; break; }
                    if (at >= 0) { body.put(0, 1); body.put(static_cast<uint64_t>(at), kReuseBits); }
                    else { body.put(1, 1); body.put(static_cast<uint64_t>(v), idx_bits); }
                    if (at >= 0) { std::memmove(&fifo[at], &fifo[at + 1], (flen - at - 1) * sizeof(int)); flen--; }
                    else if (flen == kFifo) { std::memmove(&fifo[0], &fifo[1], (kFifo - 1) * sizeof(int)); flen--; }
                    fifo[flen++] = v;
                }
            }
            // residuals in walk order
            for (auto& st : streams) st.clear();
            int64_t prev[3] = {0, 0, 0};
            int64_t anchor[3] = {0, 0, 0};
            bool first = true;
            for (size_t w = 0; w < m.walk_v.size(); w++) {
                const int32_t* tc = &gcodes[3 * m.l2g[m.walk_v[w]]];
                if (!m.walk_para[w]) {
                    if (first) { for (int d = 0; d < 3; d++) anchor[d] = tc[d]; first = false; }
                    else for (int d = 0; d < 3; d++) {
                        int64_t r = tc[d] - prev[d];
                        max_abs = std::max<uint64_t>(max_abs, static_cast<uint64_t>(r < 0 ? -r : r));
                        streams[d].push_back(zigzag(r));
                    }
                } else {
                    for (int d = 0; d < 3; d++) {
                        int64_t p = irlp(&pn[3 * d], pk[d], gcodes[3 * m.l2g[m.walk_ref[3 * w]] + d],
                                         gcodes[3 * m.l2g[m.walk_ref[3 * w + 1]] + d],
                                         gcodes[3 * m.l2g[m.walk_ref[3 * w + 2]] + d]);
                        int64_t r = tc[d] - p;
                        max_abs = std::max<uint64_t>(max_abs, static_cast<uint64_t>(r < 0 ? -r : r));
                        streams[3 + d].push_back(zigzag(r));
                    }
                }
                for (int d = 0; d < 3; d++) prev[d] = tc[d];
            }
            for (int d = 0; d < 3; d++) body.put(static_cast<uint64_t>(anchor[d]), static_cast<int>(R->g_bits[d]));
            int tag[6], kk[6];
            for (int s = 0; s < 6; s++) pick_tag_k(streams[s], &tag[s], &kk[s]);
            for (int s = 0; s < 6; s++) { body.put(tag[s], 8); body.put(kk[s], 8); }
            for (int s = 0; s < 6; s++)
                for (uint64_t u : streams[s]) {
                    if (tag[s] == 1) body.rice(u, kk[s]); else body.eg(u, kk[s]);
                }
            for (uint32_t v = 0; v < n_local; v++) {
                R->l2g.push_back(m.l2g[v]);
                for (int d = 0; d < 3; d++) R->codes.push_back(gcodes[3 * m.l2g[v] + d]);
            }
        }
        std::vector<uint8_t> body_bytes = body.finish();
        // ---- global header + offset table (paradelta_v5_dup.py:412-447)
        BitWriter h;
        auto f32bits = [](double x) { float f = static_cast<float>(x); uint32_t b; std::memcpy(&b, &f, 4); return b; };
        h.put(kMagic, 32);
        h.put(kVersion, 8);
        h.put(max_abs > 32767 ? 1 : 0, 8);
        for (int d = 0; d < 3; d++) h.put(f32bits(center[d]), 32);
        h.put(f32bits(scale), 32);
        h.put(f32bits(pce), 32);
        for (int d = 0; d < 3; d++) h.put(f32bits(gmin[d]), 32);
        for (int d = 0; d < 3; d++) h.put(f32bits(grange[d]), 32);
        for (int d = 0; d < 3; d++) h.put(R->g_bits[d], 8);
        for (int i = 0; i < 9; i++) h.put(static_cast<uint64_t>(pn[i]) & 0xFFFFu, 16);
        for (int d = 0; d < 3; d++) h.put(static_cast<uint64_t>(pk[d]) & 0xFFu, 8);
        if (total_local > 0xFFFFFFFFull || n_t > 0xFFFFFFFFull) { delete R; g_err = "mesh too large for u32 header counts"; return -3; }
        h.put(total_local, 32);
        h.put(n_t, 32);
        h.put(ms.size(), 32);
        uint64_t start = h.bitpos() + 32ull * ms.size();
        if (start + body_bytes.size() * 8ull > 0xFFFFFFFFull) { delete R; g_err = "blob exceeds 32-bit bit offsets"; return -3; }
        for (uint64_t off : offs) h.put(start + off, 32);
        R->data = h.finish();
        R->data.insert(R->data.end(), body_bytes.begin(), body_bytes.end());
        *out = R;
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -4;
    }
}

// PLDT v5 (the reference's CuPy decoder format, written by
// encode_from_prepared_v5, encoder/paradelta_v5.py:144-279, and read by
// decode_paradelta_v5, :286-462) from the same partition, strips and
// quantisation: vertices used by more than one meshlet form the global
// boundary table; a meshlet numbers its boundary vertices first (by
// boundary index), then its interior vertices; interior residuals follow
// the decoder's float64 reconstruction (canonical lin3 weights 1, 1, -1,
// boundary mean for strip roots), so every decoded interior position lies
// within half a step (2 * per_coord_err) of its normalised source position.
int pldt5_encode(const double* verts, uint64_t n_v, const int64_t* tris, uint64_t n_t,
                 const stride_encode_opts* o, void** out) {
    try {
        if (!verts || !tris || !o || !out || n_v == 0 || n_t == 0) { g_err = "bad arguments"; return -1; }
        if (o->max_verts < 3 || o->max_verts > 65535 || o->max_tris < 1 || o->max_tris > 65535) {
            g_err = "max_verts/max_tris out of range"; return -1;
        }
        for (uint64_t i = 0; i < 3 * n_t; i++)
            if (tris[i] < 0 || static_cast<uint64_t>(tris[i]) >= n_v) { g_err = "triangle index out of range"; return -1; }
        Quant Q;
        if (quantize(verts, n_v, o->precision_error, o->precision_mode, Q)) return -2;
        Encoder E{verts, n_v, tris, n_t, o->max_verts, o->max_tris, {}, {}, {}, 0};
        E.lmap.assign(n_v, -1);
        E.lstamp.assign(n_v, -1);
        E.build_adjacency();
        std::vector<std::vector<uint32_t>> parts = E.partition();
        std::vector<Meshlet> ms;
        ms.reserve(parts.size());
        std::vector<int32_t> tri_local(n_t, -1);
        for (auto& p : parts) ms.push_back(E.strips(p, tri_local));
        // boundary: vertices of more than one meshlet
        std::vector<uint32_t> cnt(n_v, 0);
        for (auto& m : ms)
            for (uint32_t g : m.l2g) cnt[g]++;
        std::vector<int64_t> bidx(n_v, -1);
        std::vector<uint32_t> blist;
        for (uint64_t g = 0; g < n_v; g++)
            if (cnt[g] >= 2) { bidx[g] = static_cast<int64_t>(blist.size()); blist.push_back(static_cast<uint32_t>(g)); }
        const uint64_t nb = blist.size();
        // header values as the decoder reads them (f32)
        double c32[3], gmin32[3], grange32[3];
        for (int d = 0; d < 3; d++) {
            c32[d] = static_cast<float>(Q.center[d]);
            gmin32[d] = static_cast<float>(Q.gmin[d]);
            grange32[d] = static_cast<float>(Q.grange[d]);
        }
        const double scale32 = static_cast<float>(Q.scale);
        const double delta = 2.0 * static_cast<double>(static_cast<float>(Q.pce));
        const double w0 = 1.0, w1 = 1.0, w2 = -1.0;
        auto code_of = [&](uint64_t g, int d) { return static_cast<int64_t>(Q.gcodes[3 * g + d]); };
        // boundary rows: g_min + code / mx * g_range (decode_paradelta_v5, :322-336)
        std::vector<double> brow(3 * nb);
        for (uint64_t b = 0; b < nb; b++)
            for (int d = 0; d < 3; d++) {
                const uint64_t mx = (1ull << Q.g_bits[d]) - 1ull;
                brow[3 * b + d] = mx == 0 ? gmin32[d]
                                          : gmin32[d] + (static_cast<double>(code_of(blist[b], d)) /
                                                         static_cast<double>(mx)) * grange32[d];
            }
        Result5* R = new Result5();
        R->n_meshlets = static_cast<uint32_t>(ms.size());
        R->n_boundary = static_cast<uint32_t>(nb);
        R->rows.assign(blist.begin(), blist.end());
        BitWriter body;
        std::vector<uint64_t> offs;
        uint64_t max_abs = 0;
        for (auto& m : ms) {
            offs.push_back(body.bitpos());
            const uint32_t nl = static_cast<uint32_t>(m.l2g.size());
            std::vector<uint32_t> bl, il;  // old local ids of boundary / interior vertices
            for (uint32_t l = 0; l < nl; l++) (bidx[m.l2g[l]] >= 0 ? bl : il).push_back(l);
            std::sort(bl.begin(), bl.end(), [&](uint32_t x, uint32_t y) { return bidx[m.l2g[x]] < bidx[m.l2g[y]]; });
            std::vector<uint32_t> nid(nl);
            for (size_t i = 0; i < bl.size(); i++) nid[bl[i]] = static_cast<uint32_t>(i);
            for (size_t i = 0; i < il.size(); i++) nid[il[i]] = static_cast<uint32_t>(bl.size() + i);
            const uint32_t n_bnd = static_cast<uint32_t>(bl.size()), n_int = static_cast<uint32_t>(il.size());
            body.put(n_bnd, 16);
            body.put(n_int, 16);
            body.put(m.n_tris, 16);
            body.put(m.strip_lens.size(), 16);
            if (n_bnd) {  // boundary references: first, then gaps minus one (:350-361)
                body.put(static_cast<uint64_t>(bidx[m.l2g[bl[0]]]), 32);
                if (n_bnd > 1) {
                    std::vector<uint64_t> gaps;
                    for (size_t i = 1; i < bl.size(); i++)
                        gaps.push_back(static_cast<uint64_t>(bidx[m.l2g[bl[i]]] - bidx[m.l2g[bl[i - 1]]] - 1));
                    const int k = best_rice_k(gaps, 11);
                    body.put(k, 8);
                    for (uint64_t u : gaps) body.rice(u, k);
                }
            }
            // strips and tokens (new ids), the decoder's first-reach order
            const int idx_bits = std::max(1, bitlen64(nl));
            int fifo[kFifo];
            int flen = 0;
            std::vector<uint8_t> seen(nl, 0);
            for (uint32_t l = 0; l < n_bnd; l++) seen[l] = 1;
            struct Emit { uint32_t v; bool para; uint32_t a, b, c; };
            std::vector<Emit> emit;
            auto token = [&](int v) {
                int at = -1;
                for (int q = 0; q < flen; q++) if (fifo[q] == v) { at = q; break; }
                if (at >= 0) { body.put(0, 1); body.put(static_cast<uint64_t>(at), kReuseBits); }
                else { body.put(1, 1); body.put(static_cast<uint64_t>(v), idx_bits); }
                if (at >= 0) { std::memmove(&fifo[at], &fifo[at + 1], (flen - at - 1) * sizeof(int)); flen--; }
                else if (flen == kFifo) { std::memmove(&fifo[0], &fifo[1], (kFifo - 1) * sizeof(int)); flen--; }
                fifo[flen++] = v;
            };
            size_t ti = 0;
            for (size_t s = 0; s < m.strip_lens.size(); s++) {
                body.put(m.strip_lens[s], 16);
                uint32_t r[3];
                for (int k = 0; k < 3; k++, ti++) {
                    r[k] = nid[m.tokens[ti] & 0xFFFFu];
                    token(static_cast<int>(r[k]));
                }
                for (int k = 0; k < 3; k++) {
                    if (r[k] >= n_bnd && !seen[r[k]]) emit.push_back({r[k], false, 0, 0, 0});
                    seen[r[k]] = 1;
                }
                uint32_t q0 = r[0], q1 = r[1], q2 = r[2];
                for (uint32_t j = 1; j < m.strip_lens[s]; j++, ti++) {
                    const uint32_t tk = m.tokens[ti];
                    const uint32_t ec = ((tk >> 16) & 0xFFu) - 1u;
                    const uint32_t v = nid[tk & 0xFFFFu];
                    body.put(ec, 1);
                    token(static_cast<int>(v));
                    uint32_t a, b, c;
                    if (ec == 0) { a = q1; b = q2; c = q0; } else { a = q0; b = q2; c = q1; }
                    if (v >= n_bnd && !seen[v]) emit.push_back({v, true, a, b, c});
                    seen[v] = 1;
                    q0 = a; q1 = b; q2 = v;
                }
            }
            if (emit.size() != n_int) { delete R; g_err = "an interior vertex is in no strip"; return -3; }
            // residual codes from the decoder's reconstruction (:426-445)
            if (n_int) {
                std::vector<double> recon(3 * static_cast<size_t>(nl), 0.0);
                for (uint32_t l = 0; l < n_bnd; l++)
                    for (int d = 0; d < 3; d++) recon[3 * l + d] = brow[3 * bidx[m.l2g[bl[l]]] + d];
                double fb[3] = {0.0, 0.0, 0.0};
                if (n_bnd) {
                    for (int d = 0; d < 3; d++) {
                        double sum = recon[d];
                        for (uint32_t l = 1; l < n_bnd; l++) sum = sum + recon[3 * l + d];
                        fb[d] = sum / static_cast<double>(n_bnd);
                    }
                }
                std::vector<int64_t> codes(3 * static_cast<size_t>(n_int));
                for (size_t i = 0; i < emit.size(); i++) {
                    const Emit& e = emit[i];
                    const uint64_t g = m.l2g[il[e.v - n_bnd]];
                    for (int d = 0; d < 3; d++) {
                        double pred = fb[d];
                        if (e.para) {
                            const double t0 = w0 * recon[3 * e.a + d], t1 = w1 * recon[3 * e.b + d];
                            const double t2 = w2 * recon[3 * e.c + d];
                            pred = (t0 + t1) + t2;
                        }
                        const double target = (verts[3 * g + d] - c32[d]) / scale32;
                        const double cd = std::nearbyint((target - pred) / delta);
                        if (!(std::fabs(cd) < 1e15)) { delete R; g_err = "residual out of range"; return -3; }
                        const int64_t code = static_cast<int64_t>(cd);
                        codes[3 * i + d] = code;
                        max_abs = std::max<uint64_t>(max_abs, static_cast<uint64_t>(code < 0 ? -code : code));
                        recon[3 * e.v + d] = pred + static_cast<double>(code) * delta;
                    }
                }
                for (int d = 0; d < 3; d++) {  // per axis: fixed width, Rice or Exp-Golomb, the smallest
                    int64_t mn = codes[d], mxv = codes[d];
                    std::vector<uint64_t> u(n_int);
                    for (uint32_t i = 0; i < n_int; i++) {
                        mn = std::min(mn, codes[3 * i + d]);
                        mxv = std::max(mxv, codes[3 * i + d]);
                        u[i] = zigzag(codes[3 * i + d]);
                    }
                    const int bw = std::max(1, bitlen64(static_cast<uint64_t>(mxv - mn)));
                    uint64_t best = (mn >= -32768 && mn <= 32767 && bw <= 32) ? 32ull + n_int * static_cast<uint64_t>(bw) : ~0ull;
                    int tag = 0, k = 0;
                    const int kr = best_rice_k(u, 11);
                    if (16 + rice_bits(u, kr) < best) { best = 16 + rice_bits(u, kr); tag = 1; k = kr; }
                    for (int kk = 0; kk <= 7; kk++)
                        if (16 + eg_bits(u, kk) < best) { best = 16 + eg_bits(u, kk); tag = 2; k = kk; }
                    body.put(tag, 8);
                    if (tag == 0) {
                        body.put(static_cast<uint64_t>(mn) & 0xFFFFu, 16);
                        body.put(bw, 8);
                        for (uint32_t i = 0; i < n_int; i++) body.put(static_cast<uint64_t>(codes[3 * i + d] - mn), bw);
                    } else {
                        body.put(k, 8);
                        for (uint64_t x : u) { if (tag == 1) body.rice(x, k); else body.eg(x, k); }
                    }
                }
            }
            for (uint32_t i = 0; i < n_int; i++) R->rows.push_back(m.l2g[il[i]]);
        }
        std::vector<uint8_t> body_bytes = body.finish();
        // global header (:228-250) and boundary table (:252-264)
        BitWriter h;
        h.put(0x504C4454u, 32);
        h.put(5, 8);
        h.put(max_abs > 32767 ? 1 : 0, 8);
        for (int d = 0; d < 3; d++) h.put(f32bits(Q.center[d]), 32);
        h.put(f32bits(Q.scale), 32);
        h.put(f32bits(Q.pce), 32);
        for (int d = 0; d < 3; d++) h.put(f32bits(Q.gmin[d]), 32);
        for (int d = 0; d < 3; d++) h.put(f32bits(Q.grange[d]), 32);
        for (int d = 0; d < 3; d++) h.put(Q.g_bits[d], 8);
        if (n_v > 0xFFFFFFFFull || n_t > 0xFFFFFFFFull) { delete R; g_err = "mesh too large for u32 header counts"; return -3; }
        h.put(n_v, 32);
        h.put(n_t, 32);
        h.put(nb, 32);
        h.put(ms.size(), 32);
        h.put(f32bits(w0), 32);
        h.put(f32bits(w1), 32);
        h.put(f32bits(w2), 32);
        for (int d = 0; d < 3 && nb > 0; d++) {
            h.put(static_cast<uint64_t>(code_of(blist[0], d)), static_cast<int>(Q.g_bits[d]));
            if (nb > 1) {
                std::vector<uint64_t> u;
                u.reserve(nb - 1);
                for (uint64_t b = 1; b < nb; b++) u.push_back(zigzag(code_of(blist[b], d) - code_of(blist[b - 1], d)));
                const int k = best_rice_k(u, 11);
                h.put(k, 8);
                for (uint64_t x : u) h.rice(x, k);
            }
        }
        h.put(0, static_cast<int>((8 - h.bitpos() % 8) % 8));
        const uint64_t start = h.bitpos() + 32ull * ms.size();
        if (start + body_bytes.size() * 8ull > 0xFFFFFFFFull) { delete R; g_err = "blob exceeds 32-bit bit offsets"; return -3; }
        for (uint64_t off : offs) h.put(start + off, 32);
        R->data = h.finish();
        R->data.insert(R->data.end(), body_bytes.begin(), body_bytes.end());
        *out = R;
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -4;
    }
}

uint64_t pldt5_encode_nbytes(void* r) { return static_cast<Result5*>(r)->data.size(); }
const uint8_t* pldt5_encode_bytes(void* r) { return static_cast<Result5*>(r)->data.data(); }
uint64_t pldt5_encode_n_rows(void* r) { return static_cast<Result5*>(r)->rows.size(); }
const uint32_t* pldt5_encode_rows(void* r) { return static_cast<Result5*>(r)->rows.data(); }
uint32_t pldt5_encode_n_meshlets(void* r) { return static_cast<Result5*>(r)->n_meshlets; }
uint32_t pldt5_encode_n_boundary(void* r) { return static_cast<Result5*>(r)->n_boundary; }
void pldt5_encode_free(void* r) { delete static_cast<Result5*>(r); }

uint64_t stride_encode_nbytes(void* r) { return static_cast<Result*>(r)->data.size(); }
const uint8_t* stride_encode_bytes(void* r) { return static_cast<Result*>(r)->data.data(); }
uint64_t stride_encode_n_dup(void* r) { return static_cast<Result*>(r)->l2g.size(); }
const uint32_t* stride_encode_l2g(void* r) { return static_cast<Result*>(r)->l2g.data(); }
const int32_t* stride_encode_codes(void* r) { return static_cast<Result*>(r)->codes.data(); }
uint32_t stride_encode_n_meshlets(void* r) { return static_cast<Result*>(r)->n_meshlets; }
void stride_encode_free(void* r) { delete static_cast<Result*>(r); }

}  // extern "C"
