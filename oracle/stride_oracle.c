/*
 * STRIDE (DPR4 v3) CPU oracle.  TEST INFRASTRUCTURE ONLY: the GPU decoder is
 * checked against it; only tests, the smoke check and the CPU-baseline leg of
 * bench.py load this library.  Nothing in the product path calls it.
 *
 * A C restatement of the reference CPU decoder
 *   decode_dup                     encoder/paradelta_v5_dup.py:471-618
 * and the helpers it calls
 *   BitReader.read_bits/_rice/_exp_golomb/_f32   utils/bit_codec.py:192-254
 *   _read_vert (+ 16-entry move-to-tail FIFO)    encoder/paradelta_codec.py:330-340
 *   _idx_bits_for, _REUSE_BITS                   encoder/paradelta_codec.py:124-128
 *   _irlp_pred                                   encoder/paradelta_v5_dup.py:91-104
 *
 * Semantics kept from the Python original:
 *   - every field is MSB-first; reads past the end of the bytes fail;
 *   - a residual tag equal to 1 selects Rice, any other tag Exp-Golomb
 *     (paradelta_v5_dup.py:563-567);
 *   - strip_len 0 still reads three root tokens and emits one triangle;
 *   - local vertices never reached by the walk keep code 0;
 *   - residual/delta additions wrap like numpy int64; the IRLP sum is exact
 *     (Python int) and must fit int64 (numpy assignment, else OverflowError);
 *   - dequantisation is the float64 expression
 *       f32((g_min + code / mx * g_range) * scale + center),  mx = 2^g_bits - 1
 *     evaluated left to right without contraction (build with
 *     -ffp-contract=off); g_bits == 0 gives g_min.
 * Limits (the Python original has none; valid streams never come close):
 *   k <= 56 for residual codes, g_bits <= 32, pred_K <= 100.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "so_bits.h"

#define SO_MAGIC 0x44505234u
#define SO_VERSION 3u

typedef struct {
    uint32_t magic, version, code_width;
    float center[3], scale, per_coord_err, g_min[3], g_range[3];
    uint32_t g_bits[3];
    int32_t pred_n[9];
    uint32_t pred_k[3];
    uint32_t n_v_total, n_t, n_meshlets;
    uint64_t body_bit; /* first bit after the offset table */
} so_header;

const char* so_error(int code) {
    switch (code) {
    case SO_OK: return "ok";
    case SO_ERR_MAGIC: return "bad magic";
    case SO_ERR_VERSION: return "bad version";
    case SO_ERR_EOF: return "read past end of data";
    case SO_ERR_FIFO: return "FIFO index out of range";
    case SO_ERR_VERTEX: return "vertex id out of range";
    case SO_ERR_OVERFLOW: return "integer overflow";
    case SO_ERR_CAPACITY: return "output capacity too small";
    case SO_ERR_UNSUPPORTED: return "field outside the oracle's limits";
    case SO_ERR_LAYOUT: return "offset table inconsistent with meshlet payloads";
    case SO_ERR_NOMEM: return "out of memory";
    default: return "unknown error";
    }
}

/* ---- global header (paradelta_v5_dup.py:472-501) ------------------------ */
int so_parse_header(const uint8_t* data, uint64_t len, so_header* h) {
    so_br r = {data, len * 8ull, 0, 0};
    memset(h, 0, sizeof(*h));
    h->magic = (uint32_t)br_read(&r, 32);
    if (r.err) return r.err;
    if (h->magic != SO_MAGIC) return SO_ERR_MAGIC;
    h->version = (uint32_t)br_read(&r, 8);
    if (r.err) return r.err;
    if (h->version != SO_VERSION) return SO_ERR_VERSION;
    h->code_width = (uint32_t)br_read(&r, 8);
    for (int i = 0; i < 3; i++) h->center[i] = f32_from_bits((uint32_t)br_read(&r, 32));
    h->scale = f32_from_bits((uint32_t)br_read(&r, 32));
    h->per_coord_err = f32_from_bits((uint32_t)br_read(&r, 32));
    for (int i = 0; i < 3; i++) h->g_min[i] = f32_from_bits((uint32_t)br_read(&r, 32));
    for (int i = 0; i < 3; i++) h->g_range[i] = f32_from_bits((uint32_t)br_read(&r, 32));
    for (int i = 0; i < 3; i++) h->g_bits[i] = (uint32_t)br_read(&r, 8);
    for (int i = 0; i < 9; i++) {
        uint32_t v = (uint32_t)br_read(&r, 16);
        h->pred_n[i] = (v & 0x8000u) ? (int32_t)v - 0x10000 : (int32_t)v;
    }
    for (int i = 0; i < 3; i++) h->pred_k[i] = (uint32_t)br_read(&r, 8);
    h->n_v_total = (uint32_t)br_read(&r, 32);
    h->n_t = (uint32_t)br_read(&r, 32);
    h->n_meshlets = (uint32_t)br_read(&r, 32);
    if (r.err) return r.err;
    uint64_t pad = (0 - r.pos) & 7u;
    r.pos += pad;
    h->body_bit = r.pos + 32ull * h->n_meshlets;
    if (h->body_bit > r.nbits) return SO_ERR_EOF;
    return SO_OK;
}

/* ---- one meshlet (paradelta_v5_dup.py:507-605) -------------------------- */
typedef struct {
    int32_t* stamp;   /* per local id: meshlet stamp when already decoded */
    int32_t stamp_id;
    uint32_t* walk_v; /* walk order */
    uint8_t* walk_para;
    uint32_t* walk_ref; /* 3 per entry */
    uint32_t* tris;     /* 3 per local triangle */
    int64_t* codes;     /* 3 per local vertex */
    int64_t* resid;     /* 3 per walk entry */
    uint64_t cap_walk, cap_tris;
} so_scratch;

static int scratch_grow(so_scratch* s, uint64_t walk, uint64_t tris) {
    if (walk > s->cap_walk) {
        uint64_t n = walk * 2;
        s->walk_v = (uint32_t*)realloc(s->walk_v, n * 4);
        s->walk_para = (uint8_t*)realloc(s->walk_para, n);
        s->walk_ref = (uint32_t*)realloc(s->walk_ref, n * 12);
        s->resid = (int64_t*)realloc(s->resid, n * 24);
        if (!s->walk_v || !s->walk_para || !s->walk_ref || !s->resid) return SO_ERR_NOMEM;
        s->cap_walk = n;
    }
    if (tris > s->cap_tris) {
        uint64_t n = tris * 2;
        s->tris = (uint32_t*)realloc(s->tris, n * 12);
        if (!s->tris) return SO_ERR_NOMEM;
        s->cap_tris = n;
    }
    return SO_OK;
}

static void scratch_free(so_scratch* s) {
    free(s->stamp); free(s->walk_v); free(s->walk_para); free(s->walk_ref);
    free(s->tris); free(s->codes); free(s->resid);
}

static int scratch_init(so_scratch* s) {
    memset(s, 0, sizeof(*s));
    s->stamp = (int32_t*)calloc(65536, sizeof(int32_t));
    s->codes = (int64_t*)malloc(65536ull * 3 * sizeof(int64_t));
    if (!s->stamp || !s->codes) return SO_ERR_NOMEM;
    return scratch_grow(s, 1024, 1024);
}

static double dequant(const so_header* h, int d, int64_t code) {
    double gmin = (double)h->g_min[d];
    double v;
    if (h->g_bits[d] == 0) {
        v = gmin;
    } else {
        double mx = (double)((1ull << h->g_bits[d]) - 1ull);
        double q = (double)code / mx;
        double t = q * (double)h->g_range[d];
        v = gmin + t;
    }
    double w = v * (double)h->scale;
    return w + (double)h->center[d];
}

/* Decode the meshlet whose header starts at r->pos.  Writes n_local positions
 * (and codes, if requested) at v_base and the emitted triangles at t_base.
 * Returns counts through n_local_out / n_tris_out. */
/* side (optional, 7 entries): the absolute bit of the anchor (start of the
 * residual part), the absolute starts of dy, dz, px, py, pz, and n_kind0.
 * pos == NULL decodes without writing outputs. */
static int decode_meshlet(so_br* r, const so_header* h, so_scratch* s,
                          uint64_t v_base, uint64_t t_base,
                          float* pos, int64_t* idx, int64_t* codes_out,
                          uint64_t cap_v, uint64_t cap_t,
                          uint32_t* n_local_out, uint64_t* n_tris_out, uint64_t* side) {
    uint32_t n_local = (uint32_t)br_read(r, 16);
    (void)br_read(r, 16); /* n_tris: not used by the reference decoder */
    uint32_t n_strips = (uint32_t)br_read(r, 16);
    if (r->err) return r->err;
    int idx_bits = bitlen(n_local);
    if (idx_bits < 1) idx_bits = 1;
    s->stamp_id++;
    if (s->stamp_id == 0x7fffffff) {
        memset(s->stamp, 0, 65536 * sizeof(int32_t));
        s->stamp_id = 1;
    }
    so_fifo fifo;
    fifo.len = 0;
    uint64_t n_walk = 0, n_tris = 0;
    uint64_t n_kind0 = 0, n_kind1 = 0;
    for (uint32_t st = 0; st < n_strips; st++) {
        uint32_t strip_len = (uint32_t)br_read(r, 16);
        if (r->err) return r->err;
        int rc = scratch_grow(s, n_walk + strip_len + 3, n_tris + strip_len + 1);
        if (rc) return rc;
        int v0, v1, v2;
        if ((rc = read_vert(r, &fifo, idx_bits, &v0))) return rc;
        if ((rc = read_vert(r, &fifo, idx_bits, &v1))) return rc;
        if ((rc = read_vert(r, &fifo, idx_bits, &v2))) return rc;
        uint32_t* t = &s->tris[3 * n_tris++];
        t[0] = (uint32_t)v0; t[1] = (uint32_t)v1; t[2] = (uint32_t)v2;
        int roots[3] = {v0, v1, v2};
        for (int i = 0; i < 3; i++) {
            int v = roots[i];
            if (s->stamp[v] != s->stamp_id) {
                s->stamp[v] = s->stamp_id;
                s->walk_v[n_walk] = (uint32_t)v;
                s->walk_para[n_walk] = 0;
                n_walk++;
                n_kind0++;
            }
        }
        int p0 = v0, p1 = v1, p2 = v2;
        for (uint32_t j = 1; j < strip_len; j++) {
            int ec = (int)br_read(r, 1);
            int nv;
            if ((rc = read_vert(r, &fifo, idx_bits, &nv))) return rc;
            int a, b, c;
            if (ec == 0) { a = p1; b = p2; c = p0; }
            else { a = p0; b = p2; c = p1; }
            t = &s->tris[3 * n_tris++];
            t[0] = (uint32_t)a; t[1] = (uint32_t)b; t[2] = (uint32_t)nv;
            if (s->stamp[nv] != s->stamp_id) {
                s->stamp[nv] = s->stamp_id;
                s->walk_v[n_walk] = (uint32_t)nv;
                s->walk_para[n_walk] = 1;
                s->walk_ref[3 * n_walk + 0] = (uint32_t)a;
                s->walk_ref[3 * n_walk + 1] = (uint32_t)b;
                s->walk_ref[3 * n_walk + 2] = (uint32_t)c;
                n_walk++;
                n_kind1++;
            }
            p0 = a; p1 = b; p2 = nv;
        }
    }
    if (side) side[0] = r->pos;
    /* anchor + (tag, k) headers */
    int64_t anchor[3];
    for (int d = 0; d < 3; d++) {
        if (h->g_bits[d] > 32) return SO_ERR_UNSUPPORTED;
        anchor[d] = (int64_t)br_read(r, (int)h->g_bits[d]);
    }
    int tags[6], ks[6];
    for (int i = 0; i < 6; i++) {
        tags[i] = (int)br_read(r, 8);
        ks[i] = (int)br_read(r, 8);
    }
    if (r->err) return r->err;
    uint64_t n_delta = n_kind0 > 0 ? n_kind0 - 1 : 0;
    /* residual substreams: dx, dy, dz, px, py, pz; stored per walk kind slot */
    int64_t* dres = s->resid;               /* n_delta x 3 */
    int64_t* pres = s->resid + 3 * n_delta; /* n_kind1 x 3 */
    if (side) side[6] = n_kind0;
    for (int sub = 0; sub < 6; sub++) {
        if (side && sub) side[sub] = r->pos;
        int d = sub % 3;
        uint64_t n = sub < 3 ? n_delta : n_kind1;
        int64_t* dst = sub < 3 ? dres : pres;
        for (uint64_t i = 0; i < n; i++) {
            uint64_t u = tags[sub] == 1 ? br_rice(r, ks[sub]) : br_eg(r, ks[sub]);
            if (r->err) return r->err;
            dst[3 * i + d] = unzigzag(u);
        }
    }
    /* IRLP reconstruction in walk order (paradelta_v5_dup.py:581-600) */
    if (n_local > 65536) return SO_ERR_UNSUPPORTED;
    int64_t* cl = s->codes;
    memset(cl, 0, (size_t)n_local * 3 * sizeof(int64_t));
    int first = 1;
    uint64_t di = 0, pi = 0;
    int64_t prev[3] = {0, 0, 0};
    for (uint64_t w = 0; w < n_walk; w++) {
        uint32_t v = s->walk_v[w];
        if (v >= n_local) return SO_ERR_VERTEX;
        int64_t* cv = &cl[3 * v];
        if (!s->walk_para[w]) {
            if (first) {
                cv[0] = anchor[0]; cv[1] = anchor[1]; cv[2] = anchor[2];
                first = 0;
            } else {
                for (int d = 0; d < 3; d++)
                    cv[d] = (int64_t)((uint64_t)prev[d] + (uint64_t)dres[3 * di + d]);
                di++;
            }
        } else {
            uint32_t a = s->walk_ref[3 * w], b = s->walk_ref[3 * w + 1], c = s->walk_ref[3 * w + 2];
            if (a >= n_local || b >= n_local || c >= n_local) return SO_ERR_VERTEX;
            for (int d = 0; d < 3; d++) {
                __int128 sum = (__int128)h->pred_n[3 * d] * cl[3 * a + d]
                             + (__int128)h->pred_n[3 * d + 1] * cl[3 * b + d]
                             + (__int128)h->pred_n[3 * d + 2] * cl[3 * c + d];
                uint32_t K = h->pred_k[d];
                if (K > 100) return SO_ERR_UNSUPPORTED;
                if (K) sum = (sum + ((__int128)1 << (K - 1))) >> K; /* floor shift */
                if (sum > (__int128)INT64_MAX || sum < (__int128)INT64_MIN) return SO_ERR_OVERFLOW;
                cv[d] = (int64_t)((uint64_t)(int64_t)sum + (uint64_t)pres[3 * pi + d]);
            }
            pi++;
        }
        prev[0] = cv[0]; prev[1] = cv[1]; prev[2] = cv[2];
    }
    if (!pos) {
        *n_local_out = n_local;
        *n_tris_out = n_tris;
        return SO_OK;
    }
    if (v_base + n_local > cap_v || t_base + n_tris > cap_t) return SO_ERR_CAPACITY;
    for (uint32_t v = 0; v < n_local; v++) {
        for (int d = 0; d < 3; d++) {
            pos[3 * (v_base + v) + d] = (float)dequant(h, d, cl[3 * v + d]);
            if (codes_out) codes_out[3 * (v_base + v) + d] = cl[3 * v + d];
        }
    }
    for (uint64_t t = 0; t < n_tris; t++)
        for (int k = 0; k < 3; k++)
            idx[3 * (t_base + t) + k] = (int64_t)(v_base + s->tris[3 * t + k]);
    *n_local_out = n_local;
    *n_tris_out = n_tris;
    return SO_OK;
}

/* Sequential decode, exactly the reference's control flow: meshlets are read
 * back to back from the first bit after the offset table. */
int so_decode(const uint8_t* data, uint64_t len, float* pos, int64_t* idx,
              int64_t* codes, uint64_t cap_v, uint64_t cap_t,
              uint64_t* n_v_out, uint64_t* n_t_out) {
    so_header h;
    int rc = so_parse_header(data, len, &h);
    if (rc) return rc;
    so_scratch s;
    if ((rc = scratch_init(&s))) { scratch_free(&s); return rc; }
    so_br r = {data, len * 8ull, h.body_bit, 0};
    uint64_t v_base = 0, t_base = 0;
    for (uint32_t m = 0; m < h.n_meshlets && !rc; m++) {
        uint32_t nl;
        uint64_t nt;
        rc = decode_meshlet(&r, &h, &s, v_base, t_base, pos, idx, codes, cap_v, cap_t, &nl, &nt, NULL);
        v_base += nl;
        t_base += nt;
    }
    scratch_free(&s);
    *n_v_out = v_base;
    *n_t_out = t_base;
    return rc;
}

/* ---- meshlet-parallel variant (CPU baseline) ----------------------------
 * Same per-meshlet decode, but every meshlet starts at its offset-table
 * entry, which lets threads take disjoint meshlet ranges.  Each meshlet must
 * end exactly where the next one starts, so the result equals the sequential
 * decode. */
typedef struct {
    const uint8_t* data;
    uint64_t len;
    const so_header* h;
    const uint64_t* off;
    const uint64_t* vb;
    const uint64_t* tb;
    uint32_t m0, m1;
    float* pos;
    int64_t* idx;
    uint64_t cap_v, cap_t;
    int rc;
} so_job;

static uint32_t be32(const uint8_t* p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

static void* so_worker(void* arg) {
    so_job* j = (so_job*)arg;
    so_scratch s;
    j->rc = scratch_init(&s);
    for (uint32_t m = j->m0; m < j->m1 && !j->rc; m++) {
        so_br r = {j->data, j->len * 8ull, j->off[m], 0};
        uint32_t nl;
        uint64_t nt;
        j->rc = decode_meshlet(&r, j->h, &s, j->vb[m], j->tb[m], j->pos, j->idx, NULL,
                               j->cap_v, j->cap_t, &nl, &nt, NULL);
        if (!j->rc && (j->vb[m] + nl != j->vb[m + 1] || j->tb[m] + nt != j->tb[m + 1]))
            j->rc = SO_ERR_LAYOUT;
        if (!j->rc && r.pos != j->off[m + 1]) {
            /* the last meshlet may be followed by < 8 zero pad bits */
            if (!(m + 1 == j->h->n_meshlets && j->off[m + 1] - r.pos < 8)) j->rc = SO_ERR_LAYOUT;
        }
    }
    scratch_free(&s);
    return NULL;
}

int so_decode_mt(const uint8_t* data, uint64_t len, float* pos, int64_t* idx,
                 uint64_t cap_v, uint64_t cap_t, int n_threads,
                 uint64_t* n_v_out, uint64_t* n_t_out) {
    so_header h;
    int rc = so_parse_header(data, len, &h);
    if (rc) return rc;
    uint32_t M = h.n_meshlets;
    uint64_t* off = (uint64_t*)malloc((M + 1) * sizeof(uint64_t));
    uint64_t* vb = (uint64_t*)malloc((M + 1) * sizeof(uint64_t));
    uint64_t* tb = (uint64_t*)malloc((M + 1) * sizeof(uint64_t));
    if (!off || !vb || !tb) { free(off); free(vb); free(tb); return SO_ERR_NOMEM; }
    uint64_t table = h.body_bit / 8 - 4ull * M;
    vb[0] = tb[0] = 0;
    for (uint32_t m = 0; m < M; m++) {
        off[m] = be32(data + table + 4ull * m);
        if (off[m] + 48 > len * 8ull || (m && off[m] < off[m - 1])) { rc = SO_ERR_LAYOUT; break; }
        so_br r = {data, len * 8ull, off[m], 0};
        uint32_t nl = (uint32_t)br_read(&r, 16);
        uint32_t nt = (uint32_t)br_read(&r, 16);
        vb[m + 1] = vb[m] + nl;
        tb[m + 1] = tb[m] + nt;
    }
    off[M] = len * 8ull;
    if (!rc) {
        if (n_threads < 1) n_threads = 1;
        if ((uint32_t)n_threads > M && M > 0) n_threads = (int)M;
        so_job* jobs = (so_job*)calloc((size_t)n_threads, sizeof(so_job));
        pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
        for (int i = 0; i < n_threads; i++) {
            jobs[i] = (so_job){data, len, &h, off, vb, tb,
                               (uint32_t)((uint64_t)M * i / n_threads),
                               (uint32_t)((uint64_t)M * (i + 1) / n_threads),
                               pos, idx, cap_v, cap_t, 0};
            pthread_create(&th[i], NULL, so_worker, &jobs[i]);
        }
        for (int i = 0; i < n_threads; i++) {
            pthread_join(th[i], NULL);
            if (jobs[i].rc && !rc) rc = jobs[i].rc;
        }
        free(jobs);
        free(th);
    }
    *n_v_out = vb[M];
    *n_t_out = tb[M];
    free(off); free(vb); free(tb);
    return rc;
}

/* Side table of the reference GPU bench's blob (DPRB v4, written by
 * scripts/dump_stride_dup_blob.py:104-160 from encoder metadata and read by
 * bench_cpp/stride_dup_decode_bench.cu:527-596), derived here from the DPR4
 * bytes alone: per meshlet its start bit, header counts, the bit where its
 * anchor (residual part) starts, n_kind0, and the starts of dy, dz, px, py,
 * pz relative to the anchor (paradelta_v5_dup.py:290-313).  All bit
 * positions are absolute in `data`. */
int so_side_table(const uint8_t* data, uint64_t len, uint64_t* start_bit, uint32_t* n_local,
                  uint32_t* n_tris, uint32_t* n_strips, uint64_t* resid_bit, uint32_t* n_kind0,
                  uint16_t* sub_offs) {
    so_header h;
    int rc = so_parse_header(data, len, &h);
    if (rc) return rc;
    so_scratch s;
    if ((rc = scratch_init(&s))) { scratch_free(&s); return rc; }
    so_br r = {data, len * 8ull, h.body_bit, 0};
    for (uint32_t m = 0; m < h.n_meshlets && !rc; m++) {
        uint64_t side[7] = {0, 0, 0, 0, 0, 0, 0};
        start_bit[m] = r.pos;
        so_br hr = r;
        n_local[m] = (uint32_t)br_read(&hr, 16);
        n_tris[m] = (uint32_t)br_read(&hr, 16);
        n_strips[m] = (uint32_t)br_read(&hr, 16);
        uint32_t nl;
        uint64_t nt;
        rc = decode_meshlet(&r, &h, &s, 0, 0, NULL, NULL, NULL, 0, 0, &nl, &nt, side);
        resid_bit[m] = side[0];
        n_kind0[m] = (uint32_t)side[6];
        for (int k = 0; k < 5 && !rc; k++) {
            const uint64_t d = side[1 + k] - side[0];
            if (d > 0xFFFFu) rc = SO_ERR_UNSUPPORTED; /* the blob stores them as u16 */
            sub_offs[5ull * m + k] = (uint16_t)d;
        }
    }
    scratch_free(&s);
    return rc;
}

/* Known-answer hook for the bit codec: read a sequence of fields
 * (kind 0 = fixed width k, 1 = Rice(k), 2 = Exp-Golomb(k)). */
int so_bitcodec_read(const uint8_t* data, uint64_t len, const int32_t* kinds,
                     const int32_t* ks, int32_t n, uint64_t* out) {
    so_br r = {data, len * 8ull, 0, 0};
    for (int i = 0; i < n; i++) {
        if (kinds[i] == 0) out[i] = br_read(&r, ks[i]);
        else if (kinds[i] == 1) out[i] = br_rice(&r, ks[i]);
        else out[i] = br_eg(&r, ks[i]);
        if (r.err) return r.err;
    }
    return SO_OK;
}
