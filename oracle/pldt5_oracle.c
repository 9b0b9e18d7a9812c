/*
 * PLDT v5 CPU oracle.  TEST INFRASTRUCTURE ONLY: the GPU decoder of this
 * format is checked against it; nothing in the product path calls it.
 *
 * A C restatement of the reference CPU decoder
 *   decode_paradelta_v5            encoder/paradelta_v5.py:286-462
 * (format written by encode_from_prepared_v5, encoder/paradelta_v5.py:144-279,
 * and read on the GPU by the reference's ParaDeltaV5GpuDecoder,
 * utils/paradelta_v5_cuda.py:515-718), with the helpers it calls
 *   MAGIC, REUSE_BUF_SIZE, _idx_bits_for, _read_vert
 *                                  encoder/paradelta_codec.py:101-128,330-340
 * and the bit reader of utils/bit_codec.py (so_bits.h).
 *
 * Semantics kept from the Python original:
 *   - every field is MSB-first; reads past the end of the bytes fail;
 *   - the boundary table is axis-major: per axis the first code (g_bits
 *     bits), then, for more than one boundary vertex, a Rice parameter (8
 *     bits) and zigzag Rice deltas; positions g_min + code / mx * g_range in
 *     float64 (g_bits == 0 gives g_min);
 *   - after byte alignment the offset table is skipped and meshlets are read
 *     back to back;
 *   - per meshlet: n_bnd, n_int, n_tris, n_strips (16 bits each); boundary
 *     references (32-bit first, then an 8-bit Rice parameter and deltas
 *     minus one); strips exactly as in the DPR4 decoder; interior vertices
 *     reached for the first time are decoded in that order; residual codes
 *     per axis with tag 0 (signed 16-bit minimum + fixed width), 1 (Rice)
 *     or 2 (Exp-Golomb), any other tag an error;
 *   - reconstruction in float64 without contraction (build with
 *     -ffp-contract=off): a strip-body vertex is
 *     (w0*a + w1*b) + w2*c, a root vertex the mean of the meshlet's boundary
 *     vertices (summed in order, divided by their count; 0 without any), plus
 *     code * (2 * per_coord_err);
 *   - interior vertices the walk never reaches stay at the normalised origin;
 *   - output rows: the boundary vertices, then each meshlet's interior
 *     vertices; positions f32(norm * scale + center); triangle indices
 *     global (int64).
 * Errors where the Python original raises (IndexError, KeyError, ValueError):
 * a FIFO index past the FIFO, a local id past the meshlet's vertices, a
 * boundary reference past the vertex rows so far, the meshlet's own interior
 * rows included (in a meshlet with interior vertices, whose reconstruction
 * reads them), more first-reached
 * interior vertices than codes, an unknown residual tag.
 * Limits (never approached by valid streams): fixed widths and Rice/EG
 * parameters of at most 56 bits.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "so_bits.h"

#define P5_MAGIC 0x504C4454u
#define P5_VERSION 5u

typedef struct {
    uint32_t magic, version, code_width;
    float center[3], scale, per_coord_err, g_min[3], g_range[3];
    uint32_t g_bits[3];
    uint32_t n_v, n_t, n_boundary, n_meshlets;
    float lin3_w[3];
    uint64_t boundary_bit; /* first bit of the boundary table */
} p5_header;

static float rd_f32(so_br* r) { return f32_from_bits((uint32_t)br_read(r, 32)); }

static int p5_header_read(so_br* r, p5_header* h) {
    memset(h, 0, sizeof(*h));
    h->magic = (uint32_t)br_read(r, 32);
    if (r->err) return r->err;
    if (h->magic != P5_MAGIC) return SO_ERR_MAGIC;
    h->version = (uint32_t)br_read(r, 8);
    if (r->err) return r->err;
    if (h->version != P5_VERSION) return SO_ERR_VERSION;
    h->code_width = (uint32_t)br_read(r, 8);
    for (int d = 0; d < 3; d++) h->center[d] = rd_f32(r);
    h->scale = rd_f32(r);
    h->per_coord_err = rd_f32(r);
    for (int d = 0; d < 3; d++) h->g_min[d] = rd_f32(r);
    for (int d = 0; d < 3; d++) h->g_range[d] = rd_f32(r);
    for (int d = 0; d < 3; d++) h->g_bits[d] = (uint32_t)br_read(r, 8);
    h->n_v = (uint32_t)br_read(r, 32);
    h->n_t = (uint32_t)br_read(r, 32);
    h->n_boundary = (uint32_t)br_read(r, 32);
    h->n_meshlets = (uint32_t)br_read(r, 32);
    for (int d = 0; d < 3; d++) h->lin3_w[d] = rd_f32(r);
    h->boundary_bit = r->pos;
    if (r->err) return r->err;
    for (int d = 0; d < 3; d++)
        if (h->g_bits[d] > 32) return SO_ERR_UNSUPPORTED;
    return SO_OK;
}

int p5_parse_header(const uint8_t* data, uint64_t len, p5_header* h) {
    so_br r = {data, len * 8ull, 0, 0};
    return p5_header_read(&r, h);
}

/* Growable float64 xyz rows and int64 triangles. */
typedef struct {
    double* v;
    uint64_t nv, capv;
    int64_t* t;
    uint64_t nt, capt;
} p5_out;

static int grow_v(p5_out* o, uint64_t need) {
    if (need <= o->capv) return SO_OK;
    uint64_t c = o->capv ? o->capv : 1024;
    while (c < need) c *= 2;
    double* p = (double*)realloc(o->v, c * 3 * sizeof(double));
    if (!p) return SO_ERR_NOMEM;
    o->v = p;
    o->capv = c;
    return SO_OK;
}

static int grow_t(p5_out* o, uint64_t need) {
    if (need <= o->capt) return SO_OK;
    uint64_t c = o->capt ? o->capt : 1024;
    while (c < need) c *= 2;
    int64_t* p = (int64_t*)realloc(o->t, c * 3 * sizeof(int64_t));
    if (!p) return SO_ERR_NOMEM;
    o->t = p;
    o->capt = c;
    return SO_OK;
}

typedef struct {
    int v, para, a, b, c;
} p5_emit;

/* One meshlet (paradelta_v5.py:342-451). */
static int decode_meshlet(so_br* r, const p5_header* h, double delta, p5_out* o) {
    const int n_bnd = (int)br_read(r, 16);
    const int n_int = (int)br_read(r, 16);
    const int n_tris = (int)br_read(r, 16);
    const int n_strips = (int)br_read(r, 16);
    (void)n_tris;
    if (r->err) return r->err;
    const int n_local = n_bnd + n_int;
    int rc = SO_OK;
    int64_t* l2g = (int64_t*)malloc((size_t)(n_local ? n_local : 1) * sizeof(int64_t));
    double* recon = (double*)calloc((size_t)(n_local ? n_local : 1) * 3, sizeof(double));
    unsigned char* seen = (unsigned char*)calloc((size_t)(n_local ? n_local : 1), 1);
    p5_emit* emit = (p5_emit*)malloc((size_t)(n_int ? n_int : 1) * sizeof(p5_emit));
    int64_t* codes = (int64_t*)calloc((size_t)(n_int ? n_int : 1) * 3, sizeof(int64_t));
    int64_t* tris = NULL;
    uint64_t nt = 0, capt = 0;
    int n_emit = 0;
    if (!l2g || !recon || !seen || !emit || !codes) { rc = SO_ERR_NOMEM; goto done; }

    /* boundary references (:350-361) */
    if (n_bnd > 0) {
        int64_t prev = (int64_t)br_read(r, 32);
        l2g[0] = prev;
        if (n_bnd > 1) {
            const int k = (int)br_read(r, 8);
            for (int i = 1; i < n_bnd; i++) {
                const uint64_t u = br_rice(r, k);
                if (r->err) { rc = r->err; goto done; }
                prev = prev + (int64_t)u + 1;
                l2g[i] = prev;
            }
        }
        if (r->err) { rc = r->err; goto done; }
    }
    const int64_t first_interior = (int64_t)o->nv;
    for (int i = 0; i < n_int; i++) l2g[n_bnd + i] = first_interior + i;
    if ((rc = grow_v(o, o->nv + (uint64_t)n_int)) != SO_OK) goto done;
    for (int i = 0; i < n_int; i++) {
        double* p = o->v + 3 * (o->nv + (uint64_t)i);
        p[0] = p[1] = p[2] = 0.0;
    }
    o->nv += (uint64_t)n_int;
    /* the reconstruction reads the referenced vertices (IndexError past the
       vertices so far, this meshlet's interior zeros included); without
       interior vertices the references only become triangle indices */
    if (n_int > 0)
        for (int i = 0; i < n_bnd; i++)
            if ((uint64_t)l2g[i] >= o->nv) { rc = SO_ERR_VERTEX; goto done; }
    for (int i = 0; i < n_bnd; i++) seen[i] = 1;

    /* connectivity + first-reach order of interior vertices (:371-400) */
    {
        so_fifo f;
        f.len = 0;
        const int idx_bits = n_local > 0 ? (bitlen((uint32_t)n_local) > 1 ? bitlen((uint32_t)n_local) : 1) : 1;
        for (int s = 0; s < n_strips; s++) {
            const int strip_len = (int)br_read(r, 16);
            int v[3];
            for (int j = 0; j < 3; j++) {
                if ((rc = read_vert(r, &f, idx_bits, &v[j])) != SO_OK) goto done;
                if (v[j] >= n_local) { rc = SO_ERR_VERTEX; goto done; }
            }
            if (r->err) { rc = r->err; goto done; }
            if (nt + 1 > capt) {
                capt = capt ? 2 * capt : 256;
                int64_t* p = (int64_t*)realloc(tris, capt * 3 * sizeof(int64_t));
                if (!p) { rc = SO_ERR_NOMEM; goto done; }
                tris = p;
            }
            tris[3 * nt] = v[0]; tris[3 * nt + 1] = v[1]; tris[3 * nt + 2] = v[2];
            nt++;
            for (int j = 0; j < 3; j++) {
                if (v[j] >= n_bnd && !seen[v[j]]) {
                    if (n_emit >= n_int) { rc = SO_ERR_VERTEX; goto done; }
                    emit[n_emit++] = (p5_emit){v[j], 0, 0, 0, 0};
                }
                seen[v[j]] = 1;
            }
            int p0 = v[0], p1 = v[1], p2 = v[2];
            for (int t = 0; t < strip_len - 1; t++) {
                const int edge = (int)br_read(r, 1);
                int nv;
                if ((rc = read_vert(r, &f, idx_bits, &nv)) != SO_OK) goto done;
                if (r->err) { rc = r->err; goto done; }
                if (nv >= n_local) { rc = SO_ERR_VERTEX; goto done; }
                int a, b, c;
                if (edge == 0) { a = p1; b = p2; c = p0; }
                else { a = p0; b = p2; c = p1; }
                if (nt + 1 > capt) {
                    capt = capt ? 2 * capt : 256;
                    int64_t* p = (int64_t*)realloc(tris, capt * 3 * sizeof(int64_t));
                    if (!p) { rc = SO_ERR_NOMEM; goto done; }
                    tris = p;
                }
                tris[3 * nt] = a; tris[3 * nt + 1] = b; tris[3 * nt + 2] = nv;
                nt++;
                if (nv >= n_bnd && !seen[nv]) {
                    if (n_emit >= n_int) { rc = SO_ERR_VERTEX; goto done; }
                    emit[n_emit++] = (p5_emit){nv, 1, a, b, c};
                }
                seen[nv] = 1;
                p0 = a; p1 = b; p2 = nv;
            }
        }
    }

    /* residual codes per axis, then reconstruction (:403-445) */
    if (n_int > 0) {
        for (int d = 0; d < 3; d++) {
            const int tag = (int)br_read(r, 8);
            if (r->err) { rc = r->err; goto done; }
            if (tag == 0) {
                const uint32_t mn_u = (uint32_t)br_read(r, 16);
                const int64_t mn = (mn_u & 0x8000u) ? (int64_t)mn_u - 0x10000 : (int64_t)mn_u;
                const int bw = (int)br_read(r, 8);
                if (bw > 56) { rc = SO_ERR_UNSUPPORTED; goto done; }
                for (int i = 0; i < n_int; i++) codes[3 * i + d] = mn + (int64_t)br_read(r, bw);
            } else if (tag == 1) {
                const int k = (int)br_read(r, 8);
                for (int i = 0; i < n_int && !r->err; i++) codes[3 * i + d] = unzigzag(br_rice(r, k));
            } else if (tag == 2) {
                const int k = (int)br_read(r, 8);
                for (int i = 0; i < n_int && !r->err; i++) codes[3 * i + d] = unzigzag(br_eg(r, k));
            } else {
                rc = SO_ERR_UNSUPPORTED;
                goto done;
            }
            if (r->err) { rc = r->err; goto done; }
        }
        for (int i = 0; i < n_bnd; i++)
            for (int d = 0; d < 3; d++) recon[3 * i + d] = o->v[3 * (uint64_t)l2g[i] + d];
        double fb[3] = {0.0, 0.0, 0.0};
        if (n_bnd > 0) {
            for (int d = 0; d < 3; d++) {
                double s = recon[d];
                for (int i = 1; i < n_bnd; i++) s = s + recon[3 * i + d];
                fb[d] = s / (double)n_bnd;
            }
        }
        const double w0 = (double)h->lin3_w[0], w1 = (double)h->lin3_w[1], w2 = (double)h->lin3_w[2];
        for (int i = 0; i < n_emit; i++) {
            const p5_emit e = emit[i];
            for (int d = 0; d < 3; d++) {
                double pred;
                if (e.para) {
                    const double t0 = w0 * recon[3 * e.a + d];
                    const double t1 = w1 * recon[3 * e.b + d];
                    const double t2 = w2 * recon[3 * e.c + d];
                    pred = (t0 + t1) + t2;
                } else {
                    pred = fb[d];
                }
                const double rec = pred + (double)codes[3 * i + d] * delta;
                recon[3 * e.v + d] = rec;
                o->v[3 * (uint64_t)l2g[e.v] + d] = rec;
            }
        }
    }

    /* global triangle indices (:447-451) */
    if ((rc = grow_t(o, o->nt + nt)) != SO_OK) goto done;
    for (uint64_t t = 0; t < 3 * nt; t++) o->t[3 * o->nt + t] = l2g[tris[t]];
    o->nt += nt;
done:
    free(l2g);
    free(recon);
    free(seen);
    free(emit);
    free(codes);
    free(tris);
    return rc;
}

/* Decode the whole stream.  With pos/idx NULL (or too small) only the sizes
 * are returned in *n_v_out / *n_t_out (SO_ERR_CAPACITY when buffers were
 * given but are too small). */
int p5_decode(const uint8_t* data, uint64_t len, float* pos, int64_t* idx, uint64_t cap_v, uint64_t cap_t,
              uint64_t* n_v_out, uint64_t* n_t_out) {
    so_br r = {data, len * 8ull, 0, 0};
    p5_header h;
    int rc = p5_header_read(&r, &h);
    if (rc) return rc;
    const double delta = 2.0 * (double)h.per_coord_err;
    p5_out o = {0};
    /* boundary table (:312-336) */
    const uint64_t nb = h.n_boundary;
    if ((rc = grow_v(&o, nb)) != SO_OK) goto fail;
    {
        int64_t* bc = (int64_t*)calloc((size_t)(nb ? nb : 1) * 3, sizeof(int64_t));
        if (!bc) { rc = SO_ERR_NOMEM; goto fail; }
        for (int d = 0; d < 3 && nb > 0; d++) {
            bc[d] = (int64_t)br_read(&r, (int)h.g_bits[d]);
            if (nb > 1) {
                const int k = (int)br_read(&r, 8);
                for (uint64_t i = 1; i < nb && !r.err; i++) bc[3 * i + d] = bc[3 * (i - 1) + d] + unzigzag(br_rice(&r, k));
            }
        }
        if (r.err) { free(bc); rc = r.err; goto fail; }
        for (uint64_t i = 0; i < nb; i++) {
            for (int d = 0; d < 3; d++) {
                const uint64_t mx = (h.g_bits[d] >= 64) ? ~0ull : ((1ull << h.g_bits[d]) - 1ull);
                double v;
                if (mx == 0) {
                    v = (double)h.g_min[d];
                } else {
                    const double q = (double)bc[3 * i + d] / (double)mx;
                    const double s = q * (double)h.g_range[d];
                    v = (double)h.g_min[d] + s;
                }
                o.v[3 * i + d] = v;
            }
        }
        o.nv = nb;
        free(bc);
    }
    /* skip to the byte boundary and past the offset table (:338-344) */
    {
        const uint64_t pad = (uint64_t)((-(int64_t)r.pos) & 7);
        r.pos += pad;
        if (r.pos + 32ull * h.n_meshlets > r.nbits) { rc = SO_ERR_EOF; goto fail; }
        r.pos += 32ull * h.n_meshlets;
    }
    for (uint32_t m = 0; m < h.n_meshlets; m++)
        if ((rc = decode_meshlet(&r, &h, delta, &o)) != SO_OK) goto fail;
    *n_v_out = o.nv;
    *n_t_out = o.nt;
    if (pos && idx) {
        if (cap_v < o.nv || cap_t < o.nt) { rc = SO_ERR_CAPACITY; goto fail; }
        const double sc = (double)h.scale;
        for (uint64_t i = 0; i < o.nv; i++)
            for (int d = 0; d < 3; d++) pos[3 * i + d] = (float)(o.v[3 * i + d] * sc + (double)h.center[d]);
        memcpy(idx, o.t, o.nt * 3 * sizeof(int64_t));
    }
    free(o.v);
    free(o.t);
    return SO_OK;
fail:
    free(o.v);
    free(o.t);
    return rc;
}

/* Per-meshlet tables of a PLDT v5 stream, as the reference GPU decoder
 * derives them (parse_globals_v5 and its sizes kernel,
 * utils/paradelta_v5_cuda.py:515-660): each meshlet's absolute start bit
 * from the offset table and its four header fields, and the boundary rows
 * in float64 (g_min + code / mx * g_range).  Any output may be NULL. */
int p5_tables(const uint8_t* data, uint64_t len, uint64_t* off_bits, int32_t* n_bnd, int32_t* n_int,
              int32_t* n_tris, int32_t* n_strips, double* bnd_rows) {
    so_br r = {data, len * 8ull, 0, 0};
    p5_header h;
    int rc = p5_header_read(&r, &h);
    if (rc) return rc;
    const uint64_t nb = h.n_boundary;
    int64_t* bc = (int64_t*)calloc((size_t)(nb ? nb : 1) * 3, sizeof(int64_t));
    if (!bc) return SO_ERR_NOMEM;
    for (int d = 0; d < 3 && nb > 0; d++) {
        bc[d] = (int64_t)br_read(&r, (int)h.g_bits[d]);
        if (nb > 1) {
            const int k = (int)br_read(&r, 8);
            for (uint64_t i = 1; i < nb && !r.err; i++) bc[3 * i + d] = bc[3 * (i - 1) + d] + unzigzag(br_rice(&r, k));
        }
    }
    if (r.err) { free(bc); return r.err; }
    if (bnd_rows) {
        for (uint64_t i = 0; i < nb; i++)
            for (int d = 0; d < 3; d++) {
                const uint64_t mx = (1ull << h.g_bits[d]) - 1ull;
                bnd_rows[3 * i + d] = mx == 0 ? (double)h.g_min[d]
                                              : (double)h.g_min[d] + ((double)bc[3 * i + d] / (double)mx) * (double)h.g_range[d];
            }
    }
    free(bc);
    r.pos += (uint64_t)((-(int64_t)r.pos) & 7);
    for (uint32_t m = 0; m < h.n_meshlets; m++) {
        const uint64_t o = br_read(&r, 32);
        if (r.err) return r.err;
        so_br q = {data, len * 8ull, o, 0};
        const int32_t b = (int32_t)br_read(&q, 16), i = (int32_t)br_read(&q, 16);
        const int32_t t = (int32_t)br_read(&q, 16), s = (int32_t)br_read(&q, 16);
        if (q.err) return q.err;
        if (off_bits) off_bits[m] = o;
        if (n_bnd) n_bnd[m] = b;
        if (n_int) n_int[m] = i;
        if (n_tris) n_tris[m] = t;
        if (n_strips) n_strips[m] = s;
    }
    return SO_OK;
}
