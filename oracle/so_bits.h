/*
 * Bit reader and vertex FIFO shared by the CPU oracles (STRIDE DPR4 v3 and
 * PLDT v5).  TEST INFRASTRUCTURE ONLY.
 *
 *   BitReader.read_bits/_rice/_exp_golomb/_f32   utils/bit_codec.py:192-254
 *   _read_vert (+ 16-entry move-to-tail FIFO)    encoder/paradelta_codec.py:330-340
 */
#ifndef SO_BITS_H
#define SO_BITS_H

#include <stdint.h>
#include <string.h>

#define SO_OK 0
#define SO_ERR_MAGIC (-1)
#define SO_ERR_VERSION (-2)
#define SO_ERR_EOF (-3)
#define SO_ERR_FIFO (-4)
#define SO_ERR_VERTEX (-5)
#define SO_ERR_OVERFLOW (-6)
#define SO_ERR_CAPACITY (-7)
#define SO_ERR_UNSUPPORTED (-8)
#define SO_ERR_LAYOUT (-9)
#define SO_ERR_NOMEM (-10)

#define SO_FIFO 16
#define SO_REUSE_BITS 5

/* ---- MSB-first bit reader (utils/bit_codec.py:192-254) ------------------ */
typedef struct {
    const uint8_t* buf;
    uint64_t nbits;
    uint64_t pos;
    int err;
} so_br;

static inline uint64_t br_read(so_br* r, int n) { /* n <= 64 */
    if (n <= 0) return 0;
    if (r->pos + (uint64_t)n > r->nbits) { r->err = SO_ERR_EOF; r->pos = r->nbits; return 0; }
    uint64_t v = 0;
    int left = n;
    while (left > 0) {
        uint64_t byte = r->pos >> 3;
        int bit = (int)(r->pos & 7);
        int avail = 8 - bit;
        int take = avail < left ? avail : left;
        uint32_t chunk = ((uint32_t)r->buf[byte] >> (avail - take)) & ((1u << take) - 1u);
        v = (v << take) | chunk;
        r->pos += (uint64_t)take;
        left -= take;
    }
    return v;
}

/* Count zeros up to and including the terminating one bit. */
static inline uint64_t br_unary(so_br* r) {
    uint64_t q = 0;
    for (;;) {
        if (r->pos >= r->nbits) { r->err = SO_ERR_EOF; return 0; }
        uint64_t byte = r->pos >> 3;
        int bit = (int)(r->pos & 7);
        r->pos++;
        if ((r->buf[byte] >> (7 - bit)) & 1u) return q;
        q++;
    }
}

static inline uint64_t br_rice(so_br* r, int k) {
    uint64_t q = br_unary(r);
    if (r->err) return 0;
    if (k > 56) { r->err = SO_ERR_UNSUPPORTED; return 0; }
    uint64_t low = k ? br_read(r, k) : 0;
    unsigned __int128 u = ((unsigned __int128)q << k) | low;
    if (u >> 64) { r->err = SO_ERR_OVERFLOW; return 0; }
    return (uint64_t)u;
}

static inline uint64_t br_eg(so_br* r, int k) {
    uint64_t lb = br_unary(r);
    if (r->err) return 0;
    if (k > 56 || lb > 64) { r->err = (lb > 64) ? SO_ERR_OVERFLOW : SO_ERR_UNSUPPORTED; return 0; }
    unsigned __int128 shifted = 0;
    if (lb > 0) {
        uint64_t off = br_read(r, (int)lb);
        shifted = (((unsigned __int128)1 << lb) - 1) + off;
    }
    uint64_t low = k ? br_read(r, k) : 0;
    unsigned __int128 u = (shifted << k) | low;
    if (u >> 64) { r->err = SO_ERR_OVERFLOW; return 0; }
    return (uint64_t)u;
}

static inline int64_t unzigzag(uint64_t u) { return (int64_t)((u >> 1) ^ (0 - (u & 1))); }

static inline int bitlen(uint32_t n) {
    int b = 0;
    while (n) { b++; n >>= 1; }
    return b;
}

static inline float f32_from_bits(uint32_t b) {
    float f;
    memcpy(&f, &b, 4);
    return f;
}

typedef struct {
    int fifo[SO_FIFO];
    int len;
} so_fifo;

static inline int read_vert(so_br* r, so_fifo* f, int idx_bits, int* out) {
    int v;
    if (br_read(r, 1) == 0) {
        int fi = (int)br_read(r, SO_REUSE_BITS);
        if (r->err) return r->err;
        if (fi >= f->len) return SO_ERR_FIFO;
        v = f->fifo[fi];
    } else {
        v = (int)br_read(r, idx_bits);
        if (r->err) return r->err;
    }
    int at = -1;
    for (int i = 0; i < f->len; i++)
        if (f->fifo[i] == v) { at = i; break; }
    if (at >= 0) {
        memmove(&f->fifo[at], &f->fifo[at + 1], (size_t)(f->len - at - 1) * sizeof(int));
        f->len--;
    } else if (f->len == SO_FIFO) {
        memmove(&f->fifo[0], &f->fifo[1], (SO_FIFO - 1) * sizeof(int));
        f->len--;
    }
    f->fifo[f->len++] = v;
    *out = v;
    return SO_OK;
}

#endif /* SO_BITS_H */
