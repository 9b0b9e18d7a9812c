// Exact STRIDE dequantisation without a per-code float64 pipeline.
//
// The reference computes every decoded coordinate as the float64 expression
//     t5 = ((g_min + (q / mx) * g_range) * scale) + center,   out = f32(t5)
// (encoder/paradelta_v5_dup.py:607-618; mx = 2^g_bits - 1, all header floats
// widened from f32, no FMA).  GB300 has very little float64 throughput, so
// the decoder evaluates the same value as a float-float affine form
//     A(q) = alpha + beta * q,   alpha = center + scale*g_min,
//                                beta  = scale*g_range/mx
// (alpha, beta split into f32 hi+lo pairs on the host) with error-free
// transformations (TwoSum, FMA-exact products), and rounds it to f32 only
// when the rounding is provably the same as the reference's:
//   |t5 - A_computed| <= err  (err = 2^-40 * M, M = |center| +
//   |scale|*(|g_min| + |g_range|), a >16x over-estimate of the float64
//   pipeline's five roundings plus the float-float representation error),
// so if [A - err, A + err] lies strictly inside the rounding cell of the f32
// value y nearest A, f32(t5) == y.  Otherwise (about 2^-16 of the codes, plus
// |y| < 2^-102, zero, inf/nan) the float64 expression is evaluated directly
// with correctly rounded operations.  This is Ziv's rounding test.
//
// Used by the CUDA kernels (STRIDE_DEQUANT_DEVICE) and, compiled as C with
// -ffp-contract=off, by the CPU tests that check every code of many random
// headers against the float64 expression.
#ifndef STRIDE_DEQUANT_H
#define STRIDE_DEQUANT_H

#include <stdint.h>

#include <math.h>

#ifdef __CUDACC__
#define SD_HD __host__ __device__ __forceinline__
#else
#define SD_HD static inline
#endif

typedef struct {
    float a_hi, a_lo, b_hi, b_lo; /* alpha, beta as float-float            */
    float err;                    /* absolute error bound (see above)      */
    float konst;                  /* value for g_bits == 0                 */
    int32_t zero_bits;            /* g_bits == 0: every code gives konst   */
    int32_t pad;
    double gmin, grange, mx, scale, center; /* exact float64 fallback       */
} stride_dequant_axis;

#if defined(__CUDA_ARCH__)
#define SD_ADD(a, b) __fadd_rn((a), (b))
#define SD_SUB(a, b) __fsub_rn((a), (b))
#define SD_MUL(a, b) __fmul_rn((a), (b))
#define SD_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define SD_DDIV(a, b) __ddiv_rn((a), (b))
#define SD_DMUL(a, b) __dmul_rn((a), (b))
#define SD_DADD(a, b) __dadd_rn((a), (b))
#define SD_D2F(a) __double2float_rn(a)
#define SD_F2U(a) __float_as_uint(a)
#define SD_U2F(a) __uint_as_float(a)
#define SD_FABS(a) fabsf(a)
#else
#include <math.h>
#include <string.h>
#define SD_ADD(a, b) ((float)((a) + (b)))
#define SD_SUB(a, b) ((float)((a) - (b)))
#define SD_MUL(a, b) ((float)((a) * (b)))
#define SD_FMA(a, b, c) fmaf((a), (b), (c))
#define SD_DDIV(a, b) ((a) / (b))
#define SD_DMUL(a, b) ((a) * (b))
#define SD_DADD(a, b) ((a) + (b))
#define SD_D2F(a) ((float)(a))
SD_HD uint32_t sd_f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
SD_HD float sd_u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
#define SD_F2U(a) sd_f2u(a)
#define SD_U2F(a) sd_u2f(a)
#define SD_FABS(a) fabsf(a)
#endif

/* The reference's float64 expression, correctly rounded step by step. */
SD_HD float stride_dequant_exact(const stride_dequant_axis* p, uint32_t q) {
    if (p->zero_bits) return p->konst;
    double t = SD_DDIV((double)q, p->mx);
    t = SD_DMUL(t, p->grange);
    t = SD_DADD(p->gmin, t);
    t = SD_DMUL(t, p->scale);
    t = SD_DADD(t, p->center);
    return SD_D2F(t);
}

/* Fast path; returns 1 and the result when the rounding test passes. */
SD_HD int stride_dequant_fast(const stride_dequant_axis* p, uint32_t q, float* out) {
    const float qf = (float)q; /* exact: q < 2^24 */
    const float pr = SD_MUL(p->b_hi, qf);
    const float pe = SD_FMA(p->b_hi, qf, -pr);          /* b_hi*q = pr + pe exactly */
    const float s = SD_ADD(p->a_hi, pr);
    const float bb = SD_SUB(s, p->a_hi);
    const float se = SD_ADD(SD_SUB(p->a_hi, SD_SUB(s, bb)), SD_SUB(pr, bb)); /* TwoSum */
    const float t1 = SD_FMA(p->b_lo, qf, p->a_lo);
    const float lo = SD_ADD(SD_ADD(se, pe), t1);
    const float y = SD_ADD(s, lo);
    const float ylo = SD_SUB(lo, SD_SUB(y, s));          /* y + ylo == s + lo */
    const uint32_t bits = SD_F2U(y);
    const uint32_t e = (bits >> 23) & 0xFFu;
    if (e < 26u || e > 253u) return 0;
    const float half_above = SD_U2F((e - 24u) << 23);    /* ulp(y) / 2 */
    const float half = (bits & 0x7FFFFFu) ? half_above : SD_MUL(half_above, 0.5f);
    /* t5 lies in (y - half, y + half) when |ylo| + err < half.  half - |ylo|
     * is exact when |ylo| >= half/2 (Sterbenz) and far above err otherwise;
     * the factor 2 absorbs its rounding in that case. */
    if (SD_SUB(half, SD_FABS(ylo)) > SD_MUL(p->err, 2.0f)) {
        *out = y;
        return 1;
    }
    return 0;
}

SD_HD float stride_dequant(const stride_dequant_axis* p, uint32_t q) {
    float y;
    if (!p->zero_bits && stride_dequant_fast(p, q, &y)) return y;
    return stride_dequant_exact(p, q);
}

/* Host-side constants for one axis (compile without FMA contraction). */
static inline void stride_dequant_setup(stride_dequant_axis* p, float center, float scale,
                                        float gmin, float grange, uint32_t g_bits) {
    volatile double c = (double)center, sc = (double)scale, gm = (double)gmin, gr = (double)grange;
    p->zero_bits = g_bits == 0;
    p->pad = 0;
    p->gmin = gm;
    p->grange = gr;
    p->scale = sc;
    p->center = c;
    p->mx = g_bits ? (double)((1ull << g_bits) - 1ull) : 0.0;
    volatile double k1 = gm * sc;
    volatile double k2 = k1 + c;
    p->konst = (float)k2; /* f32(g_min * scale + center): the g_bits == 0 case */
    volatile double am = gm * sc;
    volatile double alpha = c + am;
    volatile double bm = sc * gr;
    volatile double beta = g_bits ? bm / p->mx : 0.0;
    p->a_hi = (float)alpha;
    p->a_lo = (float)(alpha - (double)p->a_hi);
    p->b_hi = (float)beta;
    p->b_lo = (float)(beta - (double)p->b_hi);
    double M = fabs(c) + fabs(sc) * (fabs(gm) + fabs(gr));
    p->err = (float)(ldexp(M, -40) * 1.01);
}

#endif /* STRIDE_DEQUANT_H */
