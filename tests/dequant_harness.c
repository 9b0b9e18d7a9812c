/* Test harness: exposes the decoder's exact-dequantisation routine
 * (meshpress_gb300/csrc/stride_dequant.h) to the CPU tests.  Compiled with
 * gcc -ffp-contract=off so float operations round exactly like the device
 * intrinsics __fadd_rn / __fmul_rn / __fmaf_rn. */
#include "stride_dequant.h"

/* Returns the number of codes where the fast path's answer differs from the
 * float64 expression (must be 0); *n_fast counts codes decided by the fast
 * path.  Writes every result to out. */
int64_t dq_check(float center, float scale, float gmin, float grange, uint32_t g_bits,
                 uint32_t q0, uint32_t q1, float* out, int64_t* n_fast) {
    stride_dequant_axis p;
    stride_dequant_setup(&p, center, scale, gmin, grange, g_bits);
    int64_t bad = 0, fast = 0;
    for (uint32_t q = q0; q < q1; q++) {
        float e = stride_dequant_exact(&p, q);
        float y;
        int ok = !p.zero_bits && stride_dequant_fast(&p, q, &y);
        if (ok) {
            fast++;
            if (sd_f2u(y) != sd_f2u(e)) bad++;
        }
        out[q - q0] = stride_dequant(&p, q);
    }
    *n_fast = fast;
    return bad;
}
