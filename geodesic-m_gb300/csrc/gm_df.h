/* gm_df.h — double-float arithmetic: a value carried as an unevaluated sum
 * h + l of two FP32 numbers, |l| <= ~ulp(h), about 44 significant bits.
 *
 * The mixed-precision pair kernel does its arithmetic on the FP32 pipe and
 * still reaches ~1e-10 relative error per pair with these building blocks:
 *   gm_two_sum   Knuth's TwoSum: s = RN(a + b) and the exact error a + b - s;
 *   gm_fast_sum  Dekker's Fast2Sum (|a| >= |b| or a == 0);
 *   gm_dmul      product of two double-floats: the FP32 product and its exact
 *                error from one FMA (Dekker/Kahan TwoProduct), plus the two
 *                cross terms; the low*low term is dropped and the result is
 *                not renormalised (relative error a few times 2^-44);
 *   gm_dsqr      the same for a square;
 *   gm_dadd      sum of two double-floats (TwoSum of the heads, tails added).
 * Every rounding that the error terms rely on goes through __fadd_rn /
 * __fmul_rn on the device, which the compiler never contracts into an FMA.
 * tests/test_exact_arithmetic.py compiles this header as C11 (with
 * -ffp-contract=off) and checks the helpers against FP64 and long double.
 */
#ifndef GM_DF_H
#define GM_DF_H

#include <math.h>

#ifdef __CUDACC__
#define GM_DF_HD __host__ __device__ __forceinline__
#else
#define GM_DF_HD static inline
#endif

typedef struct {
    float h, l;
} gm_df;

#ifdef __CUDA_ARCH__
#define GM_FADD(a, b) __fadd_rn((a), (b))
#define GM_FSUB(a, b) __fsub_rn((a), (b))
#define GM_FMUL(a, b) __fmul_rn((a), (b))
#define GM_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define GM_FADD(a, b) ((a) + (b))
#define GM_FSUB(a, b) ((a) - (b))
#define GM_FMUL(a, b) ((a) * (b))
#define GM_FMA(a, b, c) fmaf((a), (b), (c))
#endif

GM_DF_HD gm_df gm_df_make(float h, float l) {
    gm_df r;
    r.h = h;
    r.l = l;
    return r;
}

GM_DF_HD gm_df gm_two_sum(float a, float b) {
    const float s = GM_FADD(a, b);
    const float bb = GM_FSUB(s, a);
    const float e = GM_FADD(GM_FSUB(a, GM_FSUB(s, bb)), GM_FSUB(b, bb));
    return gm_df_make(s, e);
}

GM_DF_HD gm_df gm_fast_sum(float a, float b) {
    const float s = GM_FADD(a, b);
    return gm_df_make(s, GM_FSUB(b, GM_FSUB(s, a)));
}

GM_DF_HD gm_df gm_dmul(gm_df a, gm_df b) {
    const float p = GM_FMUL(a.h, b.h);
    float e = GM_FMA(a.h, b.h, -p);
    e = GM_FMA(a.h, b.l, e);
    e = GM_FMA(a.l, b.h, e);
    return gm_df_make(p, e);
}

GM_DF_HD gm_df gm_dmulf(gm_df a, float b) {
    const float p = GM_FMUL(a.h, b);
    float e = GM_FMA(a.h, b, -p);
    e = GM_FMA(a.l, b, e);
    return gm_df_make(p, e);
}

GM_DF_HD gm_df gm_dsqr(gm_df a) {
    const float p = GM_FMUL(a.h, a.h);
    float e = GM_FMA(a.h, a.h, -p);
    e = GM_FMA(GM_FADD(a.h, a.h), a.l, e);
    return gm_df_make(p, e);
}

GM_DF_HD gm_df gm_dadd(gm_df a, gm_df b) {
    gm_df s = gm_two_sum(a.h, b.h);
    s.l = GM_FADD(s.l, GM_FADD(a.l, b.l));
    return s;
}

GM_DF_HD gm_df gm_dneg(gm_df a) { return gm_df_make(-a.h, -a.l); }

/* x as a double-float: the FP32 rounding of x and the FP32 rounding of the
 * remainder (exact to ~2^-48 relative). */
GM_DF_HD gm_df gm_df_from_double(double x) {
    const float h = (float)x;
    return gm_df_make(h, (float)(x - (double)h));
}

#endif
