/* gm_exact_math.h — exact-rounding helpers shared by the kernels and by the
 * CPU test that checks them (tests/test_exact_arithmetic.py compiles this
 * header as C11 with gcc).
 *
 * gm_f2fix:  round(v * 2^40) to the nearest integer, ties to even, for
 *            |v| < 2^22, from the bits of v with integer operations only (the
 *            value of __float2ll_rn(v * 2^40); the 64-bit conversion
 *            instruction is slow on this part).
 * gm_div_by_dt: num / dt correctly rounded from y = RN(1 / dt), computed once:
 *            Markstein's correction (P. Markstein, "IA-64 and Elementary
 *            Functions", 2000): q = RN(num y), r = num - q dt is exact in one
 *            FMA, and RN(q + r y) is the correctly rounded quotient when y is
 *            the correctly rounded reciprocal (away from overflow and
 *            underflow).  Three FP64 operations instead of a division.
 */
#ifndef GM_EXACT_MATH_H
#define GM_EXACT_MATH_H

#include <math.h>
#include <string.h>

#ifdef __CUDACC__
#define GM_HD __host__ __device__ __forceinline__
#else
#define GM_HD static inline
#endif

GM_HD long long gm_f2fix(float v) {
#ifdef __CUDA_ARCH__
    const unsigned int b = __float_as_uint(v);
#else
    unsigned int b;
    memcpy(&b, &v, sizeof b);
#endif
    const int e = (int)((b >> 23) & 0xffu);
    const long long m = (long long)((b & 0x7fffffu) | 0x800000u);
    const int sh = e - 150 + 40; /* |v| * 2^40 = m * 2^sh for normal v */
    long long r;
    if (e == 0 || sh < -25) {
        r = 0; /* below 2^-41: rounds to zero */
    } else if (sh >= 0) {
        r = m << sh;
    } else {
        const int s = -sh;
        const long long q = m >> s, rem = m & ((1ll << s) - 1), half = 1ll << (s - 1);
        r = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
    }
    return (b >> 31) ? -r : r;
}

GM_HD double gm_div_by_dt(double num, double dt, double y) {
    const double q = num * y;
    const double r = fma(-q, dt, num);
    return fma(r, y, q);
}

#endif
