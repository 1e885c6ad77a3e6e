/* Checks the exact-rounding helpers of gm_exact_math.h (compiled here as C11,
 * with contraction off) against the reference rounding they must reproduce:
 *   gm_f2fix(v)            == nearbyint(v * 2^40) (ties to even) for |v| < 2^22
 *   gm_div_by_dt(n, dt, y) == n / dt bit for bit, y = 1 / dt
 * on seeded pseudo-random samples.  Usage: exact_arith_check N_SAMPLES
 * Prints "f2fix <checked> <mismatches>" and "div <checked> <mismatches>";
 * exit status 1 on any mismatch. */
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <string.h>
#include <math.h>

#include "gm_exact_math.h"

static uint64_t s = 0x9E3779B97F4A7C15ull;
static uint64_t rnd(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double unit(void) { return (double)(rnd() >> 11) * (1.0 / 9007199254740992.0); }
static uint64_t bits64(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static double from64(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static float from32(uint32_t u) { float x; memcpy(&x, &u, 4); return x; }

int main(int argc, char **argv) {
    const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
    long long bad_f = 0, n_f = 0, bad_d = 0, n_d = 0;
    for (long long k = 0; k < n; k++) {
        /* every float below 2^22 in magnitude is a candidate bit pattern */
        const uint32_t b = (uint32_t)(rnd() % 0x4A800000u) | ((rnd() & 1u) ? 0x80000000u : 0u);
        const float v = from32(b);
        if (isfinite(v) && fabsf(v) < 4194304.0f) {
            const long long ref = (long long)nearbyint((double)v * 1099511627776.0);
            if (gm_f2fix(v) != ref) bad_f++;
            n_f++;
        }
        /* velocity-resync operands (x + dt v) - x and arbitrary numerators */
        const double dt = (k & 1) ? 0.002 : 1e-4 + unit() * 1e-2;
        const double y = 1.0 / dt;
        double num;
        if (k & 2) {
            const double p = (unit() - 0.5) * pow(10.0, (int)(unit() * 8) - 2);
            const double vel = (unit() - 0.5) * pow(10.0, (int)(unit() * 6) - 3);
            num = (p + dt * vel) - p;
        } else {
            const uint64_t m = rnd() & 0xFFFFFFFFFFFFFull;
            const int e = (int)(rnd() % 121) - 60 + 1023;
            num = from64(((rnd() & 1ull) << 63) | ((uint64_t)e << 52) | m);
        }
        if (bits64(gm_div_by_dt(num, dt, y)) != bits64(num / dt)) bad_d++;
        n_d++;
    }
    printf("f2fix %lld %lld\ndiv %lld %lld\n", n_f, bad_f, n_d, bad_d);
    return (bad_f || bad_d) ? 1 : 0;
}
