/* The Naive Surface Nets mean's division by the crossing count n (1..12) as
 * the CUDA kernels compute it (div_count in k_emit_halo.cu): y = RN(1/n),
 * q = RN(a*y), r = fma(-q, n, a), result fma(r, y, q); zeros, magnitudes
 * below 2^-959 (Float32: 2^-63) and Inf / NaN take the division.  This program
 * restates those operations in the host's IEEE arithmetic (C99 fma, correctly
 * rounded) and counts, per precision, the inputs whose result differs in any
 * bit from the IEEE quotient a / n: random significands over the whole
 * exponent range, quotients next to rounding midpoints, powers of two,
 * values at the fallback thresholds, and the largest finite values.
 * Usage: count_division <samples per n>; prints "<double mismatches> <float
 * mismatches> <cases>". */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t s = 0x9e3779b97f4a7c15ull;
static uint64_t next(void) {  /* splitmix64 */
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static double d_of(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static uint64_t b_of(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }
static float f_of(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t fb_of(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

static double rcp_d[13];
static float rcp_f[13];

static double div_count_d(double a, int n) {
    const unsigned e = (unsigned)(b_of(a) >> 52) & 0x7ffu;
    if (e < 64u || e == 0x7ffu) return a / (double)n;
    const volatile double y = rcp_d[n];
    const double q = a * y;
    return fma(fma(-q, (double)n, a), y, q);
}
static float div_count_f(float a, int n) {
    const unsigned e = (fb_of(a) >> 23) & 0xffu;
    if (e < 64u || e == 0xffu) return a / (float)n;
    const volatile float y = rcp_f[n];
    const float q = a * y;
    return fmaf(fmaf(-q, (float)n, a), y, q);
}

static long bad_d = 0, bad_f = 0, cases = 0;
static void check_d(double a, int n) {
    const double w = a / (double)n, g = div_count_d(a, n);
    cases++;
    if (b_of(w) != b_of(g) && !(isnan(w) && isnan(g))) {
        if (bad_d < 5) fprintf(stderr, "double a=%a n=%d want %a got %a\n", a, n, w, g);
        bad_d++;
    }
}
static void check_f(float a, int n) {
    const float w = a / (float)n, g = div_count_f(a, n);
    cases++;
    if (fb_of(w) != fb_of(g) && !(isnan(w) && isnan(g))) {
        if (bad_f < 5) fprintf(stderr, "float a=%a n=%d want %a got %a\n", (double)a, n, (double)w, (double)g);
        bad_f++;
    }
}

int main(int argc, char **argv) {
    const long per = argc > 1 ? atol(argv[1]) : 200000;
    for (int n = 1; n <= 12; n++) {
        rcp_d[n] = 1.0 / (double)n;
        rcp_f[n] = 1.0f / (float)n;
    }
    for (int n = 1; n <= 12; n++) {
        for (long i = 0; i < per; i++) {
            const uint64_t r = next();
            /* any finite or special double: random sign, exponent, significand */
            check_d(d_of(r), n);
            check_f(f_of((uint32_t)(r >> 32)), n);
            /* magnitudes of coordinate sums: exponents near zero */
            const uint64_t m = r & 0xfffffffffffffull;
            const uint64_t ex = 1023 - 20 + (next() % 40);
            check_d(d_of((r & 0x8000000000000000ull) | (ex << 52) | m), n);
            const uint32_t mf = (uint32_t)(r >> 9) & 0x7fffffu, exf = 127 - 20 + (uint32_t)(next() % 40);
            check_f(f_of(((uint32_t)(r >> 32) & 0x80000000u) | (exf << 23) | mf), n);
            /* a = RN(n * M) for a midpoint M of the quotient's binade: quotients next to midpoints */
            const double M = d_of((ex << 52) | m) + ldexp(1.0, (int)ex - 1023 - 53);
            const double a = (double)n * M;
            check_d(a, n);
            check_d(nextafter(a, 0.0), n);
            check_d(nextafter(a, INFINITY), n);
            const float Mf = f_of((exf << 23) | mf) + ldexpf(1.0f, (int)exf - 127 - 24);
            const float af = (float)n * Mf;
            check_f(af, n);
            check_f(nextafterf(af, 0.0f), n);
            check_f(nextafterf(af, INFINITY), n);
        }
        /* thresholds, powers of two, the largest values, zeros, specials */
        for (int k = -1074; k <= 1023; k++) {
            const double p = ldexp(1.0, k);
            check_d(p, n); check_d(-p, n);
            check_d(nextafter(p, 0.0), n); check_d(nextafter(p, INFINITY), n);
            check_d(3.0 * p, n);
        }
        for (int k = -149; k <= 127; k++) {
            const float p = ldexpf(1.0f, k);
            check_f(p, n); check_f(-p, n);
            check_f(nextafterf(p, 0.0f), n); check_f(nextafterf(p, INFINITY), n);
            check_f(3.0f * p, n);
        }
        check_d(0.0, n); check_d(-0.0, n); check_d(INFINITY, n); check_d(-INFINITY, n); check_d(NAN, n);
        check_d(1.7976931348623157e308, n); check_d(-1.7976931348623157e308, n);
        check_f(0.0f, n); check_f(-0.0f, n); check_f(INFINITY, n); check_f(NAN, n);
        check_f(3.4028234663852886e38f, n);
    }
    printf("%ld %ld %ld\n", bad_d, bad_f, cases);
    return 0;
}
