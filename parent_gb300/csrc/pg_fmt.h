// printf("%.12g") of a double, byte-identical to the C library's, as a
// function the device (the MIE text kernel) and the host (tests) share.
//
// |v| = m 2^e exactly (m < 2^53). With k = floor(log10 |v|), the twelve
// significant digits are D = round(|v| 10^(11-k)), 10^11 <= D < 10^12,
// rounded to nearest with ties to even (the C library rounds the exact binary
// value in the current rounding mode). D is formed exactly in 128-bit
// integers: m 5^s 2^(e+s) for s = 11 - k >= 0, m 2^(e-u) / 5^u for
// u = k - 11 > 0. k starts from the double log10 and moves by one while D
// falls outside [10^11, 10^12). The text then follows %g: style e when the
// exponent is below -4 or at least 12, else style f, trailing zeros and a
// bare decimal point removed, exponents with at least two digits.
// Exactness needs 5^s m < 2^128 (s <= 32) and m 2^(e-u) < 2^128: the range
// 1e-21 <= |v| < 1e47 is covered; anything else (and NaN/Inf) returns -1 so
// that the caller formats it with the C library.
#pragma once

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define PG_HD __host__ __device__ __forceinline__
#else
#define PG_HD inline
#endif

namespace pg {

typedef unsigned __int128 u128;

PG_HD u128 pow5_u128(int s) {
    u128 r = 1, b = 5;
    while (s) {
        if (s & 1) r *= b;
        b *= b;
        s >>= 1;
    }
    return r;
}

// round(n / d), ties to even (d > 0)
PG_HD uint64_t div_round_even(u128 n, u128 d) {
    const u128 q = n / d, r = n - q * d;
    const u128 r2 = r << 1;
    return (uint64_t)((r2 > d || (r2 == d && (q & 1))) ? q + 1 : q);
}

// round(m 2^e 10^s), ties to even; the result is known to be below ~2^44
PG_HD uint64_t scaled_round(uint64_t m, int e, int s) {
    if (s >= 0) {
        const u128 p = (u128)m * pow5_u128(s);
        const int t = e + s;
        if (t >= 0) return (uint64_t)(p << t);
        const int sh = -t;
        if (sh >= 128) return 0;
        const u128 q = p >> sh, r = p - (q << sh), half = (u128)1 << (sh - 1);
        return (uint64_t)((r > half || (r == half && (q & 1))) ? q + 1 : q);
    }
    const int u = -s, t = e - u;
    if (t >= 0) return div_round_even((u128)m << t, pow5_u128(u));
    return div_round_even((u128)m, pow5_u128(u) << (-t));
}

// Writes the %.12g text of v to o (no terminator) and returns its length,
// or -1 when v is outside the exact range (the caller then formats it).
PG_HD int format_g12(double v, char *o) {
    union {
        double d;
        uint64_t u;
    } cv;
    cv.d = v;
    const uint64_t bits = cv.u;
    const int ex = (int)((bits >> 52) & 0x7ff);
    const uint64_t fr = bits & ((1ull << 52) - 1);
    if (ex == 0x7ff) return -1;
    char *p = o;
    if (bits >> 63) *p++ = '-';
    if (ex == 0 && fr == 0) {
        *p++ = '0';
        return (int)(p - o);
    }
    const uint64_t m = ex ? (fr | (1ull << 52)) : fr;
    const int e = ex ? ex - 1075 : -1074;
    const double av = v < 0 ? -v : v;
    int k = (int)floor(log10(av));
    uint64_t D = 0;
    bool ok = false;
    for (int it = 0; it < 4; it++) {
        if (k < -21 || k > 46) return -1;
        D = scaled_round(m, e, 11 - k);
        if (D >= 1000000000000ull) {
            k++;
        } else if (D < 100000000000ull) {
            k--;
        } else {
            ok = true;
            break;
        }
    }
    if (!ok) return -1;
    char d[12];
    for (int i = 11; i >= 0; i--) {
        d[i] = (char)('0' + D % 10);
        D /= 10;
    }
    int last = 11;
    if (k < -4 || k >= 12) {
        while (last > 0 && d[last] == '0') last--;
        *p++ = d[0];
        if (last > 0) {
            *p++ = '.';
            for (int i = 1; i <= last; i++) *p++ = d[i];
        }
        *p++ = 'e';
        *p++ = k < 0 ? '-' : '+';
        const int ak = k < 0 ? -k : k;
        if (ak >= 100) *p++ = (char)('0' + ak / 100);
        *p++ = (char)('0' + (ak / 10) % 10);
        *p++ = (char)('0' + ak % 10);
    } else if (k >= 0) {
        while (last > k && d[last] == '0') last--;
        for (int i = 0; i <= k; i++) *p++ = d[i];
        if (last > k) {
            *p++ = '.';
            for (int i = k + 1; i <= last; i++) *p++ = d[i];
        }
    } else {
        while (last > 0 && d[last] == '0') last--;
        *p++ = '0';
        *p++ = '.';
        for (int i = 0; i < -k - 1; i++) *p++ = '0';
        for (int i = 0; i <= last; i++) *p++ = d[i];
    }
    return (int)(p - o);
}

}  // namespace pg
