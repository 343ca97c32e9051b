/*
 * oracle_math.h -- elementary functions and Julia-Base semantics for the CPU oracle.
 *
 * TEST INFRASTRUCTURE. This header belongs to the CPU oracle (a restatement of Wflow.jl's
 * algorithm used only to check the CUDA path). Product code never includes it.
 *
 * Julia-Base semantics reproduced here (the reference computes in Julia 1.12, Float64):
 *   - min/max propagate NaN and prefer -0.0 over +0.0 (Base.min/max for IEEEFloat).
 *   - clamp(x, lo, hi) = ifelse(x > hi, hi, ifelse(x < lo, lo, x)).
 *   - cld(x, y) for floats = round((x - mod(x, -y)) / y)   (Base.div(x, y, RoundUp)).
 *   - round(x; sigdigits) = round(x * 10^d) / 10^d, d = sigdigits - hidigit(x).
 *   - Wflow's own pow(x, y) = exp(y * log(x))            (Wflow/src/utils.jl:470).
 *
 * exp/log/cbrt: the reference uses Julia's libm. The oracle uses its own implementations
 * of published methods so that results do not depend on the host C library:
 *   - exp: Cody & Waite (1980) additive range reduction x = k*ln2 + r with a two-part ln2,
 *     |r| <= ln2/2, then the Taylor series of exp(r) to degree 13 in Horner form, scaled by
 *     2^k through the exponent field.
 *   - log: x = 2^e * m with m in [sqrt(2)/2, sqrt(2)), f = m - 1, s = f / (2 + f),
 *     log(1 + f) = 2 atanh(s) written as f - (f^2/2 - s (f^2/2 + R)), R = sum 2 s^(2i)/(2i+1)
 *     for i = 1..10, then + e*ln2 (two-part).
 *   - cbrt: exponent split plus Newton iterations y <- y - (y^3 - x) / (3 y^2).
 * Polynomial steps use fma(), which is correctly rounded on every IEEE platform, and the
 * oracle is compiled with -ffp-contract=off so that no other operation is fused.
 * Accuracy is within a few ulp of the exact result (checked in tests against Python's math).
 */
#ifndef WFLOW_ORACLE_MATH_H
#define WFLOW_ORACLE_MATH_H

#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

static inline double bits_to_double(uint64_t b) { double d; std::memcpy(&d, &b, 8); return d; }
static inline uint64_t double_to_bits(double d) { uint64_t b; std::memcpy(&b, &d, 8); return b; }

// Base.min / Base.max for Float64: NaN-propagating, -0.0 < +0.0.
static inline double jmin(double x, double y) {
    if (std::isnan(x) || std::isnan(y)) return x + y;
    if (x < y) return x;
    if (y < x) return y;
    return std::signbit(x) ? x : y;
}
static inline double jmax(double x, double y) {
    if (std::isnan(x) || std::isnan(y)) return x + y;
    if (x > y) return x;
    if (y > x) return y;
    return std::signbit(x) ? y : x;
}
static inline double jclamp(double x, double lo, double hi) {
    return x > hi ? hi : (x < lo ? lo : x);
}

// ---- exp (Cody-Waite reduction + Taylor polynomial) -----------------------------------
static const double kLn2Hi = 0x1.62e42fee00000p-1;   // ln2 with 21 low mantissa bits cleared
static const double kLn2Lo = 0x1.a39ef35793c76p-33;  // ln2 - kLn2Hi, rounded
static const double kInvLn2 = 0x1.71547652b82fep+0;  // 1/ln2 rounded

static inline double wexp(double x) {
    if (std::isnan(x)) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
    double k = std::nearbyint(x * kInvLn2);
    double r = (x - k * kLn2Hi) - k * kLn2Lo;
    // Taylor coefficients 1/j!, j = 13 .. 2
    double p = 0x1.6124613a86d09p-33;
    p = std::fma(p, r, 0x1.1eed8eff8d898p-29);
    p = std::fma(p, r, 0x1.ae64567f544e4p-26);
    p = std::fma(p, r, 0x1.27e4fb7789f5cp-22);
    p = std::fma(p, r, 0x1.71de3a556c734p-19);
    p = std::fma(p, r, 0x1.a01a01a01a01ap-16);
    p = std::fma(p, r, 0x1.a01a01a01a01ap-13);
    p = std::fma(p, r, 0x1.6c16c16c16c17p-10);
    p = std::fma(p, r, 0x1.1111111111111p-7);
    p = std::fma(p, r, 0x1.5555555555555p-5);
    p = std::fma(p, r, 0x1.5555555555555p-3);
    p = std::fma(p, r, 0.5);
    p = std::fma(p, r, 1.0);
    p = std::fma(p, r, 1.0);
    int ki = (int)k;
    if (ki > 1023) {
        return p * 0x1p1023 * bits_to_double((uint64_t)(ki - 1023 + 1023) << 52);
    }
    if (ki < -1022) {
        // subnormal result: scale in two steps
        return (p * bits_to_double((uint64_t)(ki + 1022 + 1023) << 52)) * 0x1p-1022;
    }
    return p * bits_to_double((uint64_t)(ki + 1023) << 52);
}

// ---- log (atanh series on [sqrt(2)/2, sqrt(2))) ----------------------------------------
static inline double wlog(double x) {
    if (std::isnan(x) || x < 0.0) return NAN;
    if (x == 0.0) return -INFINITY;
    if (std::isinf(x)) return x;
    int e = 0;
    uint64_t b = double_to_bits(x);
    if ((b >> 52) == 0) {  // subnormal
        x *= 0x1p54;
        b = double_to_bits(x);
        e = -54;
    }
    e += (int)((b >> 52) & 0x7ff) - 1023;
    double m = bits_to_double((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);  // [1,2)
    if (m > 0x1.6a09e667f3bcdp+0) {  // > sqrt(2)
        m *= 0.5;
        e += 1;
    }
    double f = m - 1.0;
    double s = f / (2.0 + f);
    double s2 = s * s;
    double R = 0x1.8618618618618p-4;             // 2/21
    R = std::fma(R, s2, 0x1.af286bca1af28p-4);   // 2/19
    R = std::fma(R, s2, 0x1.e1e1e1e1e1e1ep-4);   // 2/17
    R = std::fma(R, s2, 0x1.1111111111111p-3);   // 2/15
    R = std::fma(R, s2, 0x1.3b13b13b13b14p-3);   // 2/13
    R = std::fma(R, s2, 0x1.745d1745d1746p-3);   // 2/11
    R = std::fma(R, s2, 0x1.c71c71c71c71cp-3);   // 2/9
    R = std::fma(R, s2, 0x1.2492492492492p-2);   // 2/7
    R = std::fma(R, s2, 0x1.999999999999ap-2);   // 2/5
    R = std::fma(R, s2, 0x1.5555555555555p-1);   // 2/3
    R = R * s2;
    double hfsq = 0.5 * f * f;
    double lm = f - (hfsq - s * (hfsq + R));
    double de = (double)e;
    return de * kLn2Hi + (lm + de * kLn2Lo);
}

// ---- cbrt (exponent split + Newton) ----------------------------------------------------
static inline double wcbrt(double x) {
    if (std::isnan(x) || x == 0.0 || std::isinf(x)) return x;
    double ax = std::fabs(x);
    int e = 0;
    uint64_t b = double_to_bits(ax);
    if ((b >> 52) == 0) {
        ax *= 0x1p54;
        b = double_to_bits(ax);
        e = -54;
    }
    e += (int)((b >> 52) & 0x7ff) - 1023;
    double m = bits_to_double((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);  // [1,2)
    int r = ((e % 3) + 3) % 3;
    int q = (e - r) / 3;
    if (r == 1) m *= 2.0;
    if (r == 2) m *= 4.0;  // m in [1, 8)
    // linear first guess of m^(1/3) on [1, 8), then Newton
    double y = 0.6 + 0.2 * m;
    for (int i = 0; i < 6; ++i) y = y - (y * y * y - m) / (3.0 * y * y);
    y = y * bits_to_double((uint64_t)(q + 1023) << 52);
    return x < 0.0 ? -y : y;
}

// Wflow's pow (utils.jl:470): exp(y * log(x)).
static inline double jpow(double x, double y) { return wexp(y * wlog(x)); }

// Base.div(x, y, RoundUp) for Float64 (cld), x, y finite, y > 0:
//   round((x - mod(x, -y)) / y) with mod following the sign of -y.
static inline double jcld(double x, double y) {
    double r = std::fmod(x, -y);  // sign of x
    double m;
    if (r == 0.0) {
        m = std::copysign(0.0, -y);
    } else if ((r > 0.0) != (-y > 0.0)) {
        m = r + (-y);
    } else {
        m = r;
    }
    return std::nearbyint((x - m) / y);
}

// round(x; sigdigits = d) for finite x (Base._round_digits with hidigit by exact decade).
static inline double jround_sigdigits(double x, int sigdigits) {
    if (x == 0.0 || !std::isfinite(x)) return x;
    double ax = std::fabs(x);
    // hidigit = 1 + floor(log10(|x|)) using exact decade comparisons
    int hd;
    {
        int k = 0;
        double p = 1.0;
        if (ax >= 1.0) {
            while (ax >= p * 10.0 && k < 308) { p *= 10.0; ++k; }
        } else {
            while (ax < p && k > -330) { p /= 10.0; --k; }
        }
        hd = 1 + k;
    }
    int d = sigdigits - hd;
    if (d >= 0) {
        double sc = 1.0;
        for (int i = 0; i < d; ++i) sc *= 10.0;
        double y = std::nearbyint(x * sc) / sc;
        return std::isfinite(y) ? y : x;
    } else {
        double isc = 1.0;
        for (int i = 0; i < -d; ++i) isc *= 10.0;
        return std::nearbyint(x / isc) * isc;
    }
}

}  // namespace orc

#endif
