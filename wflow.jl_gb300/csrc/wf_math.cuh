// wf_math.cuh -- FP64 elementary functions and Julia-Base semantics used by the kernels.
//
// The FP64 form must reproduce Wflow.jl's Float64 arithmetic. Julia's Base semantics that
// matter on the path:
//   * min/max propagate NaN and order -0.0 < +0.0;
//   * clamp(x, lo, hi) = x > hi ? hi : (x < lo ? lo : x);
//   * cld(x, y) for floats = round((x - mod(x, -y)) / y)   (Base.div(x, y, RoundUp));
//   * round(x; sigdigits = d) = round(x * 10^k) / 10^k with k = d - hidigit(x);
//   * Wflow's pow(x, y) = exp(y * log(x))  (Wflow/src/utils.jl:470).
// exp/log/cbrt are implemented here from published methods so that host and device give
// identical results for identical inputs and no vendor math routine is involved:
//   * exp: Cody & Waite (1980) reduction x = k*ln2 + r with ln2 split in two, Taylor series of
//     exp(r) to degree 13, scaling by 2^k through the exponent bits;
//   * log: x = 2^e m, m in [sqrt(2)/2, sqrt(2)), f = m - 1, s = f/(2+f),
//     log(1+f) = f - (f^2/2 - s (f^2/2 + R)), R = sum_{i=1..10} 2 s^(2i) / (2i+1);
//   * cbrt: split off the exponent in thirds, Newton iterations on y^3 = m.
// Polynomials use explicit fma(); the translation units that include this header for the
// FP64 form are compiled with --fmad=false so nothing else is contracted.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define WF_HD __host__ __device__ __forceinline__
#else
#define WF_HD inline
#endif

#include <cmath>
#include <cstring>

namespace wfm {

WF_HD double from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    std::memcpy(&d, &b, 8);
    return d;
#endif
}
WF_HD uint64_t to_bits(double d) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    std::memcpy(&b, &d, 8);
    return b;
#endif
}
WF_HD bool isnan_(double x) { return x != x; }
WF_HD bool signbit_(double x) { return (to_bits(x) >> 63) != 0; }
WF_HD double fabs_(double x) { return from_bits(to_bits(x) & 0x7fffffffffffffffULL); }
WF_HD double rint_(double x) {
#ifdef __CUDA_ARCH__
    return rint(x);
#else
    return std::nearbyint(x);
#endif
}
WF_HD double fma_(double a, double b, double c) {
#ifdef __CUDA_ARCH__
    return __fma_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
WF_HD double fmod_(double x, double y) {
#ifdef __CUDA_ARCH__
    return fmod(x, y);
#else
    return std::fmod(x, y);
#endif
}
WF_HD double trunc_(double x) {
#ifdef __CUDA_ARCH__
    return trunc(x);
#else
    return std::trunc(x);
#endif
}
WF_HD double ceil_(double x) {
#ifdef __CUDA_ARCH__
    return ceil(x);
#else
    return std::ceil(x);
#endif
}
WF_HD double sqrt_(double x) {
#ifdef __CUDA_ARCH__
    return __dsqrt_rn(x);
#else
    return std::sqrt(x);
#endif
}
WF_HD double copysign_(double x, double s) {
    return from_bits((to_bits(x) & 0x7fffffffffffffffULL) | (to_bits(s) & 0x8000000000000000ULL));
}

// Julia Base.min / Base.max / clamp for Float64
WF_HD double jmin(double x, double y) {
    if (isnan_(x) || isnan_(y)) return x + y;
    if (x < y) return x;
    if (y < x) return y;
    return signbit_(x) ? x : y;
}
WF_HD double jmax(double x, double y) {
    if (isnan_(x) || isnan_(y)) return x + y;
    if (x > y) return x;
    if (y > x) return y;
    return signbit_(x) ? y : x;
}
WF_HD double jclamp(double x, double lo, double hi) { return x > hi ? hi : (x < lo ? lo : x); }

constexpr double LN2_HI = 0x1.62e42fee00000p-1;
constexpr double LN2_LO = 0x1.a39ef35793c76p-33;
constexpr double INV_LN2 = 0x1.71547652b82fep+0;

WF_HD double exp(double x) {
    if (isnan_(x)) return x;
    if (x > 709.782712893384) return from_bits(0x7ff0000000000000ULL);
    if (x < -745.1332191019412) return 0.0;
    const double k = rint_(x * INV_LN2);
    const double r = (x - k * LN2_HI) - k * LN2_LO;
    double p = 0x1.6124613a86d09p-33;            // 1/13!
    p = fma_(p, r, 0x1.1eed8eff8d898p-29);       // 1/12!
    p = fma_(p, r, 0x1.ae64567f544e4p-26);       // 1/11!
    p = fma_(p, r, 0x1.27e4fb7789f5cp-22);       // 1/10!
    p = fma_(p, r, 0x1.71de3a556c734p-19);       // 1/9!
    p = fma_(p, r, 0x1.a01a01a01a01ap-16);       // 1/8!
    p = fma_(p, r, 0x1.a01a01a01a01ap-13);       // 1/7!
    p = fma_(p, r, 0x1.6c16c16c16c17p-10);       // 1/6!
    p = fma_(p, r, 0x1.1111111111111p-7);        // 1/5!
    p = fma_(p, r, 0x1.5555555555555p-5);        // 1/4!
    p = fma_(p, r, 0x1.5555555555555p-3);        // 1/3!
    p = fma_(p, r, 0.5);
    p = fma_(p, r, 1.0);
    p = fma_(p, r, 1.0);
    const int ki = (int)k;
    if (ki > 1023) return p * 0x1p1023 * from_bits((uint64_t)ki << 52);
    if (ki < -1022) return (p * from_bits((uint64_t)(ki + 1022 + 1023) << 52)) * 0x1p-1022;
    return p * from_bits((uint64_t)(ki + 1023) << 52);
}

WF_HD double log(double x) {
    if (isnan_(x) || x < 0.0) return from_bits(0x7ff8000000000000ULL);
    if (x == 0.0) return -from_bits(0x7ff0000000000000ULL);
    if (x == from_bits(0x7ff0000000000000ULL)) return x;
    int e = 0;
    uint64_t b = to_bits(x);
    if ((b >> 52) == 0) {
        x *= 0x1p54;
        b = to_bits(x);
        e = -54;
    }
    e += (int)((b >> 52) & 0x7ff) - 1023;
    double m = from_bits((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    if (m > 0x1.6a09e667f3bcdp+0) {
        m *= 0.5;
        e += 1;
    }
    const double f = m - 1.0;
    const double s = f / (2.0 + f);
    const double s2 = s * s;
    double R = 0x1.8618618618618p-4;        // 2/21
    R = fma_(R, s2, 0x1.af286bca1af28p-4);  // 2/19
    R = fma_(R, s2, 0x1.e1e1e1e1e1e1ep-4);  // 2/17
    R = fma_(R, s2, 0x1.1111111111111p-3);  // 2/15
    R = fma_(R, s2, 0x1.3b13b13b13b14p-3);  // 2/13
    R = fma_(R, s2, 0x1.745d1745d1746p-3);  // 2/11
    R = fma_(R, s2, 0x1.c71c71c71c71cp-3);  // 2/9
    R = fma_(R, s2, 0x1.2492492492492p-2);  // 2/7
    R = fma_(R, s2, 0x1.999999999999ap-2);  // 2/5
    R = fma_(R, s2, 0x1.5555555555555p-1);  // 2/3
    R = R * s2;
    const double hfsq = 0.5 * f * f;
    const double lm = f - (hfsq - s * (hfsq + R));
    const double de = (double)e;
    return de * LN2_HI + (lm + de * LN2_LO);
}

WF_HD double cbrt(double x) {
    if (isnan_(x) || x == 0.0 || fabs_(x) == from_bits(0x7ff0000000000000ULL)) return x;
    double ax = fabs_(x);
    int e = 0;
    uint64_t b = to_bits(ax);
    if ((b >> 52) == 0) {
        ax *= 0x1p54;
        b = to_bits(ax);
        e = -54;
    }
    e += (int)((b >> 52) & 0x7ff) - 1023;
    double m = from_bits((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    const int r = ((e % 3) + 3) % 3;
    const int q = (e - r) / 3;
    if (r == 1) m *= 2.0;
    if (r == 2) m *= 4.0;
    double y = 0.6 + 0.2 * m;
    for (int i = 0; i < 6; ++i) y = y - (y * y * y - m) / (3.0 * y * y);
    y = y * from_bits((uint64_t)(q + 1023) << 52);
    return x < 0.0 ? -y : y;
}

// Wflow.pow (utils.jl:470)
WF_HD double pow(double x, double y) { return exp(y * log(x)); }

// Base.div(x, y, RoundUp) (cld) for y > 0
WF_HD double cld(double x, double y) {
    const double r = fmod_(x, -y);
    double m;
    if (r == 0.0) {
        m = copysign_(0.0, -y);
    } else if ((r > 0.0) != (-y > 0.0)) {
        m = r + (-y);
    } else {
        m = r;
    }
    return rint_((x - m) / y);
}

// round(x; sigdigits = d) for finite x >= 0 (the path only rounds |dz| / 0.1)
WF_HD double round_sigdigits(double x, int sigdigits) {
    if (x == 0.0 || isnan_(x) || fabs_(x) == from_bits(0x7ff0000000000000ULL)) return x;
    const double ax = fabs_(x);
    int k = 0;
    double p = 1.0;
    if (ax >= 1.0) {
        while (ax >= p * 10.0 && k < 308) {
            p *= 10.0;
            ++k;
        }
    } else {
        while (ax < p && k > -330) {
            p /= 10.0;
            --k;
        }
    }
    const int d = sigdigits - (1 + k);
    if (d >= 0) {
        double sc = 1.0;
        for (int i = 0; i < d; ++i) sc *= 10.0;
        const double y = rint_(x * sc) / sc;
        return (y - y == 0.0) ? y : x;
    }
    double isc = 1.0;
    for (int i = 0; i < -d; ++i) isc *= 10.0;
    return rint_(x / isc) * isc;
}

}  // namespace wfm
