// wf_ff.cuh -- double-FP32 ("float-float") arithmetic for the latency-critical sweeps.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2, which
// carries about 48 significant bits. GB300 executes a dependent FP64 instruction in 64 cycles
// and one FP64 warp instruction per ~64-80 cycles per scheduler, against 4 cycles for FP32, so
// the routing wavefronts (whose critical path is a chain of dependent solves) keep their
// discharge state and the kinematic-wave correction step in this representation and touch the
// FP64 unit not at all. The error-free transformations are the standard ones: TwoSum
// (Knuth), Fast2Sum (Dekker, |a| >= |b|) and TwoProd via a fused multiply-add.
#pragma once

#include <cstdint>

namespace wff {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = a + b;
    const float bp = s - a;
    const float e = (a - (s - bp)) + (b - bp);
    return {s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ ff add(ff a, ff b) {
    ff s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff add(ff a, float b) {
    ff s = two_sum(a.hi, b);
    s.lo += a.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff neg(ff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ ff mul(ff a, ff b) {
    ff p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ff mul(ff a, float b) {
    ff p = two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ff sub(ff a, ff b) { return add(a, neg(b)); }
__device__ __forceinline__ ff sub(ff a, float b) { return add(a, -b); }
// a / b with one Newton correction of the FP32 quotient (about 44 bits)
__device__ __forceinline__ ff div(ff a, ff b) {
    const float q1 = __fdividef(a.hi, b.hi);
    const ff r = sub(a, mul(b, q1));
    const float q2 = __fdividef(r.hi, b.hi);
    return fast_two_sum(q1, q2);
}
__device__ __forceinline__ ff div(ff a, float b) { return div(a, ff{b, 0.0f}); }
__device__ __forceinline__ bool lt(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool gt(ff a, ff b) { return lt(b, a); }
__device__ __forceinline__ bool le(ff a, ff b) { return !lt(b, a); }
__device__ __forceinline__ ff fmin(ff a, ff b) { return lt(b, a) ? b : a; }
__device__ __forceinline__ ff fmax(ff a, ff b) { return lt(a, b) ? b : a; }
__device__ __forceinline__ ff fmax0(ff a) { return a.hi > 0.0f ? a : ff{0.0f, 0.0f}; }
__device__ __forceinline__ float to_f(ff a) { return a.hi + a.lo; }
__device__ __forceinline__ ff from_f(float x) { return {x, 0.0f}; }
__device__ __forceinline__ ff ld(const float* h, const float* l, int64_t i) { return {h[i], l[i]}; }
__device__ __forceinline__ void st(float* h, float* l, int64_t i, ff v) {
    h[i] = v.hi;
    l[i] = v.lo;
}
__host__ __device__ __forceinline__ double to_d(ff a) { return (double)a.hi + (double)a.lo; }
__host__ __device__ __forceinline__ ff from_d(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ bool is_zero(ff a) { return a.hi == 0.0f; }

// 64-bit word holding an ff value (hi in the low half), for single-copy-atomic hand-off.
__device__ __forceinline__ unsigned long long pack(ff a) {
    return (unsigned long long)(uint32_t)__float_as_uint(a.hi) |
           ((unsigned long long)(uint32_t)__float_as_uint(a.lo) << 32);
}
__device__ __forceinline__ ff unpack(unsigned long long w) {
    return {__uint_as_float((uint32_t)(w & 0xffffffffULL)), __uint_as_float((uint32_t)(w >> 32))};
}

}  // namespace wff
