// Float-float ("double-word") arithmetic on the FP32 pipes.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| at most a few ulp(hi): about 48
// significant bits.  GB300 executes FP64 at 1/64 of its FP32 rate, so the column kernels of the
// precision form, which need more than FP32 (the FC-Gram continuation amplifies rounding in the
// wall-adjacent rows by up to 1e4), compute in this format instead of FP64.
//
// Building blocks are the error-free transformations TwoSum (Knuth, TAOCP vol. 2) and
// Fast2Sum (Dekker 1971), and the FMA-based exact product; the compositions follow Joldes,
// Muller and Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic" (ACM TOMS 44, 2017):
//   add  (their SloppyDWPlusDW without its final renormalisation, 8 flops): error
//        <= ~3 u^2 (|a| + |b|), u = 2^-24 -- a normwise bound, which is what FFT butterflies
//        and sums need;
//   mul  (DWTimesDW with FMAs, 7 flops):   relative error <= ~5 u^2;
//   by a float (DWTimesFP, 6 flops).
// Nothing here relies on reassociation: nvcc keeps IEEE order without --use_fast_math, and the
// only contractions are the explicit fmaf calls.
#pragma once

#include <cuda_runtime.h>

namespace sg {

struct ff {
    float hi, lo;
    ff() = default;
    __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ constexpr ff(float h) : hi(h), lo(0.f) {}
    __host__ __device__ constexpr ff(int h) : hi((float)h), lo(0.f) {}
    // From a double: exact split of its top 48 bits.  Meant for constants (folded at compile
    // time) and host code; on the device a runtime double costs FP64 operations.
    __host__ __device__ constexpr explicit ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

// complex float-float (16 bytes: the footprint of a double2)
struct __align__(16) ffc {
    ff x, y;
};

// host: the float-float nearest to a long double value (tables computed in extended precision)
inline ff ff_split(long double v) {
    const float h = (float)v;
    return ff(h, (float)(v - (long double)h));
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    e = b - (s - a);
}

// Sums leave the pair unnormalised (|lo| may grow to a few ulp(hi) along a chain of additions):
// the leading words' rounding is still captured exactly by TwoSum, lo's own rounding is
// 2^-24 |lo|, and the products renormalise.  8 flops instead of 11.
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    return ff(s, e + (a.lo + b.lo));
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float h, l;
    fast_two_sum(p, e, h, l);
    return ff(h, l);
}
__device__ __forceinline__ ff ff_mulf(ff a, float b) {
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    float h, l;
    fast_two_sum(p, e, h, l);
    return ff(h, l);
}
// 1 / b: a float reciprocal refined by one Newton step in float-float
__device__ __forceinline__ ff ff_rcp(ff b) {
    const float r = 1.0f / b.hi;
    // residual 1 - b r, exact in its leading part by FMA
    const float e0 = fmaf(-b.hi, r, 1.0f);
    const float e1 = fmaf(-b.lo, r, e0);
    float h, l;
    fast_two_sum(r, r * e1, h, l);
    return ff(h, l);
}
__device__ __forceinline__ ff ff_div(ff a, ff b) { return ff_mul(a, ff_rcp(b)); }

__device__ __forceinline__ ff operator+(ff a, ff b) { return ff_add(a, b); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return ff_sub(a, b); }
__device__ __forceinline__ ff operator-(ff a) { return ff_neg(a); }
__device__ __forceinline__ ff operator*(ff a, ff b) { return ff_mul(a, b); }
__device__ __forceinline__ ff operator*(ff a, float b) { return ff_mulf(a, b); }
__device__ __forceinline__ ff operator*(float a, ff b) { return ff_mulf(b, a); }
__device__ __forceinline__ ff operator*(int a, ff b) { return ff_mulf(b, (float)a); }
__device__ __forceinline__ ff operator/(ff a, ff b) { return ff_div(a, b); }
__device__ __forceinline__ ff &operator+=(ff &a, ff b) { a = ff_add(a, b); return a; }
__device__ __forceinline__ ff &operator-=(ff &a, ff b) { a = ff_sub(a, b); return a; }
__device__ __forceinline__ ff &operator*=(ff &a, ff b) { a = ff_mul(a, b); return a; }
__device__ __forceinline__ ff &operator*=(ff &a, float b) { a = ff_mulf(a, b); return a; }

// a b + c d with one renormalisation: exact leading products (FMA), TwoSum of them, every
// lower-order term folded into the error word.  Normwise error ~u^2 (|a b| + |c d|): what a
// complex multiply in an FFT needs.
__device__ __forceinline__ ff ff_dot2(ff a, ff b, ff c, ff d) {
    const float p1 = a.hi * b.hi, p2 = c.hi * d.hi;
    const float e1 = fmaf(a.hi, b.hi, -p1), e2 = fmaf(c.hi, d.hi, -p2);
    float s, t;
    two_sum(p1, p2, s, t);
    t += e1 + e2;
    t = fmaf(a.hi, b.lo, t);
    t = fmaf(a.lo, b.hi, t);
    t = fmaf(c.hi, d.lo, t);
    t = fmaf(c.lo, d.hi, t);
    float h, l;
    fast_two_sum(s, t, h, l);
    return ff(h, l);
}

// complex float-float product: 38 flops (four exact products, two TwoSums)
__device__ __forceinline__ ffc cmul(ffc a, ffc b) {
    ffc r;
    r.x = ff_dot2(a.x, b.x, ff_neg(a.y), b.y);
    r.y = ff_dot2(a.x, b.y, a.y, b.x);
    return r;
}

// conversions with FP64 (FP64 pipe: use at kernel boundaries only)
__device__ __forceinline__ ff ff_from_double(double d) {
    const float h = __double2float_rn(d);
    return ff(h, __double2float_rn(d - (double)h));
}
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

}  // namespace sg
