// Double-FP32 complex arithmetic for the FP64 meshes' transforms.
//
// The GB300 issues FP64 at about 1/68 of its FP32 rate, so the FP64 mesh's
// z pass and inverse passes carry each complex value as an unevaluated sum
// of two FP32 complex numbers, hi + lo with |lo| <= ulp(hi)/2 per part
// (48 significant bits).  Sums use Knuth's two-sum on the high parts, the
// low parts added to its error and one renormalising fast two-sum (the
// "sloppy" double-word addition: its error is bounded by a few 2^-48 of
// |a| + |b|, which is the norm-wise bound a Fourier transform needs);
// products form the high product exactly with an FMA (Dekker's two-product
// by fused multiply-add) and add the cross terms in FP32.  The FP32 pairs
// use the paired FP32 instructions of sm_100 where one instruction covers
// both parts.  Nothing here is compiled with fast-math, so no step is
// reassociated or contracted.
#pragma once

#include <cuda_runtime.h>

#include "cells.cuh"

namespace sc {

struct __align__(16) ddc {
    float2 h, l;  // value = h + l, componentwise (x real part, y imaginary part)
};

__device__ __forceinline__ float2 dd_add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 dd_sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ void dd_two_sum(float2 a, float2 b, float2& s, float2& e) {
    s = dd_add2(a, b);
    const float2 bb = dd_sub2(s, a);
    e = dd_add2(dd_sub2(a, dd_sub2(s, bb)), dd_sub2(b, bb));
}
// h + l = s + e, with |e| small against |s|
__device__ __forceinline__ ddc dd_renorm(float2 s, float2 e) {
    const float2 h = dd_add2(s, e);
    return ddc{h, dd_sub2(e, dd_sub2(h, s))};
}

__device__ __forceinline__ ddc dd_add(ddc a, ddc b) {
    float2 s, e;
    dd_two_sum(a.h, b.h, s, e);
    return dd_renorm(s, dd_add2(e, dd_add2(a.l, b.l)));
}
__device__ __forceinline__ ddc dd_neg(ddc a) {
    return ddc{make_float2(-a.h.x, -a.h.y), make_float2(-a.l.x, -a.l.y)};
}
__device__ __forceinline__ ddc dd_sub(ddc a, ddc b) { return dd_add(a, dd_neg(b)); }

// the real products x*y (x = xh + xl, y = yh + yl) of both parts at once,
// returned as an unnormalised pair (p, e): p = xh*yh rounded, e its error
// plus the cross terms
__device__ __forceinline__ void dd_prod2(float2 xh, float2 xl, float2 yh, float2 yl, float2& p, float2& e) {
    p = __fmul2_rn(xh, yh);
    e = __ffma2_rn(xh, yh, make_float2(-p.x, -p.y));
    e = dd_add2(e, __ffma2_rn(xh, yl, __fmul2_rn(xl, yh)));
}

// complex product a * w (conj: a * conj(w))
template <bool CONJ>
__device__ __forceinline__ ddc dd_cmul_t(ddc a, ddc w) {
    // (ar + i ai)(wr + i wi): re = ar wr - ai wi, im = ar wi + ai wr
    const float wiy = CONJ ? -w.h.y : w.h.y, wly = CONJ ? -w.l.y : w.l.y;
    float2 p1, e1, p2, e2;
    // {ar wr, ar wi} and {ai wi, ai wr}
    dd_prod2(make_float2(a.h.x, a.h.x), make_float2(a.l.x, a.l.x), make_float2(w.h.x, wiy), make_float2(w.l.x, wly),
             p1, e1);
    dd_prod2(make_float2(a.h.y, a.h.y), make_float2(a.l.y, a.l.y), make_float2(wiy, w.h.x), make_float2(wly, w.l.x),
             p2, e2);
    // re = p1.x - p2.x, im = p1.y + p2.y
    const float2 q = make_float2(-p2.x, p2.y), f = make_float2(-e2.x, e2.y);
    float2 s, e;
    dd_two_sum(p1, q, s, e);
    return dd_renorm(s, dd_add2(e, dd_add2(e1, f)));
}
__device__ __forceinline__ ddc dd_cmul(ddc a, ddc w) { return dd_cmul_t<false>(a, w); }
__device__ __forceinline__ ddc dd_cmulc(ddc a, ddc w) { return dd_cmul_t<true>(a, w); }

// a times a real value g = gh + gl
__device__ __forceinline__ ddc dd_scale(ddc a, float gh, float gl) {
    float2 p, e;
    dd_prod2(a.h, a.l, make_float2(gh, gh), make_float2(gl, gl), p, e);
    return dd_renorm(p, e);
}

// A double split into hi + lo without FP64 instructions: hi keeps the top
// 24 significand bits (truncated), lo is the remaining 29 bits rounded to
// FP32, so hi + lo equals x to about 2^-47 relative.  Magnitudes outside
// [2^-74, 2^100] (and zero, subnormal or non-finite values) take the FP64
// conversion instead.
__device__ __forceinline__ void dd_split(double x, float& hi, float& lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e >= 1023 - 74 && e <= 1023 + 100) {
        const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
        hi = __uint_as_float(sgn | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)((b >> 29) & 0x7FFFFFu));
        const unsigned rem = (unsigned)(b & ((1ull << 29) - 1));  // weight 2^(e - 1075)
        const float pw = __uint_as_float((unsigned)(e - 1075 + 127) << 23);
        lo = __uint_as_float(__float_as_uint((float)rem * pw) | sgn);
        return;
    }
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

__device__ __forceinline__ ddc dd_from(double2 v) {
    ddc r;
    dd_split(v.x, r.h.x, r.l.x);
    dd_split(v.y, r.h.y, r.l.y);
    return r;
}
// back to FP64: the parts widened with integer operations, then one FP64
// addition per part
__device__ __forceinline__ double2 dd_to(ddc v) {
    return make_double2(f32_to_f64(v.h.x) + f32_to_f64(v.l.x), f32_to_f64(v.h.y) + f32_to_f64(v.l.y));
}


// loads and stores of a buffer between passes that holds FP64 (double2) or
// double-FP32 (ddc) values
__device__ __forceinline__ ddc dd_load(const double2* p) { return dd_from(*p); }
__device__ __forceinline__ ddc dd_load(const ddc* p) { return *p; }
__device__ __forceinline__ void dd_store(double2* p, ddc v) { *p = dd_to(v); }
__device__ __forceinline__ void dd_store(ddc* p, ddc v) { *p = v; }

}  // namespace sc
