// Double-FP32 arithmetic for the FP64 meshes' double-FP32 mode
// (sc_mesh_set_fp64_arithmetic).
//
// The GB300 issues FP64 at about 1/68 of its FP32 rate, so in that mode the
// FP64 mesh's transforms, deposit weights and gather carry each value as an
// unevaluated sum of two FP32 numbers, hi + lo with |lo| <= ulp(hi)/2 (48
// significant bits): complex values as ddc, real ones as dreal or a float2
// {hi, lo}.  Sums use Knuth's two-sum on the high parts, the
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

// A double split into hi + lo with integer operations only (split_f64 of
// cells.cuh: no FP64 instruction, not even in a branch the compiler could
// if-convert): hi keeps the top 24 significand bits (truncated), lo the
// remaining 29 rounded to FP32, so hi + lo equals x to 2^-47 relative
// within FP32's range (lo flushes below |x| ~ 2^-104, hi below 2^-126;
// +-inf from 2^128 on).
__device__ __forceinline__ void dd_split(double x, float& hi, float& lo) { split_f64(x, hi, lo); }
__device__ __forceinline__ void dd_split(float x, float& hi, float& lo) {
    hi = x;
    lo = 0.0f;
}

// An FP32 value widened to FP64 exactly, with integer operations only
__device__ __forceinline__ double dd_widen(float v) { return f32_to_f64(v); }

// A real double-FP32 value, for kernels written over a real type (the Green
// transform): the arithmetic of the complex pairs above, one lane.
struct __align__(8) dreal {
    float h, l;
    dreal() = default;
    __host__ __device__ constexpr dreal(float a, float b) : h(a), l(b) {}
    __host__ __device__ constexpr dreal(int v) : h((float)v), l(0.0f) {}  // |v| < 2^24
    __host__ __device__ constexpr dreal(float v) : h(v), l(0.0f) {}
    __host__ __device__ dreal(double v) {
#ifdef __CUDA_ARCH__
        dd_split(v, h, l);
#else
        h = (float)v;
        l = (float)(v - (double)h);
#endif
    }
};
__device__ __forceinline__ dreal dd_renorm1(float s, float e) {
    const float h = s + e;
    return dreal(h, e - (h - s));
}
__device__ __forceinline__ dreal operator+(dreal a, dreal b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb);
    return dd_renorm1(s, e + (a.l + b.l));
}
__device__ __forceinline__ dreal operator-(dreal a) { return dreal(-a.h, -a.l); }
__device__ __forceinline__ dreal operator-(dreal a, dreal b) { return a + (-b); }
__device__ __forceinline__ dreal operator*(dreal a, dreal b) {
    const float p = a.h * b.h;
    return dd_renorm1(p, fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p))));
}
// a / b: the FP32 quotient, corrected by one step on the double-FP32 residual
__device__ __forceinline__ dreal operator/(dreal a, dreal b) {
    const float q1 = a.h / b.h;
    const dreal r = a - b * dreal(q1);
    return dd_renorm1(q1, r.h / b.h);
}
__device__ __forceinline__ dreal& operator+=(dreal& a, dreal b) {
    a = a + b;
    return a;
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
    return make_double2(dd_widen(v.h.x) + dd_widen(v.l.x), dd_widen(v.h.y) + dd_widen(v.l.y));
}


// real double-FP32 values as float2 {hi, lo}: a * b, and 1 - a for a in [0, 1]
__device__ __forceinline__ float2 ddr_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    const float e = fmaf(a.x, b.y, fmaf(a.y, b.x, fmaf(a.x, b.x, -p)));
    const float h = p + e;
    return make_float2(h, e - (h - p));
}
// 1 - (h + l) for h + l in [0, 1]
__device__ __forceinline__ float2 ddr_one_minus(float2 a) {
    const float s = 1.0f - a.x;
    const float bb = s - 1.0f;
    const float e = ((1.0f - (s - bb)) + (-a.x - bb)) - a.y;
    const float h = s + e;
    return make_float2(h, e - (h - s));
}
// a real double-FP32 value to FP64
__device__ __forceinline__ double ddr_to(float2 v) { return dd_widen(v.x) + dd_widen(v.y); }

__device__ __forceinline__ double dd_f64(double x) { return x; }
__device__ __forceinline__ double dd_f64(float x) { return dd_widen(x); }

// The reference's i (decided in FP32 as in cell_df32) and its in-cell
// fraction f = (x - min)/delta - i in double-FP32, fh + fl: the cell's
// lower face min + i*delta by one FP64 FMA, r = x - face by one FP64
// subtraction (exact, or within 2^-53 of the cell, since x lies within a
// cell of the face), r split and multiplied by the FP64 1/delta split into
// ih + il.  f is then within about 2^-53 (i + 1) + 2^-47 f of the exact
// quotient, as close as the reference's FP64 division.  Near a face the
// exact FP64 division decides, and its f is split.
template <typename P>
__device__ __forceinline__ bool cell_dd(P x, const AxisP& a, int& i, float& fh, float& fl) {
    float xh, xr;
    dd_split(x, xh, xr);
    const float s = xh - a.loh;
    const float bb = s - xh;
    const float t = (xh - (s - bb)) + (-a.loh - bb);
    const float v = t + (xr - a.lol);
    const float qf = (s + v) * a.invf;
    const float fq = floorf(qf);
    const float m = 4.0e-7f * fabsf(qf) + a.mabs * (fabsf(xh) + fabsf(a.loh)) + 1e-30f;
    const float rq = qf - fq;
    if (rq < m || rq > 1.0f - m || !(fabsf(qf) < 1.6e7f)) {
        double fe;
        if (!cell_exact(x, a, i, fe)) return false;
        dd_split(fe, fh, fl);
        return true;
    }
    if (!(fq >= 0.0f && fq <= (float)(a.n - 2))) return false;
    i = (int)fq;
    const double face = fma(dd_widen(fq), a.delta, a.lo);
    float rh, rl;
    dd_split(dd_f64(x) - face, rh, rl);
    // (rh + rl) (ih + il)
    float ih, il;
    dd_split(a.inv, ih, il);
    const float ph = rh * ih;
    const float pl = fmaf(rh, il, fmaf(rl, ih, fmaf(rh, ih, -ph)));
    fh = ph + pl;
    fl = pl - (fh - ph);
    return true;
}

// loads and stores of a buffer between passes that holds FP64 (double2) or
// double-FP32 (ddc) values
__device__ __forceinline__ ddc dd_load(const double2* p) { return dd_from(*p); }
__device__ __forceinline__ ddc dd_load(const ddc* p) { return *p; }
__device__ __forceinline__ void dd_store(double2* p, ddc v) { *p = dd_to(v); }
__device__ __forceinline__ void dd_store(ddc* p, ddc v) { *p = v; }

}  // namespace sc
