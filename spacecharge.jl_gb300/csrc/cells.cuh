// Cell-index and CIC-weight arithmetic shared by the deposit, gather and
// adjoint kernels.
//
// The reference computes, per axis (src/deposition.jl:39-51,
// src/interpolation.jl:31-43):
//     norm = (x - min) / delta      (FP64, IEEE division)
//     i    = floor(Int, norm)
//     f    = norm - i
// `cell_exact` restates that.  `cell_df32` returns the same i with an
// FP32-precision f while issuing no FP64 instruction in the common case
// (GB300 has ~1/64 of its FP32 rate in FP64): x - min is formed in
// double-FP32 (Dekker/Knuth two-sum) from an integer split of the FP64
// input, the quotient is estimated in FP32, and whenever the estimate lies
// within its error bound of an integer the exact FP64 division decides.
#pragma once

#include <stdint.h>

namespace sc {

struct AxisP {
    double lo, delta;  // exact mesh geometry (FP64)
    double inv;        // 1/delta rounded to FP64
    float loh, lol;    // lo = loh + lol (+ <2^-48 |lo|)
    float dh, dl;      // delta = dh + dl
    float invf;        // 1/delta rounded to FP32
    float mabs;        // absolute term of the estimate's error bound, per |x|
    int n;             // nodes on this axis
};

struct Axes {
    AxisP a[3];
};

// Host-side construction (also used by tests through the ABI indirectly).
inline AxisP make_axis(double lo, double delta, int n) {
    AxisP p;
    p.lo = lo;
    p.delta = delta;
    p.inv = 1.0 / delta;
    p.loh = (float)lo;
    p.lol = (float)(lo - (double)p.loh);
    p.dh = (float)delta;
    p.dl = (float)(delta - (double)p.dh);
    p.invf = (float)(1.0 / delta);
    // |error of the double-FP32 offset| <= ~2^-46 (|x| + |lo|); in cells that
    // is 2^-46 (|x| + |lo|) / delta.  Use 2^-42 for headroom.
    p.mabs = (float)(2.2737367544323206e-13 / delta);
    p.n = n;
    return p;
}

// ------------------------------------------------ FP64 <-> FP32 with INT ops
// These issue no FP64 instruction on any path: the GB300's FP64 pipe is
// slow enough that even a conversion in a rarely taken branch, once the
// compiler turns the branch into predicated code, is paid on every call.
//
// x = h + r exactly up to the rounding of r: h is x truncated to 24
// significant bits, r the remainder rounded to FP32.  Outside the FP32
// normal range h is +-0 (|x| < 2^-126) or +-inf (|x| >= 2^128; NaN stays
// NaN), with r = 0; below |x| ~ 2^-104 r flushes to zero.
__device__ __forceinline__ void split_f64(double x, float& h, float& r) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7FF);
    const unsigned sgn = hi & 0x80000000u;
    const unsigned top = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // 23 fraction bits
    unsigned hb;
    if (e >= 1023 - 126 && e <= 1023 + 127)
        hb = sgn | ((unsigned)(e - 1023 + 127) << 23) | top;
    else if (e < 1023 - 126)
        hb = sgn;
    else
        hb = sgn | 0x7F800000u | ((e == 2047 && (top | (lo & 0x1FFFFFFFu))) ? 0x400000u : 0u);
    h = __uint_as_float(hb);
    // remainder: (lo & (2^29-1)) * 2^(e-1075), formed as (m * 2^-29) *
    // 2^(e-1046)
    const unsigned m = lo & 0x1FFFFFFFu;
    const float mf = __uint2float_rn(m) * 1.862645149230957e-09f;  // m * 2^-29
    const int pe = e - 1075 + 29 + 127;                             // biased exponent of 2^(e-1046)
    const float scale = (pe > 0 && e <= 1023 + 127) ? __uint_as_float((unsigned)pe << 23) : 0.0f;
    r = __uint_as_float(__float_as_uint(mf * scale) | sgn);
}
__device__ __forceinline__ void split_f64(float x, float& h, float& r) {
    h = x;
    r = 0.0f;
}

// Round an FP64 value to FP32 (nearest, ties away) with integer ops only;
// below the FP32 normal range +-0, from 2^128 on +-inf (NaN stays NaN).
__device__ __forceinline__ float f64_to_f32(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7FF);
    const unsigned sgn = hi & 0x80000000u;
    const unsigned top = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    unsigned f;
    if (e >= 1023 - 126 && e <= 1023 + 127)
        f = (((unsigned)(e - 1023 + 127) << 23) | top) + ((lo >> 28) & 1u);  // round half away; a carry
                                                                            // may bump the exponent (to inf)
    else if (e < 1023 - 126)
        f = 0u;
    else
        f = 0x7F800000u | ((e == 2047 && (top | (lo & 0x1FFFFFFFu))) ? 0x400000u : 0u);
    return __uint_as_float(sgn | f);
}
__device__ __forceinline__ float f64_to_f32(float x) { return x; }

// Widen an FP32 value to FP64 exactly with integer ops only (zeros,
// subnormals, infinities and NaN included).
__device__ __forceinline__ double f32_to_f64(float v) {
    const unsigned u = __float_as_uint(v);
    const unsigned e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    const unsigned long long sg = (unsigned long long)(u & 0x80000000u) << 32;
    unsigned long long b;
    if (e != 0 && e != 0xFF) {
        b = sg | ((unsigned long long)(e + 896) << 52) | ((unsigned long long)m << 29);
    } else if (e == 0xFF) {
        b = sg | (0x7FFull << 52) | ((unsigned long long)m << 29);
    } else if (m == 0) {
        b = sg;
    } else {  // subnormal: m * 2^-149, normalised
        const int lz = __clz(m);
        b = sg | ((unsigned long long)(905 - lz) << 52) | ((unsigned long long)((m << (lz - 8)) & 0x7FFFFFu) << 29);
    }
    return __longlong_as_double((long long)b);
}

template <typename P>
__device__ __forceinline__ P store_cast(float v);
template <>
__device__ __forceinline__ float store_cast<float>(float v) { return v; }
template <>
__device__ __forceinline__ double store_cast<double>(float v) { return f32_to_f64(v); }

// ------------------------------------------------------ cell computations
// Reference arithmetic: returns false when the particle's cell is not in
// [0, n-2] (the reference writes out of bounds there; we skip).
template <typename P>
__device__ __forceinline__ bool cell_exact(P x, const AxisP& a, int& i, double& f) {
    const double norm = ((double)x - a.lo) / a.delta;
    const double fl = floor(norm);
    if (!(fl >= 0.0 && fl <= (double)(a.n - 2))) return false;  // also rejects NaN
    i = (int)fl;
    f = norm - fl;
    return true;
}

// FP64 estimate by multiplication with 1/delta, exact division near faces.
template <typename P>
__device__ __forceinline__ bool cell_dp(P x, const AxisP& a, int& i, double& f) {
    const double d = (double)x - a.lo;
    double q = d * a.inv;
    double fl = floor(q);
    double r = q - fl;
    const double m = 1e-12 * (fabs(q) + 1.0);
    if (r < m || r > 1.0 - m) {
        q = d / a.delta;
        fl = floor(q);
        r = q - fl;
    }
    if (!(fl >= 0.0 && fl <= (double)(a.n - 2))) return false;
    i = (int)fl;
    f = r;
    return true;
}

// Double-FP32 estimate, no FP64 instruction unless within the error bound
// of a face.  Returns the reference's i and f rounded to ~1e-7.
template <typename P>
__device__ __forceinline__ bool cell_df32(P x, const AxisP& a, int& i, float& f) {
    float xh, xr;
    split_f64(x, xh, xr);
    // two-sum: s + t = xh - loh exactly
    const float s = xh - a.loh;
    const float bb = s - xh;
    const float t = (xh - (s - bb)) + (-a.loh - bb);
    const float v = t + (xr - a.lol);
    const float qf = (s + v) * a.invf;
    const float fl = floorf(qf);
    // bound on |qf - q_ref|: ~3 ulp relative plus the absolute split error
    const float m = 4.0e-7f * fabsf(qf) + a.mabs * (fabsf(xh) + fabsf(a.loh)) + 1e-30f;
    float r = qf - fl;
    if (r < m || r > 1.0f - m || !(fabsf(qf) < 1.6e7f)) {
        double fe;
        if (!cell_exact(x, a, i, fe)) return false;
        f = f64_to_f32(fe);
        return true;
    }
    if (!(fl >= 0.0f && fl <= (float)(a.n - 2))) return false;
    i = (int)fl;
    // in-cell fraction from the double-FP32 offset: (d - i*delta) / delta
    const float g = fmaf(-fl, a.dh, s) + fmaf(-fl, a.dl, v);
    f = fminf(fmaxf(g * a.invf, 0.0f), 1.0f);
    return true;
}

}  // namespace sc
