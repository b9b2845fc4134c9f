// Shared-memory batched FFT building blocks for the hand-written pruned
// convolution.  A CTA holds `ncol` columns of a power-of-two length L in
// shared memory, element (j, col) at [j * ncol + col], and transforms all of
// them with Stockham autosort stages (radix 16 butterflies in registers, one
// radix 2/4/8 stage for the remainder) ping-ponging between two buffers.  Twiddles come from a
// per-device table of exp(-2 pi i k / kMaxL) rounded once from FP64, so the
// FP32 transform uses correctly rounded roots of unity.
#pragma once

#include <type_traits>

#include "dd.cuh"
#include "sc_internal.cuh"

namespace sc {

template <typename T>
struct Cplx;
template <>
struct Cplx<float> {
    using T2 = float2;
    __device__ __forceinline__ static float2 make(float a, float b) { return make_float2(a, b); }
};
template <>
struct Cplx<double> {
    using T2 = double2;
    __device__ __forceinline__ static double2 make(double a, double b) { return make_double2(a, b); }
};
template <>
struct Cplx<dreal> {
    using T2 = ddc;
    __device__ __forceinline__ static ddc make(dreal a, dreal b) {
        return ddc{make_float2(a.h, b.h), make_float2(a.l, b.l)};
    }
};

// Real and imaginary parts, and loads of a real value, for kernels written
// over the real type (float, double or dreal)
__device__ __forceinline__ float c_re(float2 v) { return v.x; }
__device__ __forceinline__ float c_im(float2 v) { return v.y; }
__device__ __forceinline__ double c_re(double2 v) { return v.x; }
__device__ __forceinline__ double c_im(double2 v) { return v.y; }
__device__ __forceinline__ dreal c_re(ddc v) { return dreal(v.h.x, v.l.x); }
__device__ __forceinline__ dreal c_im(ddc v) { return dreal(v.h.y, v.l.y); }
template <typename T>
__device__ __forceinline__ T ldg_r(const T* p) {
    return __ldg(p);
}
template <>
__device__ __forceinline__ dreal ldg_r<dreal>(const dreal* p) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return dreal(v.x, v.y);
}
template <typename T>
__device__ __forceinline__ T ldcg_r(const T* p) {
    return __ldcg(p);
}
template <>
__device__ __forceinline__ dreal ldcg_r<dreal>(const dreal* p) {
    const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
    return dreal(v.x, v.y);
}

// Complex add and subtract.  FP32 pairs use the paired FP32 instructions of
// sm_100 and later (one instruction for both lanes of a float2, each lane
// rounded as the scalar operation); a - b is the exact fma(b, -1, a).
template <typename T2>
__device__ __forceinline__ T2 cadd(T2 a, T2 b) {
    if constexpr (std::is_same<T2, float2>::value) {
        return __fadd2_rn(a, b);
    } else if constexpr (std::is_same<T2, ddc>::value) {
        return dd_add(a, b);
    } else {
        a.x += b.x;
        a.y += b.y;
        return a;
    }
}
template <typename T2>
__device__ __forceinline__ T2 csub(T2 a, T2 b) {
    if constexpr (std::is_same<T2, float2>::value) {
        return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
    } else if constexpr (std::is_same<T2, ddc>::value) {
        return dd_sub(a, b);
    } else {
        a.x -= b.x;
        a.y -= b.y;
        return a;
    }
}
template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
    if constexpr (std::is_same<T2, ddc>::value) {
        return dd_cmul(a, b);
    } else {
        T2 r;
        r.x = a.x * b.x - a.y * b.y;
        r.y = a.x * b.y + a.y * b.x;
        return r;
    }
}
// a * conj(b)
template <typename T2>
__device__ __forceinline__ T2 cmulc(T2 a, T2 b) {
    if constexpr (std::is_same<T2, ddc>::value) {
        return dd_cmulc(a, b);
    } else {
        T2 r;
        r.x = a.x * b.x + a.y * b.y;
        r.y = a.y * b.x - a.x * b.y;
        return r;
    }
}
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename T2>
__device__ __forceinline__ T2 rot(T2 d) {
    if constexpr (std::is_same<T2, ddc>::value) {
        return INV ? ddc{make_float2(-d.h.y, d.h.x), make_float2(-d.l.y, d.l.x)}
                   : ddc{make_float2(d.h.y, -d.h.x), make_float2(d.l.y, -d.l.x)};
    } else {
        T2 r;
        if (INV) {
            r.x = -d.y;
            r.y = d.x;
        } else {
            r.x = d.y;
            r.y = -d.x;
        }
        return r;
    }
}

// Twiddles of the in-register butterflies: cos/sin(2 pi k / 16), k < 8.
__host__ __device__ constexpr double c16(int k) {
    return k == 0 ? 1.0
         : k == 1 ? 0.92387953251128675613
         : k == 2 ? 0.70710678118654752440
         : k == 3 ? 0.38268343236508977173
         : k == 4 ? 0.0
         : k == 5 ? -0.38268343236508977173
         : k == 6 ? -0.70710678118654752440
                  : -0.92387953251128675613;
}
// sin(2 pi k / 16) = cos(2 pi (k - 4) / 16)
__host__ __device__ constexpr double s16(int k) { return k == 0 ? 0.0 : c16(k <= 4 ? 4 - k : k - 4); }

// v * exp(-+2 pi i k / R) for a compile-time R in {2, 4, 8, 16} and k < R/2
template <int R, int K, bool INV, typename T2>
__device__ __forceinline__ T2 twc(T2 v) {
    constexpr int k16 = K * (16 / R);  // same angle on the 16-point circle
    if (k16 == 0) return v;
    if (k16 == 4) return rot<INV>(v);  // -+i
    constexpr double cd = c16(k16), sd = s16(k16);
    if constexpr (std::is_same<T2, ddc>::value) {
        // the constant (c, s) as double-FP32
        constexpr double sdd = INV ? sd : -sd;
        constexpr float ch = (float)cd, sh = (float)sdd;
        constexpr float cl = (float)(cd - (double)ch), sl = (float)(sdd - (double)sh);
        return dd_cmul(v, ddc{make_float2(ch, sh), make_float2(cl, sl)});
    } else {
        using T = decltype(v.x);
        const T c = (T)cd, s = INV ? (T)sd : -(T)sd;
        T2 r;
        r.x = v.x * c - v.y * s;
        r.y = v.x * s + v.y * c;
        return r;
    }
}

template <bool INV, typename T2>
__device__ __forceinline__ void dft2(T2& a, T2& b) {
    const T2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}
template <bool INV, typename T2>
__device__ __forceinline__ void dft4(T2& v0, T2& v1, T2& v2, T2& v3) {
    const T2 a0 = cadd(v0, v2), a1 = csub(v0, v2);
    const T2 a2 = cadd(v1, v3);
    v0 = cadd(a0, a2);
    v2 = csub(a0, a2);
    if constexpr (std::is_same<T2, float2>::value) {
        // a1 +- rot(d) lane by lane: the rotation swaps the lanes, which a
        // paired instruction cannot do without moves
        const T2 d = csub(v1, v3);
        const float dy = INV ? -d.y : d.y, dx = INV ? -d.x : d.x;
        v1 = make_float2(a1.x + dy, a1.y - dx);
        v3 = make_float2(a1.x - dy, a1.y + dx);
    } else {
        const T2 a3 = rot<INV>(csub(v1, v3));
        v1 = cadd(a1, a3);
        v3 = csub(a1, a3);
    }
}
template <bool INV, typename T2>
__device__ __forceinline__ void dft8(T2* v) {
    T2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    T2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    o1 = twc<8, 1, INV>(o1);
    o2 = twc<8, 2, INV>(o2);
    o3 = twc<8, 3, INV>(o3);
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}
template <bool INV, typename T2>
__device__ __forceinline__ void dft16(T2* v) {
    T2 e[8], o[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        e[k] = v[2 * k];
        o[k] = v[2 * k + 1];
    }
    dft8<INV>(e);
    dft8<INV>(o);
    o[1] = twc<16, 1, INV>(o[1]);
    o[2] = twc<16, 2, INV>(o[2]);
    o[3] = twc<16, 3, INV>(o[3]);
    o[4] = twc<16, 4, INV>(o[4]);
    o[5] = twc<16, 5, INV>(o[5]);
    o[6] = twc<16, 6, INV>(o[6]);
    o[7] = twc<16, 7, INV>(o[7]);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = cadd(e[k], o[k]);
        v[k + 8] = csub(e[k], o[k]);
    }
}

template <int R, bool INV, typename T2>
__device__ __forceinline__ void dft(T2* v) {
    if (R == 2) dft2<INV>(v[0], v[1]);
    if (R == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
    if (R == 8) dft8<INV>(v);
    if (R == 16) dft16<INV>(v);
}

// One Stockham stage: for every column and j in [0, L/R), read the R
// elements j + r L/R, apply twiddles w^(r (j mod Ns)) with w = e^(-+2pi i /(Ns R)),
// do an R-point DFT and write them to (j/Ns) Ns R + (j mod Ns) + r Ns.
template <int R, bool INV, typename T2>
__device__ __forceinline__ void stockham_stage(const T2* __restrict__ in, T2* __restrict__ out, int L, int Ns,
                                               int lgc, const T2* __restrict__ tw) {
    const int ncol = 1 << lgc;
    const int m = L / R;
    const int items = m << lgc;
    const int tstep = kMaxL / (Ns * R);
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int j = it >> lgc;
        const int col = it & (ncol - 1);
        const int jm = j & (Ns - 1);
        T2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = in[(j + r * m) * ncol + col];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                const T2 w = __ldg(tw + r * jm * tstep);
                v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
            }
        }
        dft<R, INV>(v);
        const int d = (j - jm) * R + jm;
#pragma unroll
        for (int r = 0; r < R; ++r) out[(d + r * Ns) * ncol + col] = v[r];
    }
}

// Transforms the 2^lgc columns held in `a` (the caller has synchronised after
// filling it); returns the buffer holding the result, synchronised.  The
// inverse is unnormalised.  Radix-16 stages, with one smaller first stage
// (no twiddles) when log2 L is not a multiple of 4.
template <bool INV, typename T2>
__device__ __forceinline__ T2* smem_fft(T2* a, T2* b, int L, int logL, int lgc, const T2* __restrict__ tw) {
    T2* in = a;
    T2* out = b;
    int Ns = 1;
    const int rem = logL & 3;
    if (rem) {
        if (rem == 1) stockham_stage<2, INV>(in, out, L, Ns, lgc, tw);
        if (rem == 2) stockham_stage<4, INV>(in, out, L, Ns, lgc, tw);
        if (rem == 3) stockham_stage<8, INV>(in, out, L, Ns, lgc, tw);
        Ns = 1 << rem;
        T2* t = in;
        in = out;
        out = t;
        __syncthreads();
    }
    while (Ns < L) {
        stockham_stage<16, INV>(in, out, L, Ns, lgc, tw);
        Ns *= 16;
        T2* t = in;
        in = out;
        out = t;
        __syncthreads();
    }
    return in;
}

}  // namespace sc
