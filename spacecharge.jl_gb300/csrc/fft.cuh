// Shared-memory batched FFT building blocks for the hand-written pruned
// convolution.  A CTA holds `ncol` columns of a power-of-two length L in
// shared memory, element (j, col) at [j * ncol + col], and transforms all of
// them with Stockham autosort stages (radix 4, plus one radix-2 stage when
// log2 L is odd) ping-ponging between two buffers.  Twiddles come from a
// per-device table of exp(-2 pi i k / kMaxL) rounded once from FP64, so the
// FP32 transform uses correctly rounded roots of unity.
#pragma once

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

template <typename T2>
__device__ __forceinline__ T2 cadd(T2 a, T2 b) {
    a.x += b.x;
    a.y += b.y;
    return a;
}
template <typename T2>
__device__ __forceinline__ T2 csub(T2 a, T2 b) {
    a.x -= b.x;
    a.y -= b.y;
    return a;
}
template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
    T2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
// a * conj(b)
template <typename T2>
__device__ __forceinline__ T2 cmulc(T2 a, T2 b) {
    T2 r;
    r.x = a.x * b.x + a.y * b.y;
    r.y = a.y * b.x - a.x * b.y;
    return r;
}
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename T2>
__device__ __forceinline__ T2 rot(T2 d) {
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

template <int R, bool INV, typename T2>
__device__ __forceinline__ void dft(T2* v) {
    if (R == 2) {
        const T2 a = v[0];
        v[0] = cadd(a, v[1]);
        v[1] = csub(a, v[1]);
    } else {  // R == 4
        const T2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        const T2 a2 = cadd(v[1], v[3]), a3 = rot<INV>(csub(v[1], v[3]));
        v[0] = cadd(a0, a2);
        v[2] = csub(a0, a2);
        v[1] = cadd(a1, a3);
        v[3] = csub(a1, a3);
    }
}

// One Stockham stage: for every column and j in [0, L/R), read the R
// elements j + r L/R, apply twiddles w^(r (j mod Ns)) with w = e^(-+2pi i /(Ns R)),
// do an R-point DFT and write them to (j/Ns) Ns R + (j mod Ns) + r Ns.
template <int R, bool INV, typename T2>
__device__ __forceinline__ void stockham_stage(const T2* __restrict__ in, T2* __restrict__ out, int L, int Ns,
                                               int ncol, const T2* __restrict__ tw) {
    const int m = L / R;
    const int items = m * ncol;
    const int tstep = kMaxL / (Ns * R);
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int j = it / ncol;
        const int col = it - j * ncol;
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

// Transforms the ncol columns held in `a` (the caller has synchronised after
// filling it); returns the buffer holding the result, synchronised.  The
// inverse is unnormalised.
template <bool INV, typename T2>
__device__ __forceinline__ T2* smem_fft(T2* a, T2* b, int L, int logL, int ncol, const T2* __restrict__ tw) {
    T2* in = a;
    T2* out = b;
    int Ns = 1;
    if (logL & 1) {
        stockham_stage<2, INV>(in, out, L, Ns, ncol, tw);
        Ns = 2;
        T2* t = in;
        in = out;
        out = t;
        __syncthreads();
    }
    while (Ns < L) {
        stockham_stage<4, INV>(in, out, L, Ns, ncol, tw);
        Ns *= 4;
        T2* t = in;
        in = out;
        out = t;
        __syncthreads();
    }
    return in;
}

}  // namespace sc
