// Building blocks shared by the forward pipeline (native.cu) and the adjoint
// (adjoint.cu): the pruned real<->half-spectrum x passes, the strided column
// FFT pass, the packed field node types and the launch helpers.
#pragma once

#include <math.h>

#include <map>
#include <mutex>

#include "fft.cuh"
#include "sc_internal.cuh"

namespace sc {

// green_functions.jl:35-38 (same expression as the plain path)
__device__ __forceinline__ double field_green_n(double x, double y, double z) {
    const double r = sqrt(x * x + y * y + z * z);
    return x * atan((y * z) / (r * x)) - z * log(r + y) + y * log((r - z) / (r + z)) / 2;
}

static int ilog2(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

// ------------------------------------------------------------ pass kernels
// All tile widths (P row pairs, W columns) and transform lengths are powers
// of two, so tile indices are shifts and masks.

// Two-for-one real FFT split: Z = FFT(a + i b) -> A(k), B(k) for k <= L/2.
template <typename T2>
__device__ __forceinline__ void split_pair(T2 Z, T2 Y, T2& xa, T2& xb) {
    // Xa = (Z + conj Y)/2, Xb = (Z - conj Y)/(2i), Y = Z(L - k)
    xa.x = 0.5f * (Z.x + Y.x);
    xa.y = 0.5f * (Z.y - Y.y);
    xb.x = 0.5f * (Z.y + Y.y);
    xb.y = 0.5f * (Y.x - Z.x);
}

template <typename T>
__global__ void __launch_bounds__(256) k_fwd_x(const T* __restrict__ rho, typename Cplx<T>::T2* __restrict__ A,
                                               int nx, int rows, int Lx, int logLx, int Hx, int lgP,
                                               const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int P = 1 << lgP;
    T2* a = reinterpret_cast<T2*>(smraw);
    T2* b = a + (P << logLx);
    const int pair0 = blockIdx.x << lgP;
    for (int it = threadIdx.x; it < (P << logLx); it += blockDim.x) {
        const int p = it >> logLx, x = it & (Lx - 1);
        const int r0 = 2 * (pair0 + p), r1 = r0 + 1;
        T re = 0, im = 0;
        if (x < nx) {
            if (r0 < rows) re = rho[(int64_t)r0 * nx + x];
            if (r1 < rows) im = rho[(int64_t)r1 * nx + x];
        }
        a[(x << lgP) + p] = Cplx<T>::make(re, im);
    }
    __syncthreads();
    const T2* res = smem_fft<false>(a, b, Lx, logLx, lgP, tw);
    const int lgh = logLx - 1, half = Lx >> 1;
    for (int it = threadIdx.x; it < (P << lgh); it += blockDim.x) {
        const int p = it >> lgh, k0 = it & (half - 1);
        const int r0 = 2 * (pair0 + p), r1 = r0 + 1;
        if (r0 >= rows) continue;
        // k0 and, for k0 == 0, also the Nyquist bin Lx/2
        for (int e = 0; e < (k0 == 0 ? 2 : 1); ++e) {
            const int k = e ? half : k0;
            T2 xa, xb;
            split_pair(res[(k << lgP) + p], res[(((Lx - k) & (Lx - 1))) << lgP | p], xa, xb);
            A[(int64_t)r0 * Hx + k] = xa;
            if (r1 < rows) A[(int64_t)r1 * Hx + k] = xb;
        }
    }
}

// Batched column FFT along a strided axis: element (col, j, batch, comp) of
// the input at in[col + j*as_in + batch*bs_in + comp*cs_in]; the first
// n_valid elements are read (the rest are zero), the first n_store written.
template <bool INV, typename T>
__global__ void __launch_bounds__(256) k_col_fft(const typename Cplx<T>::T2* __restrict__ in,
                                                 typename Cplx<T>::T2* __restrict__ out, int ncols, int lgW, int L,
                                                 int logL, int n_valid, int n_store, int64_t as_in, int64_t bs_in,
                                                 int64_t cs_in, int64_t as_out, int64_t bs_out, int64_t cs_out,
                                                 const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int W = 1 << lgW;
    T2* a = reinterpret_cast<T2*>(smraw);
    T2* b = a + (W << logL);
    const int c0 = blockIdx.x << lgW;
    const int64_t ib = blockIdx.y * bs_in + blockIdx.z * cs_in;
    const int64_t ob = blockIdx.y * bs_out + blockIdx.z * cs_out;
    for (int it = threadIdx.x; it < (W << logL); it += blockDim.x) {
        const int j = it >> lgW, col = c0 + (it & (W - 1));
        T2 v = Cplx<T>::make(0, 0);
        if (j < n_valid && col < ncols) v = in[ib + col + j * as_in];
        a[it] = v;
    }
    __syncthreads();
    const T2* res = smem_fft<INV>(a, b, L, logL, lgW, tw);
    for (int it = threadIdx.x; it < (n_store << lgW); it += blockDim.x) {
        const int j = it >> lgW, col = c0 + (it & (W - 1));
        if (col < ncols) out[ob + col + j * as_out] = res[it];
    }
}

// Green-spectrum lookup.  Free space: s[c] = Im(K^_c) at folded (kx, ky, kz),
// purely imaginary, odd in the component's own axis.  Image: complex g[c] at
// folded (kx, ky) and all kz, odd in y for c = 1, with the flip phase of the
// reversed charge folded in.
struct GreenView {
    const void* gfree;
    const void* gimg;
    int Hx, Hy, Hz, Ly, Lz;
    int64_t cs_free, cs_img;
    int image;
    int img_half;  // image spectrum stored for kz <= Lz/2 only (img_at)
};

inline GreenView make_green_view(const NativeWork& w, int image) {
    GreenView gv;
    gv.gfree = w.gfree;
    gv.gimg = w.gimg;
    gv.Hx = w.Hx;
    gv.Hy = w.L[1] / 2 + 1;
    gv.Hz = w.L[2] / 2 + 1;
    gv.Ly = w.L[1];
    gv.Lz = w.L[2];
    gv.cs_free = (int64_t)w.Hx * gv.Hy * gv.Hz;
    gv.img_half = w.img_half ? 1 : 0;
    gv.cs_img = (int64_t)w.Hx * gv.Hy * (w.img_half ? gv.Hz : w.L[2]);
    gv.image = image;
    return gv;
}

// Image spectrum value at kz from a (kx, folded ky) column `gic` with kz
// stride `gstep`.  Each stored column is the z transform of a real line
// times -i^p and the phase of its offset start (p = 1 for components 0 and
// 1), so S(Lz - kz) = eps conj S(kz) with eps = -1 for components 0 and 1,
// +1 for component 2: half storage keeps kz <= Lz/2.
template <typename T2>
__device__ __forceinline__ T2 img_at(const T2* __restrict__ gic, int64_t gstep, int kz, const GreenView& gv,
                                     int comp) {
    if (!gv.img_half || kz <= gv.Lz / 2) return __ldg(gic + gstep * kz);
    T2 v = __ldg(gic + gstep * (gv.Lz - kz));
    if (comp < 2)
        v.x = -v.x;  // -conj
    else
        v.y = -v.y;  // conj
    return v;
}

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
    using V = float4;
    __device__ __forceinline__ static float4 make(float a, float b, float c) { return make_float4(a, b, c, 0.f); }
};
template <>
struct Vec4<double> {
    using V = dnode4;
    __device__ __forceinline__ static dnode4 make(double a, double b, double c) {
        return dnode4{a, b, c, 0.0};
    }
};

template <typename T>
__device__ __forceinline__ void st4(typename Vec4<T>::V* p, typename Vec4<T>::V v) {
    *p = v;
}
template <>
__device__ __forceinline__ void st4<double>(dnode4* p, dnode4 v) {
    double2* q = reinterpret_cast<double2*>(p);
    q[0] = make_double2(v.x, v.y);
    q[1] = make_double2(v.z, v.w);
}

// Inverse x pass of one component into the spare fourth lane of the packed
// field nodes (the adjoint charge density rhobar, the scalar potential).
template <typename T>
__global__ void __launch_bounds__(256) k_inv_x1(const typename Cplx<T>::T2* __restrict__ D, T* __restrict__ E4,
                                                int nx, int rows, int Lx, int logLx, int Hx, int lgP,
                                                const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int P = 1 << lgP;
    const int n = P << logLx;
    T2* a = reinterpret_cast<T2*>(smraw);
    T2* b = a + n;
    const int pair0 = blockIdx.x << lgP;
    for (int it = threadIdx.x; it < n; it += blockDim.x) {
        const int p = it >> logLx, k = it & (Lx - 1);
        const int r0 = 2 * (pair0 + p), r1 = r0 + 1;
        T2 xa = Cplx<T>::make(0, 0), xb = Cplx<T>::make(0, 0);
        const bool cj = k >= Hx;
        const int kk = cj ? Lx - k : k;
        if (r0 < rows) xa = D[(int64_t)r0 * Hx + kk];
        if (r1 < rows) xb = D[(int64_t)r1 * Hx + kk];
        if (cj) {
            xa.y = -xa.y;
            xb.y = -xb.y;
        }
        a[(k << lgP) + p] = Cplx<T>::make(xa.x - xb.y, xa.y + xb.x);
    }
    __syncthreads();
    const T2* res = smem_fft<true>(a, b, Lx, logLx, lgP, tw);
    for (int it = threadIdx.x; it < 2 * n; it += blockDim.x) {
        const int rp = it >> logLx, x = it & (Lx - 1);
        if (x >= nx) continue;
        const int p = rp >> 1, half = rp & 1;
        const int row = 2 * (pair0 + p) + half;
        if (row >= rows) continue;
        const T2 v = res[(x << lgP) + p];
        E4[4 * ((int64_t)row * nx + x) + 3] = half ? v.y : v.x;
    }
}

// ------------------------------------------------------------- launching
// log2 of the row pairs per CTA of the x passes (P * L = 2048 elements)
static int pick_rows(int logL) { return logL >= 11 ? 0 : 11 - logL; }
// log2 of the columns per CTA of the strided passes (W in [4, 32])
static int pick_cols(int logL) {
    int lg = 11 - logL;
    if (lg < 2) lg = 2;
    if (lg > 5) lg = 5;
    return lg;
}

template <typename T>
static const typename Cplx<T>::T2* twiddles(DeviceCtx* c);
template <>
const float2* twiddles<float>(DeviceCtx* c) {
    return c->tw32;
}
template <>
const double2* twiddles<double>(DeviceCtx* c) {
    return c->tw64;
}

// Opt a kernel in to more than 48 KB of dynamic shared memory.  The
// attribute is per device; it is raised once to the largest size requested.
template <typename K>
static int set_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return SC_OK;
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> done;
    int dev = 0;
    SC_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    size_t& cur = done[{dev, (const void*)kernel}];
    if (bytes > cur) {
        SC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        cur = bytes;
    }
    return SC_OK;
}

// real rows (nx_valid of Lx nonzero) -> half spectra
template <typename T>
static int run_fwd_x(const T* src, typename Cplx<T>::T2* dst, int nx_valid, int rows, const NativeWork& w,
                     const typename Cplx<T>::T2* tw, cudaStream_t s) {
    using T2 = typename Cplx<T>::T2;
    const int lgP = pick_rows(w.log2L[0]);
    const size_t smem = sizeof(T2) * 2 * ((size_t)1 << lgP) * w.L[0];
    SC_TRY(set_smem(k_fwd_x<T>, smem));
    const int pairs = (rows + 1) / 2;
    const int P = 1 << lgP;
    k_fwd_x<T><<<(pairs + P - 1) / P, 256, smem, s>>>(src, dst, nx_valid, rows, w.L[0], w.log2L[0], w.Hx, lgP, tw);
    SC_LAUNCH_CHECK("k_fwd_x");
    return SC_OK;
}

template <bool INV, typename T>
static int run_col(const typename Cplx<T>::T2* in, typename Cplx<T>::T2* out, int ncols, int L, int logL,
                   int n_valid, int n_store, int64_t as_in, int64_t bs_in, int64_t cs_in, int64_t as_out,
                   int64_t bs_out, int64_t cs_out, int nbatch, int ncomp, const typename Cplx<T>::T2* tw,
                   cudaStream_t s, int lgW_override = -1) {
    using T2 = typename Cplx<T>::T2;
    const int lgW = lgW_override >= 0 ? lgW_override : pick_cols(logL);
    const int W = 1 << lgW;
    const size_t smem = sizeof(T2) * 2 * W * L;
    SC_TRY(set_smem(k_col_fft<INV, T>, smem));
    dim3 grid((ncols + W - 1) / W, nbatch, ncomp);
    k_col_fft<INV, T><<<grid, 256, smem, s>>>(in, out, ncols, lgW, L, logL, n_valid, n_store, as_in, bs_in, cs_in,
                                               as_out, bs_out, cs_out, tw);
    SC_LAUNCH_CHECK("k_col_fft");
    return SC_OK;
}

template <typename T>
static int alloc_work(sc_mesh* m) {
    using T2 = typename Cplx<T>::T2;
    NativeWork& w = m->nw;
    const int64_t ny = m->n[1], nz = m->n[2];
    const int64_t Hx = w.Hx, Ly = w.L[1], Lz = w.L[2];
    const int64_t Hy = Ly / 2 + 1, Hz = Lz / 2 + 1;
    // each buffer on its own: a call after a failed allocation completes the set
    if (!w.A) SC_CUDA(dev_alloc(&w.A, sizeof(T2) * Hx * ny * nz));
    if (!w.B) SC_CUDA(dev_alloc(&w.B, sizeof(T2) * Hx * Ly * nz));
    if (!w.C) SC_CUDA(dev_alloc(&w.C, sizeof(T2) * 3 * Hx * Ly * nz));
    if (!w.D) SC_CUDA(dev_alloc(&w.D, sizeof(T2) * 3 * Hx * ny * nz));
    if (!w.gfree) SC_CUDA(dev_alloc(&w.gfree, sizeof(T) * 3 * Hx * Hy * Hz));
    return SC_OK;
}

}  // namespace sc
