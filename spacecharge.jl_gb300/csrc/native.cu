// Hand-written pruned FFT convolution for SC_PREC_MIXED (T = float) and
// SC_PREC_FP64 (T = double): the replacement for solve_freespace!
// (src/solvers/free_space.jl:56-101) and the image-charge solve (:14-47).
//
// The reference convolves on a 2nx x 2ny x 2nz complex grid with 7 c2c FFTs.
// Its output window only reads displacements d in [-(n-1), n-1] of the
// Green function (free_space.jl:98-99), so the same values follow from a
// linear convolution of length L >= 2n-1 per axis (here the next power of
// two) of the real charge with the kernel K[d] placed at index d mod L:
//
//   fwd_x : real rows of rho (nx of Lx nonzero), two rows per complex FFT,
//           split into two half spectra           -> A: Hx x ny x nz
//   fwd_y : ny of Ly nonzero                      -> B: Hx x Ly x nz
//   zpass : z FFT (nz of Lz nonzero), multiply by the three cached Green
//           spectra (+ the image spectra on the flipped kz), three inverse
//           z FFTs, keep z < nz                   -> C: 3 x Hx x Ly x nz
//   inv_y : keep y < ny                           -> D: 3 x Hx x ny x nz
//   inv_x : two rows per complex inverse FFT, keep x < nx, write packed
//           (Ex,Ey,Ez,0) nodes                    -> efield
//
// The Green function (green_functions.jl:35-112) is evaluated in FP64 on the
// corner lattice of one octant (free space) or one quadrant (image), 8-point
// differenced in FP64, placed with its odd/even symmetry, rounded to T,
// transformed with the same passes and stored compressed (it is purely
// imaginary with odd/even symmetry in free space).  FPEI/(Lx Ly Lz) is folded
// into it, so the inverse passes produce E directly.
#include <math.h>

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
template <typename T>
__global__ void __launch_bounds__(256) k_fwd_x(const T* __restrict__ rho, typename Cplx<T>::T2* __restrict__ A,
                                               int nx, int rows, int Lx, int logLx, int Hx, int P,
                                               const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* a = reinterpret_cast<T2*>(smraw);
    T2* b = a + P * Lx;
    const int pair0 = blockIdx.x * P;
    for (int it = threadIdx.x; it < P * Lx; it += blockDim.x) {
        const int p = it / Lx, x = it - p * Lx;
        const int r0 = 2 * (pair0 + p), r1 = r0 + 1;
        T re = 0, im = 0;
        if (x < nx) {
            if (r0 < rows) re = rho[(int64_t)r0 * nx + x];
            if (r1 < rows) im = rho[(int64_t)r1 * nx + x];
        }
        a[x * P + p] = Cplx<T>::make(re, im);
    }
    __syncthreads();
    const T2* res = smem_fft<false>(a, b, Lx, logLx, P, tw);
    for (int it = threadIdx.x; it < P * Hx; it += blockDim.x) {
        const int p = it / Hx, k = it - p * Hx;
        const int r0 = 2 * (pair0 + p), r1 = r0 + 1;
        if (r0 >= rows) continue;
        const T2 Z = res[k * P + p];
        const T2 Y = res[((Lx - k) & (Lx - 1)) * P + p];
        // Xa = (Z + conj Y)/2, Xb = (Z - conj Y)/(2i)
        A[(int64_t)r0 * Hx + k] = Cplx<T>::make(T(0.5) * (Z.x + Y.x), T(0.5) * (Z.y - Y.y));
        if (r1 < rows) A[(int64_t)r1 * Hx + k] = Cplx<T>::make(T(0.5) * (Z.y + Y.y), T(0.5) * (Y.x - Z.x));
    }
}

// Batched column FFT along a strided axis: element (col, j, batch, comp) of
// the input at in[col + j*as_in + batch*bs_in + comp*cs_in]; the first
// n_valid elements are read (the rest are zero), the first n_store written.
template <bool INV, typename T>
__global__ void __launch_bounds__(256) k_col_fft(const typename Cplx<T>::T2* __restrict__ in,
                                                 typename Cplx<T>::T2* __restrict__ out, int ncols, int W, int L,
                                                 int logL, int n_valid, int n_store, int64_t as_in, int64_t bs_in,
                                                 int64_t cs_in, int64_t as_out, int64_t bs_out, int64_t cs_out,
                                                 const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* a = reinterpret_cast<T2*>(smraw);
    T2* b = a + W * L;
    const int c0 = blockIdx.x * W;
    const int64_t ib = blockIdx.y * bs_in + blockIdx.z * cs_in;
    const int64_t ob = blockIdx.y * bs_out + blockIdx.z * cs_out;
    for (int it = threadIdx.x; it < W * L; it += blockDim.x) {
        const int j = it / W, w = it - j * W;
        const int col = c0 + w;
        T2 v = Cplx<T>::make(0, 0);
        if (j < n_valid && col < ncols) v = in[ib + col + j * as_in];
        a[it] = v;
    }
    __syncthreads();
    const T2* res = smem_fft<INV>(a, b, L, logL, W, tw);
    for (int it = threadIdx.x; it < W * n_store; it += blockDim.x) {
        const int j = it / W, w = it - j * W;
        const int col = c0 + w;
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
};

template <typename T>
__global__ void __launch_bounds__(256) k_zpass(const typename Cplx<T>::T2* __restrict__ B,
                                               typename Cplx<T>::T2* __restrict__ C, int Hx, int Ly, int nz, int Lz,
                                               int logLz, int W, GreenView gv,
                                               const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* spec = reinterpret_cast<T2*>(smraw);
    T2* a = spec + W * Lz;
    T2* b = a + W * Lz;
    const int kx0 = blockIdx.x * W;
    const int ky = blockIdx.y;
    const int64_t plane = (int64_t)Hx * Ly;
    for (int it = threadIdx.x; it < W * Lz; it += blockDim.x) {
        const int z = it / W, w = it - z * W;
        const int kx = kx0 + w;
        T2 v = Cplx<T>::make(0, 0);
        if (z < nz && kx < Hx) v = B[kx + (int64_t)Hx * ky + plane * z];
        spec[it] = v;
    }
    __syncthreads();
    const T2* s = smem_fft<false>(spec, a, Lz, logLz, W, tw);
    if (s != spec) {
        // keep the spectrum in `spec`, free a and b for the inverse transforms
        for (int it = threadIdx.x; it < W * Lz; it += blockDim.x) spec[it] = s[it];
        __syncthreads();
    }
    const int kyf = ky <= Ly / 2 ? ky : Ly - ky;
    const T ysign = ky <= Ly / 2 ? T(1) : T(-1);
    const T* gf = reinterpret_cast<const T*>(gv.gfree);
    const T2* gi = reinterpret_cast<const T2*>(gv.gimg);
    for (int comp = 0; comp < 3; ++comp) {
        for (int it = threadIdx.x; it < W * Lz; it += blockDim.x) {
            const int kz = it / W, w = it - kz * W;
            const int kx = kx0 + w;
            T2 r = Cplx<T>::make(0, 0);
            if (kx < Hx) {
                const int kzf = kz <= Lz / 2 ? kz : Lz - kz;
                T sg = T(1);
                if (comp == 1) sg = ysign;
                if (comp == 2 && kz > Lz / 2) sg = T(-1);
                const T g = sg * gf[comp * gv.cs_free + kx + (int64_t)gv.Hx * (kyf + (int64_t)gv.Hy * kzf)];
                const T2 p = spec[it];
                r = Cplx<T>::make(-p.y * g, p.x * g);  // p * (i g)
                if (gv.image) {
                    T2 gc = gi[comp * gv.cs_img + kx + (int64_t)gv.Hx * (kyf + (int64_t)gv.Hy * kz)];
                    if (comp == 1) {
                        gc.x *= ysign;
                        gc.y *= ysign;
                    }
                    const T2 pf = spec[((Lz - kz) & (Lz - 1)) * W + w];  // rho^(kx, ky, -kz)
                    r = cadd(r, cmul(pf, gc));
                }
            }
            a[it] = r;
        }
        __syncthreads();
        const T2* res = smem_fft<true>(a, b, Lz, logLz, W, tw);
        T2* Cc = C + comp * (plane * nz);
        for (int it = threadIdx.x; it < W * nz; it += blockDim.x) {
            const int z = it / W, w = it - z * W;
            const int kx = kx0 + w;
            if (kx < Hx) Cc[kx + (int64_t)Hx * ky + plane * z] = res[it];
        }
        __syncthreads();
    }
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

template <typename T>
__global__ void __launch_bounds__(256) k_inv_x(const typename Cplx<T>::T2* __restrict__ D,
                                               typename Vec4<T>::V* __restrict__ E, int nx, int rows, int Lx,
                                               int logLx, int Hx, int P, int64_t cs,
                                               const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* a = reinterpret_cast<T2*>(smraw);
    T2* b = a + P * Lx;
    T2* keep = b + P * Lx;  // [comp][p][x] for x < nx
    const int pair0 = blockIdx.x * P;
    for (int comp = 0; comp < 3; ++comp) {
        const T2* Dc = D + comp * cs;
        for (int it = threadIdx.x; it < P * Lx; it += blockDim.x) {
            const int p = it / Lx, k = it - p * Lx;
            const int r0 = 2 * (pair0 + p), r1 = r0 + 1;
            T2 xa = Cplx<T>::make(0, 0), xb = Cplx<T>::make(0, 0);
            const int kk = k < Hx ? k : Lx - k;
            const bool cj = k >= Hx;
            if (r0 < rows) xa = Dc[(int64_t)r0 * Hx + kk];
            if (r1 < rows) xb = Dc[(int64_t)r1 * Hx + kk];
            if (cj) {
                xa.y = -xa.y;
                xb.y = -xb.y;
            }
            // Z = Xa + i Xb
            a[k * P + p] = Cplx<T>::make(xa.x - xb.y, xa.y + xb.x);
        }
        __syncthreads();
        const T2* res = smem_fft<true>(a, b, Lx, logLx, P, tw);
        for (int it = threadIdx.x; it < P * nx; it += blockDim.x) {
            const int p = it / nx, x = it - p * nx;
            keep[(comp * P + p) * nx + x] = res[x * P + p];
        }
        __syncthreads();
    }
    for (int it = threadIdx.x; it < 2 * P * nx; it += blockDim.x) {
        const int rp = it / nx, x = it - rp * nx;
        const int p = rp >> 1, half = rp & 1;
        const int row = 2 * (pair0 + p) + half;
        if (row >= rows) continue;
        const T2 ex = keep[(0 * P + p) * nx + x], ey = keep[(1 * P + p) * nx + x], ez = keep[(2 * P + p) * nx + x];
        const typename Vec4<T>::V v =
            half ? Vec4<T>::make(ex.y, ey.y, ez.y) : Vec4<T>::make(ex.x, ey.x, ez.x);
        st4<T>(E + (int64_t)row * nx + x, v);
    }
}

// ----------------------------------------------------- Green construction
// F * factor on the corner lattice e in [0, nx] x [0, ny] x [ez0, nz]; the
// corner e sits where the reference's doubled-grid point i = e + n - 1 does
// (green_functions.jl:82-88 with isize = 2n), evaluated with the same
// expressions so the values match the reference's to rounding of libm.
__global__ void __launch_bounds__(256) k_igf_corners(double* __restrict__ F, int nx, int ny, int nz, int ez0,
                                                     double dx, double dy, double dz_lab, double gamma, int icomp,
                                                     double offz) {
    const int cx = nx + 1, cy = ny + 1, cz = nz + 1 - ez0;
    const int64_t total = (int64_t)cx * cy * cz;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int ex = (int)(t % cx);
    const int ey = (int)((t / cx) % cy);
    const int ez = (int)(t / ((int64_t)cx * cy)) + ez0;
    const int isize = 2 * nx, jsize = 2 * ny, ksize = 2 * nz;
    const double dz = dz_lab * gamma;
    const double factor = (icomp == 1 || icomp == 2) ? gamma / (dx * dy * dz) : 1.0 / (dx * dy * dz);
    const double umin = (double)(1 - isize) * dx / 2;
    const double vmin = (double)(1 - jsize) * dy / 2;
    const double wmin = (double)(1 - ksize) * dz / 2 + offz * gamma;
    const double u = (double)(ex + nx - 1) * dx + umin;
    const double v = (double)(ey + ny - 1) * dy + vmin;
    const double w = (double)(ez + nz - 1) * dz + wmin;
    double val;
    if (icomp == 1)
        val = field_green_n(u, v, w) * factor;
    else if (icomp == 2)
        val = field_green_n(v, w, u) * factor;
    else
        val = field_green_n(w, u, v) * factor;
    F[t] = val;
}

// 8-point difference (green_functions.jl:108-111) for displacements
// d in [0,nx-1] x [0,ny-1] x [dz0, nz-1], scaled by FPEI/(Lx Ly Lz) and
// written with the component's parity to every mirrored index mod L.
template <typename T>
__global__ void __launch_bounds__(256) k_igf_place(const double* __restrict__ F, T* __restrict__ K, int nx, int ny,
                                                   int nz, int ez0, int Lx, int Ly, int Lz, int icomp, int image,
                                                   double scale) {
    const int cx = nx + 1, cy = ny + 1;
    const int dzn = nz - ez0;  // number of dz values: [ez0, nz-1]
    const int64_t total = (int64_t)nx * ny * dzn;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int dx = (int)(t % nx);
    const int dy = (int)((t / nx) % ny);
    const int dzi = (int)(t / ((int64_t)nx * ny));  // corner-lattice z index of the lower corner
    const int64_t sy = cx, sz = (int64_t)cx * cy;
    const double* f = F + dx + sy * dy + sz * dzi;
    auto Fv = [&](int a, int b, int c) { return f[a + sy * b + sz * c]; };
    const double g = Fv(1, 1, 1) - Fv(0, 1, 1) - Fv(1, 0, 1) - Fv(1, 1, 0) - Fv(0, 0, 0) + Fv(0, 0, 1) +
                     Fv(0, 1, 0) + Fv(1, 0, 0);
    const T val = (T)(g * scale);
    const int dz = dzi + ez0;
    const int nsx = dx == 0 ? 1 : 2, nsy = dy == 0 ? 1 : 2;
    const int nsz = (image || dz == 0) ? 1 : 2;
    for (int a = 0; a < nsx; ++a)
        for (int b = 0; b < nsy; ++b)
            for (int c = 0; c < nsz; ++c) {
                const int sxg = a ? -1 : 1, syg = b ? -1 : 1, szg = c ? -1 : 1;
                const int ix = (sxg * dx + Lx) & (Lx - 1);
                const int iy = (syg * dy + Ly) & (Ly - 1);
                const int iz = ((szg * dz) % Lz + Lz) & (Lz - 1);
                const int sgn = icomp == 1 ? sxg : (icomp == 2 ? syg : szg);
                K[ix + (int64_t)Lx * (iy + (int64_t)Ly * iz)] = sgn > 0 ? val : -val;
            }
}

// Compress the half spectrum S (Hx x Ly x Lz) of one component.
template <typename T>
__global__ void __launch_bounds__(256) k_green_compress(const typename Cplx<T>::T2* __restrict__ S,
                                                        void* __restrict__ dst, int Hx, int Ly, int Lz, int Hy,
                                                        int Hz, int image, int nz,
                                                        const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    const int zc = image ? Lz : Hz;
    const int64_t total = (int64_t)Hx * Hy * zc;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int kx = (int)(t % Hx);
    const int ky = (int)((t / Hx) % Hy);
    const int kz = (int)(t / ((int64_t)Hx * Hy));
    const T2 v = S[kx + (int64_t)Hx * (ky + (int64_t)Ly * kz)];
    if (!image) {
        reinterpret_cast<T*>(dst)[t] = v.y;
    } else {
        // -exp(-2 pi i kz (nz-1) / Lz): rho_img[z] = -rho[nz-1-z] gives
        // rho_img^(kz) = -e^{-2 pi i kz (nz-1)/Lz} rho^(-kz)
        const int idx = (int)(((int64_t)kz * (nz - 1)) & (Lz - 1)) * (kMaxL / Lz);
        const T2 w = tw[idx];
        T2 r = cmul(v, w);
        r.x = -r.x;
        r.y = -r.y;
        reinterpret_cast<T2*>(dst)[t] = r;
    }
}

// ------------------------------------------------------------- launching
static int pick_rows(int L) {
    int P = 2048 / L;
    if (P < 1) P = 1;
    return P;
}
static int pick_cols(int L) {
    int W = 2048 / L;
    if (W < 4) W = 4;
    if (W > 32) W = 32;
    return W;
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

template <typename K>
static int set_smem(K kernel, size_t bytes) {
    if (bytes > 48 * 1024) SC_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return SC_OK;
}

// real rows (nx_valid of Lx nonzero) -> half spectra
template <typename T>
static int run_fwd_x(const T* src, typename Cplx<T>::T2* dst, int nx_valid, int rows, const NativeWork& w,
                     const typename Cplx<T>::T2* tw, cudaStream_t s) {
    using T2 = typename Cplx<T>::T2;
    const int P = pick_rows(w.L[0]);
    const size_t smem = sizeof(T2) * 2 * P * w.L[0];
    SC_TRY(set_smem(k_fwd_x<T>, smem));
    const int pairs = (rows + 1) / 2;
    k_fwd_x<T><<<(pairs + P - 1) / P, 256, smem, s>>>(src, dst, nx_valid, rows, w.L[0], w.log2L[0], w.Hx, P, tw);
    SC_LAUNCH_CHECK("k_fwd_x");
    return SC_OK;
}

template <bool INV, typename T>
static int run_col(const typename Cplx<T>::T2* in, typename Cplx<T>::T2* out, int ncols, int L, int logL,
                   int n_valid, int n_store, int64_t as_in, int64_t bs_in, int64_t cs_in, int64_t as_out,
                   int64_t bs_out, int64_t cs_out, int nbatch, int ncomp, const typename Cplx<T>::T2* tw,
                   cudaStream_t s) {
    using T2 = typename Cplx<T>::T2;
    const int W = pick_cols(L);
    const size_t smem = sizeof(T2) * 2 * W * L;
    SC_TRY(set_smem(k_col_fft<INV, T>, smem));
    dim3 grid((ncols + W - 1) / W, nbatch, ncomp);
    k_col_fft<INV, T><<<grid, 256, smem, s>>>(in, out, ncols, W, L, logL, n_valid, n_store, as_in, bs_in, cs_in,
                                               as_out, bs_out, cs_out, tw);
    SC_LAUNCH_CHECK("k_col_fft");
    return SC_OK;
}

template <typename T>
static int alloc_work(sc_mesh* m) {
    using T2 = typename Cplx<T>::T2;
    NativeWork& w = m->nw;
    if (w.A) return SC_OK;
    const int64_t nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int64_t Hx = w.Hx, Ly = w.L[1], Lz = w.L[2];
    const int64_t Hy = Ly / 2 + 1, Hz = Lz / 2 + 1;
    SC_CUDA(cudaMalloc(&w.A, sizeof(T2) * Hx * ny * nz));
    SC_CUDA(cudaMalloc(&w.B, sizeof(T2) * Hx * Ly * nz));
    SC_CUDA(cudaMalloc(&w.C, sizeof(T2) * 3 * Hx * Ly * nz));
    SC_CUDA(cudaMalloc(&w.D, sizeof(T2) * 3 * Hx * ny * nz));
    SC_CUDA(cudaMalloc(&w.gfree, sizeof(T) * 3 * Hx * Hy * Hz));
    return SC_OK;
}

template <typename T>
static int alloc_green_tmp(sc_mesh* m, bool image) {
    using T2 = typename Cplx<T>::T2;
    NativeWork& w = m->nw;
    const int64_t nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int64_t Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    const int64_t Hy = Ly / 2 + 1;
    if (!w.fcorner) SC_CUDA(cudaMalloc(&w.fcorner, sizeof(double) * (nx + 1) * (ny + 1) * (2 * nz)));
    if (!w.kgrid) SC_CUDA(cudaMalloc(&w.kgrid, sizeof(T) * Lx * Ly * Lz));
    if (!w.kspec) SC_CUDA(cudaMalloc(&w.kspec, sizeof(T2) * 2 * Hx * Ly * Lz));
    if (image && !w.gimg) SC_CUDA(cudaMalloc(&w.gimg, sizeof(T2) * 3 * Hx * Hy * Lz));
    return SC_OK;
}

// Build the compressed spectra of the three components for one offset.
template <typename T>
static int build_green(sc_mesh* m, bool image, double offz, cudaStream_t s) {
    using T2 = typename Cplx<T>::T2;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const T2* tw = twiddles<T>(ctx);
    SC_TRY(alloc_green_tmp<T>(m, image));
    NativeWork& w = m->nw;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    const int Hy = Ly / 2 + 1, Hz = Lz / 2 + 1;
    const int ez0 = image ? -(nz - 1) : 0;
    const double scale = kFpei / ((double)Lx * Ly * Lz);
    T* K = (T*)w.kgrid;
    T2* S1 = (T2*)w.kspec;
    T2* S2 = S1 + (int64_t)Hx * Ly * Lz;
    for (int comp = 1; comp <= 3; ++comp) {
        const int64_t ncorner = (int64_t)(nx + 1) * (ny + 1) * (nz + 1 - ez0);
        k_igf_corners<<<(ncorner + 255) / 256, 256, 0, s>>>(w.fcorner, nx, ny, nz, ez0, m->delta[0], m->delta[1],
                                                             m->delta[2], m->gamma, comp, image ? offz : 0.0);
        SC_LAUNCH_CHECK("k_igf_corners");
        SC_CUDA(cudaMemsetAsync(K, 0, sizeof(T) * (int64_t)Lx * Ly * Lz, s));
        const int64_t ncell = (int64_t)nx * ny * (nz - ez0);
        k_igf_place<T><<<(ncell + 255) / 256, 256, 0, s>>>(w.fcorner, K, nx, ny, nz, ez0, Lx, Ly, Lz, comp,
                                                            image ? 1 : 0, scale);
        SC_LAUNCH_CHECK("k_igf_place");
        // full forward R2C of the L grid: x (all Lx valid), y, z
        SC_TRY(run_fwd_x<T>(K, S1, Lx, Ly * Lz, w, tw, s));
        SC_TRY(run_col<false, T>(S1, S2, Hx, Ly, w.log2L[1], Ly, Ly, Hx, (int64_t)Hx * Ly, 0, Hx,
                                 (int64_t)Hx * Ly, 0, Lz, 1, tw, s));
        SC_TRY(run_col<false, T>(S2, S1, Hx, Lz, w.log2L[2], Lz, Lz, (int64_t)Hx * Ly, Hx, 0, (int64_t)Hx * Ly, Hx,
                                 0, Ly, 1, tw, s));
        void* dst;
        int64_t cnt;
        if (image) {
            cnt = (int64_t)Hx * Hy * Lz;
            dst = (T2*)w.gimg + (comp - 1) * cnt;
        } else {
            cnt = (int64_t)Hx * Hy * Hz;
            dst = (T*)w.gfree + (comp - 1) * cnt;
        }
        k_green_compress<T><<<(cnt + 255) / 256, 256, 0, s>>>(S1, dst, Hx, Ly, Lz, Hy, Hz, image ? 1 : 0, nz, tw);
        SC_LAUNCH_CHECK("k_green_compress");
    }
    return SC_OK;
}

static bool key_matches(const GreenKey& k, const sc_mesh* m, double offz) {
    return k.valid && k.delta[0] == m->delta[0] && k.delta[1] == m->delta[1] && k.delta[2] == m->delta[2] &&
           k.gamma == m->gamma && k.offset_z == offz;
}
static void set_key(GreenKey& k, const sc_mesh* m, double offz) {
    for (int d = 0; d < 3; ++d) k.delta[d] = m->delta[d];
    k.gamma = m->gamma;
    k.offset_z = offz;
    k.valid = true;
}

template <typename T>
static int solve_t(sc_mesh* m, int at_cathode, cudaStream_t s) {
    using T2 = typename Cplx<T>::T2;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const T2* tw = twiddles<T>(ctx);
    SC_TRY(alloc_work<T>(m));
    NativeWork& w = m->nw;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    (void)Lx;
    const double offz = 2 * m->lo[2] + (m->hi[2] - m->lo[2]);  // free_space.jl:39
    if (!(m->green_cache && key_matches(w.key_free, m, 0.0))) {
        SC_TRY(build_green<T>(m, false, 0.0, s));
        set_key(w.key_free, m, 0.0);
    }
    if (at_cathode && !(m->green_cache && key_matches(w.key_img, m, offz))) {
        SC_TRY(build_green<T>(m, true, offz, s));
        set_key(w.key_img, m, offz);
    }
    T2* A = (T2*)w.A;
    T2* B = (T2*)w.B;
    T2* C = (T2*)w.C;
    T2* D = (T2*)w.D;
    const int rows = ny * nz;
    SC_TRY(run_fwd_x<T>((const T*)m->rho, A, nx, rows, w, tw, s));
    // y: A (Hx x ny x nz) -> B (Hx x Ly x nz)
    SC_TRY(run_col<false, T>(A, B, Hx, Ly, w.log2L[1], ny, Ly, Hx, (int64_t)Hx * ny, 0, Hx, (int64_t)Hx * Ly, 0, nz,
                             1, tw, s));
    // z + Green + inverse z
    {
        GreenView gv;
        gv.gfree = w.gfree;
        gv.gimg = w.gimg;
        gv.Hx = Hx;
        gv.Hy = Ly / 2 + 1;
        gv.Hz = Lz / 2 + 1;
        gv.Ly = Ly;
        gv.Lz = Lz;
        gv.cs_free = (int64_t)Hx * gv.Hy * gv.Hz;
        gv.cs_img = (int64_t)Hx * gv.Hy * Lz;
        gv.image = at_cathode ? 1 : 0;
        const int W = pick_cols(Lz);
        const size_t smem = sizeof(T2) * 3 * W * Lz;
        SC_TRY(set_smem(k_zpass<T>, smem));
        dim3 grid((Hx + W - 1) / W, Ly);
        k_zpass<T><<<grid, 256, smem, s>>>(B, C, Hx, Ly, nz, Lz, w.log2L[2], W, gv, tw);
        SC_LAUNCH_CHECK("k_zpass");
    }
    // inverse y: C (3 x Hx x Ly x nz) -> D (3 x Hx x ny x nz)
    SC_TRY(run_col<true, T>(C, D, Hx, Ly, w.log2L[1], Ly, ny, Hx, (int64_t)Hx * Ly, (int64_t)Hx * Ly * nz, Hx,
                            (int64_t)Hx * ny, (int64_t)Hx * ny * nz, nz, 3, tw, s));
    // inverse x -> packed efield
    {
        const int P = pick_rows(w.L[0]);
        const size_t smem = sizeof(T2) * (2 * P * w.L[0] + 3 * P * nx);
        SC_TRY(set_smem(k_inv_x<T>, smem));
        const int pairs = (rows + 1) / 2;
        k_inv_x<T><<<(pairs + P - 1) / P, 256, smem, s>>>(D, (typename Vec4<T>::V*)m->efield, nx, rows, w.L[0],
                                                           w.log2L[0], Hx, P, (int64_t)Hx * rows, tw);
        SC_LAUNCH_CHECK("k_inv_x");
    }
    return SC_OK;
}

int native_prepare(sc_mesh* m) {
    NativeWork& w = m->nw;
    for (int d = 0; d < 3; ++d) {
        int L = 1;
        while (L < 2 * m->n[d] - 1) L *= 2;
        if (L < 4) L = 4;
        if (L > kMaxL)
            return fail(SC_ERR_UNSUPPORTED, "grid_size[%d] = %d exceeds the hand-written FFT limit (%d)", d, m->n[d],
                        kMaxL / 2);
        w.L[d] = L;
        w.log2L[d] = ilog2(L);
    }
    w.Hx = w.L[0] / 2 + 1;
    w.elem = m->precision == SC_PREC_MIXED ? sizeof(float2) : sizeof(double2);
    return SC_OK;
}

int native_solve(sc_mesh* m, int at_cathode, cudaStream_t s) {
    if (m->precision == SC_PREC_MIXED) return solve_t<float>(m, at_cathode, s);
    return solve_t<double>(m, at_cathode, s);
}

int native_release(sc_mesh* m) {
    NativeWork& w = m->nw;
    void* ptrs[] = {w.A, w.B, w.C, w.D, w.fcorner, w.kgrid, w.kspec, w.gfree, w.gimg};
    for (void* p : ptrs) cudaFree(p);
    int L[3] = {w.L[0], w.L[1], w.L[2]};
    int lg[3] = {w.log2L[0], w.log2L[1], w.log2L[2]};
    int Hx = w.Hx;
    size_t el = w.elem;
    w = NativeWork();
    for (int d = 0; d < 3; ++d) {
        w.L[d] = L[d];
        w.log2L[d] = lg[d];
    }
    w.Hx = Hx;
    w.elem = el;
    return SC_OK;
}

}  // namespace sc
