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

#include <stdio.h>
#include <stdlib.h>

#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "pipeline2.cuh"

namespace sc {

template <typename T>
__global__ void __launch_bounds__(256) k_zpass(const typename Cplx<T>::T2* __restrict__ B,
                                               typename Cplx<T>::T2* __restrict__ C, int Hx, int Ly, int nz, int Lz,
                                               int logLz, int lgW, GreenView gv,
                                               const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int W = 1 << lgW;
    const int n = W << logLz;
    T2* spec = reinterpret_cast<T2*>(smraw);
    T2* a = spec + n;
    T2* b = a + n;
    const int kx0 = blockIdx.x << lgW;
    const int ky = blockIdx.y;
    const int64_t plane = (int64_t)Hx * Ly;
    // forward z FFT: put the input where the result lands in `spec`
    const int stages = ((logLz & 3) ? 1 : 0) + (logLz >> 2);
    T2* first = (stages & 1) ? a : spec;
    T2* second = (stages & 1) ? spec : a;
    for (int it = threadIdx.x; it < n; it += blockDim.x) {
        const int z = it >> lgW, kx = kx0 + (it & (W - 1));
        T2 v = Cplx<T>::make(0, 0);
        if (z < nz && kx < Hx) v = B[kx + (int64_t)Hx * ky + plane * z];
        first[it] = v;
    }
    __syncthreads();
    smem_fft<false>(first, second, Lz, logLz, lgW, tw);  // result in spec
    const int kyf = ky <= Ly / 2 ? ky : Ly - ky;
    const T ysign = ky <= Ly / 2 ? T(1) : T(-1);
    const T* gf = reinterpret_cast<const T*>(gv.gfree);
    const T2* gi = reinterpret_cast<const T2*>(gv.gimg);
    const int halfz = Lz >> 1;
    for (int comp = 0; comp < 3; ++comp) {
        const T* gfc = gf + comp * gv.cs_free + (int64_t)gv.Hx * kyf;
        const T2* gic = gi + comp * gv.cs_img + (int64_t)gv.Hx * kyf;
        for (int it = threadIdx.x; it < n; it += blockDim.x) {
            const int kz = it >> lgW, w = it & (W - 1);
            const int kx = kx0 + w;
            T2 r = Cplx<T>::make(0, 0);
            if (kx < Hx) {
                const int kzf = kz <= halfz ? kz : Lz - kz;
                T sg = T(1);
                if (comp == 1) sg = ysign;
                if (comp == 2 && kz > halfz) sg = T(-1);
                const T g = sg * gfc[kx + (int64_t)gv.Hx * gv.Hy * kzf];
                const T2 p = spec[it];
                r = Cplx<T>::make(-p.y * g, p.x * g);  // p * (i g)
                if (gv.image) {
                    T2 gc = img_at(gic + kx, (int64_t)gv.Hx * gv.Hy, kz, gv, comp);
                    if (comp == 1) {
                        gc.x *= ysign;
                        gc.y *= ysign;
                    }
                    const T2 pf = spec[(((Lz - kz) & (Lz - 1)) << lgW) + w];  // rho^(kx, ky, -kz)
                    r = cadd(r, cmul(pf, gc));
                }
            }
            a[it] = r;
        }
        __syncthreads();
        const T2* res = smem_fft<true>(a, b, Lz, logLz, lgW, tw);
        T2* Cc = C + comp * (plane * nz);
        for (int it = threadIdx.x; it < (nz << lgW); it += blockDim.x) {
            const int z = it >> lgW, kx = kx0 + (it & (W - 1));
            if (kx < Hx) Cc[kx + (int64_t)Hx * ky + plane * z] = res[it];
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_inv_x(const typename Cplx<T>::T2* __restrict__ D,
                                               typename Vec4<T>::V* __restrict__ E, int nx, int rows, int Lx,
                                               int logLx, int Hx, int lgP, int64_t cs,
                                               const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int P = 1 << lgP;
    const int n = P << logLx;
    T2* a = reinterpret_cast<T2*>(smraw);
    T2* b = a + n;
    T2* keep = b + n;  // [comp][p][x], x < Lx
    const int pair0 = blockIdx.x << lgP;
    for (int comp = 0; comp < 3; ++comp) {
        const T2* Dc = D + comp * cs;
        for (int it = threadIdx.x; it < n; it += blockDim.x) {
            const int p = it >> logLx, k = it & (Lx - 1);
            const int r0 = 2 * (pair0 + p), r1 = r0 + 1;
            T2 xa = Cplx<T>::make(0, 0), xb = Cplx<T>::make(0, 0);
            const bool cj = k >= Hx;
            const int kk = cj ? Lx - k : k;
            if (r0 < rows) xa = Dc[(int64_t)r0 * Hx + kk];
            if (r1 < rows) xb = Dc[(int64_t)r1 * Hx + kk];
            if (cj) {
                xa.y = -xa.y;
                xb.y = -xb.y;
            }
            // Z = Xa + i Xb
            a[(k << lgP) + p] = Cplx<T>::make(xa.x - xb.y, xa.y + xb.x);
        }
        __syncthreads();
        const T2* res = smem_fft<true>(a, b, Lx, logLx, lgP, tw);
        for (int it = threadIdx.x; it < n; it += blockDim.x) {
            const int p = it >> logLx, x = it & (Lx - 1);
            if (x < nx) keep[comp * n + it] = res[(x << lgP) + p];
        }
        __syncthreads();
    }
    for (int it = threadIdx.x; it < 2 * n; it += blockDim.x) {
        const int rp = it >> logLx, x = it & (Lx - 1);
        if (x >= nx) continue;
        const int p = rp >> 1, half = rp & 1;
        const int row = 2 * (pair0 + p) + half;
        if (row >= rows) continue;
        const int o = (p << logLx) + x;
        const T2 ex = keep[o], ey = keep[n + o], ez = keep[2 * n + o];
        const typename Vec4<T>::V v = half ? Vec4<T>::make(ex.y, ey.y, ez.y) : Vec4<T>::make(ex.x, ey.x, ez.x);
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

// The same corners for all three components in one launch, one (corner,
// component) per thread (the FP64 antiderivative's FP64 issue time spread
// over many warps): F[c][ez - ez0][ey][ex].
__global__ void __launch_bounds__(128) k_igf_corners3(double* __restrict__ F, int nx, int ny, int nz, int ez0,
                                                      double dx, double dy, double dz_lab, double gamma,
                                                      double offz) {
    const int cx = nx + 1, cy = ny + 1, cz = nz + 1 - ez0;
    const int64_t per = (int64_t)cx * cy * cz;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= 3 * per) return;
    const int icomp = (int)(t / per) + 1;
    const int64_t e = t - (icomp - 1) * per;
    const int ex = (int)(e % cx);
    const int ey = (int)((e / cx) % cy);
    const int ez = (int)(e / ((int64_t)cx * cy)) + ez0;
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

// 8-point difference (green_functions.jl:108-111) of every stored cell of
// the three components, scaled by FPEI/(Lx Ly Lz), into the octant array
// G[c][dz - ez0][dy][dx] that the parity-reduced transform reads.
template <typename OT>  // double, or dreal (double-FP32) for the double-FP32 transform
__global__ void __launch_bounds__(128) k_igf_place_oct(const double* __restrict__ F, OT* __restrict__ G, int nx,
                                                       int ny, int nz, int ez0, double scale) {
    const int cx = nx + 1, cy = ny + 1, cz = nz + 1 - ez0;
    const int64_t per = (int64_t)cx * cy * cz;
    const int64_t cells = (int64_t)nx * ny * (nz - ez0);
    pdl_wait();  // the corners come from the preceding k_igf_corners3
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= 3 * cells) return;
    const int c = (int)(t / cells);
    const int64_t e = t - c * cells;
    const int dx = (int)(e % nx);
    const int dy = (int)((e / nx) % ny);
    const int dzi = (int)(e / ((int64_t)nx * ny));
    const int64_t sy = cx, sz = (int64_t)cx * cy;
    const double* f = F + c * per + dx + sy * dy + sz * dzi;
    auto Fv = [&](int a, int b, int d) { return f[a + sy * b + sz * d]; };
    const double g = Fv(1, 1, 1) - Fv(0, 1, 1) - Fv(1, 0, 1) - Fv(1, 1, 0) - Fv(0, 0, 0) + Fv(0, 0, 1) +
                     Fv(0, 1, 0) + Fv(1, 0, 0);
    G[t] = OT(g * scale);
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

// Green x and y passes as one (k3_green_xy) where it applies
#ifndef SC_FUSED_GREEN_XY
#define SC_FUSED_GREEN_XY 1
#endif
// the field kernel's components paired, four real lines per FFT
// (k4_green_xy, k4_green_col) where they apply
#ifndef SC_PAIRED_GREEN
#define SC_PAIRED_GREEN 1
#endif

// ------------------------------------------- hybrid Green build (FP32 path)
// One thread per displacement d of the stored region (octant in free space;
// quadrant x all dz for the image) computes all three components.  Cells
// within kNearRatio half-widths of the origin use the reference's FP64
// antiderivative corner differences (green_functions.jl:35-38, 82-112, with
// the reference's corner coordinates); elsewhere the cell integral of
// (u, v, w)/r^3 is done by FP32 Gauss-Legendre quadrature (4 points per axis
// below kQ3Ratio, 3 below kQ2Ratio, 2 beyond), which is exact to < 1e-7
// relative there (measured against 16-point rules over cell shapes with
// aspect ratios up to 5) while the FP64 corner differences lose digits to
// cancellation.  The three components
// integrate over the same cell: component y's antiderivative F(v, w, u) and
// z's F(w, u, v) difference to the integrals of v/r^3 and w/r^3.
constexpr double kNearRatio = 6.0;
constexpr double kQ3Ratio = 16.0;
constexpr double kQ2Ratio = 48.0;  // 2 points per axis beyond: < 9e-8 relative (worst cell shape)

struct OctantGeom {
    int nx, ny, nz;
    int image;           // dz range [-(nz-1), nz-1] instead of [0, nz-1]
    double dx, dy, dz;   // full cell widths, dz already scaled by gamma
    double offw;         // cathode offset * gamma on the w axis
    double gamma;
    double hmax;         // half of the largest width
    double scale;        // FPEI / (Lx Ly Lz)
    int64_t cs;          // component stride of the output
    // FP32 copies for the quadrature branch, in units of hmax
    float ux, uy, uz;    // cell widths / hmax
    float uoff;          // offw / hmax
    float kxy, kz;       // gamma_c * scale / (8 hmax^2), per component group
    // box of cells (ix < nbx, iy < nby, bz0 <= dz < bz1) holding every near
    // cell, with the FP64 antiderivative on its corners precomputed in fnear
    int nbx, nby, bz0, bz1;
    const double* fnear;  // [3][(bz1-bz0+1)][nby+1][nbx+1]
};

// FP64 antiderivative F * factor at the corners of the near box, one
// evaluation per thread so that the FP64 pipe's long per-warp issue time is
// spread over many warps and SMs (green_functions.jl:35-38, 69-101 with the
// reference's corner coordinates u = i0*dx + (1 - 2n)*dx/2, i0 = e + n - 1).
__global__ void __launch_bounds__(32) k_igf_near_F(double* __restrict__ F, OctantGeom g) {
    const int cx = g.nbx + 1, cy = g.nby + 1, cz = g.bz1 - g.bz0 + 1;
    const int64_t per = (int64_t)cx * cy * cz;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= 3 * per) return;
    const int c = (int)(t / per);
    const int64_t e = t - c * per;
    const int ex = (int)(e % cx), ey = (int)((e / cx) % cy), ez = (int)(e / ((int64_t)cx * cy)) + g.bz0;
    const double umin = (double)(1 - 2 * g.nx) * g.dx / 2;
    const double vmin = (double)(1 - 2 * g.ny) * g.dy / 2;
    const double wmin = (double)(1 - 2 * g.nz) * g.dz / 2 + g.offw;
    const double u = (double)(ex + g.nx - 1) * g.dx + umin;
    const double v = (double)(ey + g.ny - 1) * g.dy + vmin;
    const double w = (double)(ez + g.nz - 1) * g.dz + wmin;
    const double fxy = g.gamma / (g.dx * g.dy * g.dz), fz = 1.0 / (g.dx * g.dy * g.dz);
    const double val = c == 0 ? field_green_n(u, v, w) : c == 1 ? field_green_n(v, w, u) : field_green_n(w, u, v);
    F[t] = val * (c == 2 ? fz : fxy);
}

__device__ __forceinline__ void gl_accumulate(float cx, float cy, float cz, float hx, float hy, float hz,
                                              const float* t, const float* w, int m, float& ax, float& ay,
                                              float& az) {
    for (int i = 0; i < m; ++i) {
        const float px = fmaf(hx, t[i], cx);
        for (int j = 0; j < m; ++j) {
            const float py = fmaf(hy, t[j], cy);
            const float wij = w[i] * w[j];
            for (int k = 0; k < m; ++k) {
                const float pz = fmaf(hz, t[k], cz);
                const float r2 = fmaf(px, px, fmaf(py, py, pz * pz));
                const float ir = rsqrtf(r2);
                const float q = wij * w[k] * ir * ir * ir;
                ax = fmaf(q, px, ax);
                ay = fmaf(q, py, ay);
                az = fmaf(q, pz, az);
            }
        }
    }
}

// Cell centre in units of hmax and whether the cell takes the FP64 corner
// difference (FP32: the test only decides near/far and the centre feeds the
// quadrature, whose own error is ~1e-7).
struct OctCell {
    float px, py, pz;
    bool near;
};
__device__ __forceinline__ OctCell oct_cell(const OctantGeom& g, int ix, int iy, int dz) {
    OctCell c;
    c.px = (float)ix * g.ux;
    c.py = (float)iy * g.uy;
    c.pz = fmaf((float)dz, g.uz, g.uoff);
    const float ratio = sqrtf(fmaf(c.px, c.px, fmaf(c.py, c.py, c.pz * c.pz)));
    c.near = ratio < (float)kNearRatio && ix < g.nbx && iy < g.nby && dz >= g.bz0 && dz < g.bz1;
    return c;
}

// Far cell: Gauss-Legendre quadrature of (u, v, w)/r^3 over the cell.
__device__ __forceinline__ void oct_far(const OctantGeom& g, const OctCell& c, float out[3]) {
    const float t4[4] = {-0.86113631159405258f, -0.33998104358485626f, 0.33998104358485626f, 0.86113631159405258f};
    const float w4[4] = {0.34785484513745386f, 0.65214515486254614f, 0.65214515486254614f, 0.34785484513745386f};
    const float t3[3] = {-0.77459666924148338f, 0.0f, 0.77459666924148338f};
    const float w3[3] = {0.55555555555555556f, 0.88888888888888889f, 0.55555555555555556f};
    const float hx = 0.5f * g.ux, hy = 0.5f * g.uy, hz = 0.5f * g.uz;
    const float ratio = sqrtf(fmaf(c.px, c.px, fmaf(c.py, c.py, c.pz * c.pz)));
    float ax = 0.f, ay = 0.f, az = 0.f;
    const float t2[2] = {-0.57735026918962576f, 0.57735026918962576f};
    const float w2[2] = {1.0f, 1.0f};
    if (ratio < (float)kQ3Ratio)
        gl_accumulate(c.px, c.py, c.pz, hx, hy, hz, t4, w4, 4, ax, ay, az);
    else if (ratio < (float)kQ2Ratio)
        gl_accumulate(c.px, c.py, c.pz, hx, hy, hz, t3, w3, 3, ax, ay, az);
    else
        gl_accumulate(c.px, c.py, c.pz, hx, hy, hz, t2, w2, 2, ax, ay, az);
    // G_c = gamma_c / 8 * sum w w w p'_c / r'^3 / hmax^2, times FPEI/(L^3)
    out[0] = g.kxy * ax;
    out[1] = g.kxy * ay;
    out[2] = g.kz * az;
}

// The three terms of field_green_n (green_functions.jl:35-38),
// F = T0 - T1 + T2: T0 = x atan(yz/(rx)), T1 = z log(r+y),
// T2 = y log((r-z)/(r+z)) / 2, each on its own thread.
__device__ __forceinline__ double field_green_term(int term, double x, double y, double z) {
    const double r = sqrt(x * x + y * y + z * z);
    if (term == 0) return x * atan((y * z) / (r * x));
    if (term == 1) return z * log(r + y);
    return y * log((r - z) / (r + z)) / 2;
}

// One launch, two block roles.  Blocks [0, near_blocks): the FP64
// antiderivative terms on the near-box corners, T[term][comp][corner],
// one per thread, spread over as many SMs as there are blocks.  The other
// blocks: every far cell of the octant by quadrature (near cells are left to
// k_igf_near_cells, which runs after this).
__global__ void __launch_bounds__(64) k_igf_split(float* __restrict__ G, double* __restrict__ T, OctantGeom g,
                                                  int near_blocks) {
    if ((int)blockIdx.x < near_blocks) {
        const int cx = g.nbx + 1, cy = g.nby + 1, cz = g.bz1 - g.bz0 + 1;
        const int64_t per = (int64_t)cx * cy * cz;
        const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
        if (t >= 9 * per) return;
        const int term = (int)(t / (3 * per));
        const int64_t rest = t - term * 3 * per;
        const int c = (int)(rest / per);
        const int64_t e = rest - c * per;
        const int ex = (int)(e % cx), ey = (int)((e / cx) % cy), ez = (int)(e / ((int64_t)cx * cy)) + g.bz0;
        const double umin = (double)(1 - 2 * g.nx) * g.dx / 2;
        const double vmin = (double)(1 - 2 * g.ny) * g.dy / 2;
        const double wmin = (double)(1 - 2 * g.nz) * g.dz / 2 + g.offw;
        const double u = (double)(ex + g.nx - 1) * g.dx + umin;
        const double v = (double)(ey + g.ny - 1) * g.dy + vmin;
        const double w = (double)(ez + g.nz - 1) * g.dz + wmin;
        // argument permutations of get_green_kernel!, green_functions.jl:76-80
        T[t] = c == 0 ? field_green_term(term, u, v, w)
             : c == 1 ? field_green_term(term, v, w, u)
                      : field_green_term(term, w, u, v);
        return;
    }
    const int zc = g.image ? 2 * g.nz - 1 : g.nz;
    const int64_t total = (int64_t)g.nx * g.ny * zc;
    const int64_t t = (blockIdx.x - near_blocks) * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    int ix, iy, iz;
    if (total <= 0x7FFFFFFF) {  // 32-bit index arithmetic
        const unsigned u = (unsigned)t, r = u / (unsigned)g.nx;
        ix = (int)(u - r * (unsigned)g.nx);
        iy = (int)(r % (unsigned)g.ny);
        iz = (int)(r / (unsigned)g.ny);
    } else {
        ix = (int)(t % g.nx);
        iy = (int)((t / g.nx) % g.ny);
        iz = (int)(t / ((int64_t)g.nx * g.ny));
    }
    const int dz = g.image ? iz - (g.nz - 1) : iz;
    const OctCell cell = oct_cell(g, ix, iy, dz);
    if (cell.near) return;
    float out[3];
    oct_far(g, cell, out);
    for (int c = 0; c < 3; ++c) G[c * g.cs + t] = out[c];
}

// Near cells: the 8-point difference (green_functions.jl:108-111) of the
// corner antiderivatives F = (T0 - T1 + T2) * factor_c, one (cell,
// component) per thread.
__global__ void __launch_bounds__(64) k_igf_near_cells(float* __restrict__ G, const double* __restrict__ T,
                                                       OctantGeom g) {
    pdl_wait();  // the corner terms come from the preceding k_igf_split
    const int bz = g.bz1 - g.bz0;
    const int64_t box = (int64_t)g.nbx * g.nby * bz;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= 3 * box) return;
    const int c = (int)(t / box);
    const int64_t e = t - c * box;
    const int ix = (int)(e % g.nbx), iy = (int)((e / g.nbx) % g.nby), dz = (int)(e / ((int64_t)g.nbx * g.nby)) + g.bz0;
    const OctCell cell = oct_cell(g, ix, iy, dz);
    if (!cell.near) return;
    const int cx = g.nbx + 1, cy = g.nby + 1, cz = bz + 1;
    const int64_t per = (int64_t)cx * cy * cz;
    const int64_t sy = cx, sz = (int64_t)cx * cy;
    const double fc = c == 2 ? 1.0 / (g.dx * g.dy * g.dz) : g.gamma / (g.dx * g.dy * g.dz);  // :82-86
    const int iz = g.image ? dz + g.nz - 1 : dz;
    const int64_t o = ix + (int64_t)g.nx * (iy + (int64_t)g.ny * iz);
    const double* t0 = T + c * per + ix + sy * iy + sz * (dz - g.bz0);
    const double* t1 = t0 + 3 * per;
    const double* t2 = t1 + 3 * per;
    double F[8];  // corner (a, b, e) at a + 2b + 4e
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int64_t q = (k & 1) + sy * ((k >> 1) & 1) + sz * (k >> 2);
        F[k] = (__ldg(t0 + q) - __ldg(t1 + q) + __ldg(t2 + q)) * fc;
    }
    const double G3 = F[7] - F[6] - F[5] - F[3] - F[0] + F[4] + F[2] + F[1];
    G[c * g.cs + o] = (float)(G3 * g.scale);
}

__global__ void __launch_bounds__(256) k_igf_octant(float* __restrict__ G, OctantGeom g) {
    const int zc = g.image ? 2 * g.nz - 1 : g.nz;
    const int64_t total = (int64_t)g.nx * g.ny * zc;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    int ix, iy, iz;
    if (total <= 0x7FFFFFFF) {  // 32-bit index arithmetic
        const unsigned u = (unsigned)t, r = u / (unsigned)g.nx;
        ix = (int)(u - r * (unsigned)g.nx);
        iy = (int)(r % (unsigned)g.ny);
        iz = (int)(r / (unsigned)g.ny);
    } else {
        ix = (int)(t % g.nx);
        iy = (int)((t / g.nx) % g.ny);
        iz = (int)(t / ((int64_t)g.nx * g.ny));
    }
    const int dz = g.image ? iz - (g.nz - 1) : iz;
    const OctCell cell = oct_cell(g, ix, iy, dz);
    float out[3];
    if (cell.near) {
        // 8-point difference of the precomputed corners, green_functions.jl:108-111
        const int cx = g.nbx + 1, cy = g.nby + 1, cz = g.bz1 - g.bz0 + 1;
        const int64_t per = (int64_t)cx * cy * cz;
        const int64_t sy = cx, sz = (int64_t)cx * cy;
        for (int c = 0; c < 3; ++c) {
            const double* f = g.fnear + c * per + ix + sy * iy + sz * (dz - g.bz0);
            auto F = [&](int a, int b, int e) { return f[a + sy * b + sz * e]; };
            const double G3 = F(1, 1, 1) - F(0, 1, 1) - F(1, 0, 1) - F(1, 1, 0) - F(0, 0, 0) + F(0, 0, 1) +
                              F(0, 1, 0) + F(1, 0, 0);
            out[c] = (float)(G3 * g.scale);
        }
    } else {
        oct_far(g, cell, out);
    }
    for (int c = 0; c < 3; ++c) G[c * g.cs + t] = out[c];
}

// Rows of the L grid that hold kernel values: displacement index c in
// [0, 2n-1) maps to L-grid row c (c < n) or L - (2n-1) + c (negative d).
__device__ __forceinline__ int wrap_row(int c, int n, int L) { return c < n ? c : L - (2 * n - 1) + c; }

// x pass of the kernel transform, three components (blockIdx.y): each valid
// row (y, z) of the L grid is expanded from the stored octant/quadrant with
// the component's parity, two rows per complex FFT.
__global__ void __launch_bounds__(256) k_green_x(const float* __restrict__ G, float2* __restrict__ S, int nx,
                                                 int ny, int nz, int image, int Lx, int logLx, int Ly, int Lz,
                                                 int Hx, int lgP, int64_t gcs, int64_t scs,
                                                 const float2* __restrict__ tw) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int P = 1 << lgP;
    const int n = P << logLx;
    float2* a = reinterpret_cast<float2*>(smraw);
    float2* b = a + n;
    int* meta = reinterpret_cast<int*>(b + n);  // per row: source offset, sign flags, output row
    const int comp = blockIdx.y;
    const float* Gc = G + comp * gcs;
    const int rows = (2 * ny - 1) * (2 * nz - 1);
    const int pair0 = blockIdx.x << lgP;
    for (int h = threadIdx.x; h < 2 * P; h += blockDim.x) {
        const int r = 2 * pair0 + h;
        int src = -1, neg = 0, orow = 0;
        if (r < rows) {
            const int cy = r % (2 * ny - 1), cz = r / (2 * ny - 1);
            const int dy = cy < ny ? cy : cy - (2 * ny - 1);
            const int dz = cz < nz ? cz : cz - (2 * nz - 1);
            const int ay = dy < 0 ? -dy : dy;
            const int iz = image ? dz + nz - 1 : (dz < 0 ? -dz : dz);
            src = nx * (ay + ny * iz);
            // parity: comp 0 odd in x (per element), comp 1 odd in y, comp 2 odd in z (free space)
            neg = (comp == 1 && dy < 0) || (comp == 2 && !image && dz < 0);
            orow = wrap_row(cy, ny, Ly) + Ly * wrap_row(cz, nz, Lz);
        }
        meta[3 * h] = src;
        meta[3 * h + 1] = neg;
        meta[3 * h + 2] = orow;
    }
    __syncthreads();
    for (int it = threadIdx.x; it < n; it += blockDim.x) {
        const int p = it >> logLx, x = it & (Lx - 1);
        float v[2] = {0.f, 0.f};
        const int dx = x < nx ? x : (x > Lx - nx ? x - Lx : Lx);
        if (dx != Lx) {
            const int ax = dx < 0 ? -dx : dx;
            const bool xneg = comp == 0 && dx < 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int src = meta[3 * (2 * p + h)];
                if (src < 0) continue;
                const float val = Gc[src + ax];
                v[h] = (xneg != (meta[3 * (2 * p + h) + 1] != 0)) ? -val : val;
            }
        }
        a[(x << lgP) + p] = make_float2(v[0], v[1]);
    }
    __syncthreads();
    const float2* res = smem_fft<false>(a, b, Lx, logLx, lgP, tw);
    float2* Sc = S + comp * scs;
    const int lgh = logLx - 1, half = Lx >> 1;
    for (int it = threadIdx.x; it < (P << lgh); it += blockDim.x) {
        const int p = it >> lgh, k0 = it & (half - 1);
        if (meta[3 * (2 * p)] < 0) continue;
        const int o0 = meta[3 * (2 * p) + 2], o1 = meta[3 * (2 * p + 1) + 2];
        const bool has1 = meta[3 * (2 * p + 1)] >= 0;
        for (int e = 0; e < (k0 == 0 ? 2 : 1); ++e) {
            const int k = e ? half : k0;
            float2 xa, xb;
            split_pair(res[(k << lgP) + p], res[(((Lx - k) & (Lx - 1)) << lgP) + p], xa, xb);
            Sc[(int64_t)o0 * Hx + k] = xa;
            if (has1) Sc[(int64_t)o1 * Hx + k] = xb;
        }
    }
}

// y pass in place: columns (kx) at every valid z (blockIdx.y over the
// compact z index), inputs only on the valid rows, all Ly outputs.
__global__ void __launch_bounds__(256) k_green_y(float2* __restrict__ S, int ny, int nz, int Ly, int logLy,
                                                 int Lz, int Hx, int lgW, int64_t scs,
                                                 const float2* __restrict__ tw) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int W = 1 << lgW;
    const int n = W << logLy;
    float2* a = reinterpret_cast<float2*>(smraw);
    float2* b = a + n;
    const int z = wrap_row(blockIdx.y, nz, Lz);
    float2* Sc = S + blockIdx.z * scs + (int64_t)Hx * Ly * z;
    const int c0 = blockIdx.x << lgW;
    for (int it = threadIdx.x; it < n; it += blockDim.x) {
        const int y = it >> lgW, col = c0 + (it & (W - 1));
        float2 v = make_float2(0.f, 0.f);
        if (col < Hx && (y < ny || y > Ly - ny)) v = Sc[col + (int64_t)Hx * y];
        a[it] = v;
    }
    __syncthreads();
    const float2* res = smem_fft<false>(a, b, Ly, logLy, lgW, tw);
    for (int it = threadIdx.x; it < n; it += blockDim.x) {
        const int y = it >> lgW, col = c0 + (it & (W - 1));
        if (col < Hx) Sc[col + (int64_t)Hx * y] = res[it];
    }
}

// z pass for ky in [0, Ly/2] with the compression fused: free space keeps
// Im(K^) for kz in [0, Lz/2]; the image keeps all kz with the flip phase
// -exp(-2 pi i kz (nz-1)/Lz) folded in.
__global__ void __launch_bounds__(256) k_green_z(const float2* __restrict__ S, void* __restrict__ dst, int nz,
                                                 int image, int Ly, int Lz, int logLz, int Hx, int lgW, int64_t scs,
                                                 int64_t dcs, const float2* __restrict__ tw) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int W = 1 << lgW;
    const int n = W << logLz;
    float2* a = reinterpret_cast<float2*>(smraw);
    float2* b = a + n;
    const int ky = blockIdx.y;
    const int comp = blockIdx.z;
    const int Hy = Ly / 2 + 1;
    const float2* Sc = S + comp * scs;
    const int c0 = blockIdx.x << lgW;
    const int64_t plane = (int64_t)Hx * Ly;
    for (int it = threadIdx.x; it < n; it += blockDim.x) {
        const int z = it >> lgW, col = c0 + (it & (W - 1));
        float2 v = make_float2(0.f, 0.f);
        if (col < Hx && (z < nz || z > Lz - nz)) v = Sc[col + (int64_t)Hx * ky + plane * z];
        a[it] = v;
    }
    __syncthreads();
    const float2* res = smem_fft<false>(a, b, Lz, logLz, lgW, tw);
    const int zc = image ? Lz : Lz / 2 + 1;
    for (int it = threadIdx.x; it < (zc << lgW); it += blockDim.x) {
        const int kz = it >> lgW, col = c0 + (it & (W - 1));
        if (col >= Hx) continue;
        const float2 v = res[it];
        const int64_t o = col + (int64_t)Hx * (ky + (int64_t)Hy * kz);
        if (!image) {
            reinterpret_cast<float*>(dst)[comp * dcs + o] = v.y;
        } else {
            const float2 ph = tw[(int)(((int64_t)kz * (nz - 1)) & (Lz - 1)) * (kMaxL / Lz)];
            const float2 r = cmul(v, ph);
            reinterpret_cast<float2*>(dst)[comp * dcs + o] = make_float2(-r.x, -r.y);
        }
    }
}

template <typename T>
static int alloc_green_tmp(sc_mesh* m, bool image) {
    using T2 = typename Cplx<T>::T2;
    NativeWork& w = m->nw;
    const int64_t nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int64_t Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    const int64_t Hy = Ly / 2 + 1;
    if (!w.fcorner) SC_CUDA(dev_alloc(&w.fcorner, sizeof(double) * (nx + 1) * (ny + 1) * (2 * nz)));
    if (!w.kgrid) SC_CUDA(dev_alloc(&w.kgrid, sizeof(T) * Lx * Ly * Lz));
    if (!w.kspec) SC_CUDA(dev_alloc(&w.kspec, sizeof(T2) * 2 * Hx * Ly * Lz));
    if (image && !w.gimg) SC_CUDA(dev_alloc(&w.gimg, sizeof(T2) * 3 * Hx * Hy * Lz));
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
            w.img_half = false;
        } else {
            cnt = (int64_t)Hx * Hy * Hz;
            dst = (T*)w.gfree + (comp - 1) * cnt;
        }
        k_green_compress<T><<<(cnt + 255) / 256, 256, 0, s>>>(S1, dst, Hx, Ly, Lz, Hy, Hz, image ? 1 : 0, nz, tw);
        SC_LAUNCH_CHECK("k_green_compress");
    }
    return SC_OK;
}

// FP32 path: hybrid octant kernel + three batched transform passes.
static int build_green_mixed(sc_mesh* m, bool image, double offz, cudaStream_t s) {
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const float2* tw = ctx->tw32;
    NativeWork& w = m->nw;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    const int Hy = Ly / 2 + 1, Hz = Lz / 2 + 1;
    const int64_t gcs = (int64_t)nx * ny * (2 * nz - 1);
    const int64_t scs = (int64_t)Hx * Ly * Lz;
    // the free-space and image builds have their own scratch: they may run
    // concurrently on two streams (native_green_async)
    void*& goct = image ? w.goct_img : w.goct;
    void*& gtmp = image ? w.gtmp_img : w.gtmp;
    double*& fnear = image ? w.fnear_img : w.fnear;
    int64_t& fnear_cap = image ? w.fnear_img_cap : w.fnear_cap;
    if (!goct) SC_CUDA(dev_alloc(&goct, sizeof(float) * 3 * gcs));
    if (image && !w.gimg) SC_CUDA(dev_alloc(&w.gimg, sizeof(float2) * 3 * (int64_t)Hx * Hy * Lz));
    OctantGeom g;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.image = image ? 1 : 0;
    g.dx = m->delta[0];
    g.dy = m->delta[1];
    g.dz = m->delta[2] * m->gamma;  // green_functions.jl:73
    g.offw = image ? offz * m->gamma : 0.0;
    g.gamma = m->gamma;
    g.hmax = 0.5 * fmax(g.dx, fmax(g.dy, g.dz));
    g.scale = kFpei / ((double)Lx * Ly * Lz);
    g.cs = gcs;
    g.ux = (float)(g.dx / g.hmax);
    g.uy = (float)(g.dy / g.hmax);
    g.uz = (float)(g.dz / g.hmax);
    g.uoff = (float)(g.offw / g.hmax);
    g.kxy = (float)(g.gamma * g.scale / (8.0 * g.hmax * g.hmax));
    g.kz = (float)(g.scale / (8.0 * g.hmax * g.hmax));
    // near box: every cell with |centre| < kNearRatio * hmax, plus a margin
    {
        const double reach = kNearRatio * g.hmax;
        g.nbx = (int)fmin((double)nx, floor(reach / g.dx) + 2.0);
        g.nby = (int)fmin((double)ny, floor(reach / g.dy) + 2.0);
        const int dzmin = image ? -(nz - 1) : 0;
        g.bz0 = (int)fmax((double)dzmin, floor((-reach - g.offw) / g.dz) - 1.0);
        g.bz1 = (int)fmin((double)nz, ceil((reach - g.offw) / g.dz) + 2.0);
        if (g.bz1 <= g.bz0) g.nbx = g.nby = 0, g.bz0 = g.bz1 = 0;
    }
    // FP64 antiderivative terms on the near-box corners (3 terms x 3 comps)
    const bool has_near = g.nbx > 0 && g.nby > 0 && g.bz1 > g.bz0;
    const int64_t nterm = has_near ? 9 * (int64_t)(g.nbx + 1) * (g.nby + 1) * (g.bz1 - g.bz0 + 1) : 0;
    if (fnear_cap < nterm) {
        fnear_cap = 0;
        SC_CUDA(dev_realloc(&fnear, sizeof(double) * nterm));
        fnear_cap = nterm;
    }
    g.fnear = fnear;
    const int zc = image ? 2 * nz - 1 : nz;
    const int64_t cells = (int64_t)nx * ny * zc;
    const int near_blocks = (int)((nterm + 63) / 64);
    k_igf_split<<<(unsigned)(near_blocks + (cells + 63) / 64), 64, 0, s>>>((float*)goct, fnear, g, near_blocks);
    SC_LAUNCH_CHECK("k_igf_split");
    // the near cells' differences: inside the paired x+y pass where that
    // runs, else their own launch before the transform
    GreenNear gn{};
    if (has_near) {
        gn.T = fnear;
        gn.nx = nx;
        gn.ny = ny;
        gn.nz = nz;
        gn.image = g.image;
        gn.nbx = g.nbx;
        gn.nby = g.nby;
        gn.bz0 = g.bz0;
        gn.bz1 = g.bz1;
        gn.ux = g.ux;
        gn.uy = g.uy;
        gn.uz = g.uz;
        gn.uoff = g.uoff;
        gn.ratio = (float)kNearRatio;
        gn.fz = 1.0 / (g.dx * g.dy * g.dz);
        gn.fxy = g.gamma / (g.dx * g.dy * g.dz);
        gn.scale = g.scale;
    }
    const bool two_step = fft_engine() == 0 && w.log2L[0] <= 8 && w.log2L[1] <= 8 && w.log2L[2] <= 8;
    if (two_step && SC_PAIRED_GREEN && has_near) {
        const int64_t t1max = (int64_t)Hx * ny * (2 * nz - 1), t2max = (int64_t)Hx * Hy * (2 * nz - 1);
        if (!gtmp) SC_CUDA(dev_alloc(&gtmp, sizeof(float) * 3 * (t1max + t2max)));
        float* T2p = (float*)gtmp + 3 * t1max;
        const int64_t t2cs = (int64_t)Hx * Hy * zc;
        const int64_t plane = (int64_t)Hx * Hy;
        if (launch_green_xy_field(w.log2L[0], w.log2L[1], (float*)goct, T2p, nx, ny, zc, Hx, gcs, t2cs, tw, s, gn)) {
            SC_LAUNCH_CHECK("k4_green_xy");
            const bool zok = image ? launch3_green_col(true, w.log2L[2], T2p, w.gimg, (int)plane, 1, nz, 2, plane, 0,
                                                       t2cs, plane, 0, plane * Hz, tw, s)
                                   : launch_green_z_field(w.log2L[2], (const float*)T2p, (float*)w.gfree, (int)plane,
                                                          nz, plane, t2cs, plane, plane * Hz, m->gamma, tw, s);
            if (!zok) return fail(SC_ERR_UNSUPPORTED, "Green z pass: transform length out of range");
            SC_LAUNCH_CHECK("green z pass");
            if (image) w.img_half = true;
            m->launches += 3;
            return SC_OK;
        }
    }
    if (has_near) {
        const int64_t box = (int64_t)g.nbx * g.nby * (g.bz1 - g.bz0);
        launch_pdl(k_igf_near_cells, (unsigned)((3 * box + 63) / 64), 64, 0, s, (float*)goct, (const double*)fnear, g);
        SC_LAUNCH_CHECK("k_igf_near_cells");
    }
    if (two_step) {
        // parity-reduced transform: real octant lines only (pipeline2.cuh)
        const int64_t t1max = (int64_t)Hx * ny * (2 * nz - 1), t2max = (int64_t)Hx * Hy * (2 * nz - 1);
        if (!gtmp) SC_CUDA(dev_alloc(&gtmp, sizeof(float) * 3 * (t1max + t2max)));
        float* T1 = (float*)gtmp;
        float* T2 = T1 + 3 * t1max;
        const int64_t t1cs = (int64_t)Hx * ny * zc, t2cs = (int64_t)Hx * Hy * zc;
        const int64_t plane = (int64_t)Hx * Hy;
        // x and y fused per z slice where the slice fits in shared memory:
        // components 0 and 1 paired (four real lines per FFT), 2 alone
        bool xy = false;
        int nl = 0;
        if (SC_PAIRED_GREEN &&
            launch_green_xy_field(w.log2L[0], w.log2L[1], (float*)goct, T2, nx, ny, zc, Hx, gcs, t2cs, tw, s)) {
            xy = true;
            nl = 1;
        } else if (SC_FUSED_GREEN_XY &&
                   launch3_green_xy(w.log2L[0], w.log2L[1], (const float*)goct, T2, nx, ny, zc, Hx, gcs, t2cs, tw, s)) {
            xy = true;
            nl = 1;
        }
        if (xy) {
            SC_LAUNCH_CHECK("green x+y pass");
            bool zok;
            if (!image && SC_PAIRED_GREEN) {
                zok = launch_green_z_field(w.log2L[2], (const float*)T2, (float*)w.gfree, (int)plane, nz, plane, t2cs,
                                           plane, plane * Hz, m->gamma, tw, s);
                nl += 1;
            } else {
                zok = launch3_green_col(image, w.log2L[2], T2, image ? w.gimg : w.gfree, (int)plane, 1, nz, 2, plane, 0,
                                        t2cs, plane, 0, plane * Hz, tw, s);
                nl += 1;
            }
            if (!zok) return fail(SC_ERR_UNSUPPORTED, "Green z pass: transform length out of range");
            SC_LAUNCH_CHECK("green z pass");
            if (image) w.img_half = true;
            m->launches += nl + (has_near ? 2 : 1);
            return SC_OK;
        }
        if (launch3_green_x(w.log2L[0], (const float*)goct, T1, nx, ny * zc, Hx, gcs, t1cs, tw, s) &&
            launch3_green_col(false, w.log2L[1], T1, T2, Hx, zc, ny, 1, Hx, (int64_t)Hx * ny, t1cs, Hx, plane, t2cs,
                              tw, s) &&
            launch3_green_col(image, w.log2L[2], T2, image ? w.gimg : w.gfree, (int)plane, 1, nz, 2, plane, 0, t2cs,
                              plane, 0, plane * Hz, tw, s)) {
            SC_LAUNCH_CHECK("green two-step");
            if (image) w.img_half = true;
            m->launches += has_near ? 5 : 4;
            return SC_OK;
        }
    }
    if (!w.gspec) SC_CUDA(dev_alloc(&w.gspec, sizeof(float2) * 3 * scs));
    float2* S = (float2*)w.gspec;
    {
        const int lgP = pick_rows(w.log2L[0]);
        const int P = 1 << lgP;
        const size_t smem = sizeof(float2) * 2 * P * Lx + sizeof(int) * 6 * P;
        SC_TRY(set_smem(k_green_x, smem));
        const int rows = (2 * ny - 1) * (2 * nz - 1);
        dim3 grid(((rows + 1) / 2 + P - 1) / P, 3);
        k_green_x<<<grid, 256, smem, s>>>((const float*)goct, S, nx, ny, nz, g.image, Lx, w.log2L[0], Ly, Lz, Hx,
                                          lgP, gcs, scs, tw);
        SC_LAUNCH_CHECK("k_green_x");
    }
    {
        const int lgW = pick_cols(w.log2L[1]);
        const int W = 1 << lgW;
        const size_t smem = sizeof(float2) * 2 * W * Ly;
        SC_TRY(set_smem(k_green_y, smem));
        dim3 grid((Hx + W - 1) / W, 2 * nz - 1, 3);
        k_green_y<<<grid, 256, smem, s>>>(S, ny, nz, Ly, w.log2L[1], Lz, Hx, lgW, scs, tw);
        SC_LAUNCH_CHECK("k_green_y");
    }
    {
        const int lgW = pick_cols(w.log2L[2]);
        const int W = 1 << lgW;
        const size_t smem = sizeof(float2) * 2 * W * Lz;
        SC_TRY(set_smem(k_green_z, smem));
        dim3 grid((Hx + W - 1) / W, Hy, 3);
        void* dst = image ? w.gimg : w.gfree;
        const int64_t dcs = image ? (int64_t)Hx * Hy * Lz : (int64_t)Hx * Hy * Hz;
        if (image) w.img_half = false;
        k_green_z<<<grid, 256, smem, s>>>(S, dst, nz, g.image, Ly, Lz, w.log2L[2], Hx, lgW, scs, dcs, tw);
        SC_LAUNCH_CHECK("k_green_z");
    }
    m->launches += has_near ? 5 : 4;
    return SC_OK;
}

template <typename T>
static int build_green_any(sc_mesh* m, bool image, double offz, cudaStream_t s, bool dd, int* fmt);
template <>
int build_green_any<float>(sc_mesh* m, bool image, double offz, cudaStream_t s, bool, int* fmt) {
    *fmt = 0;
    return build_green_mixed(m, image, offz, s);
}
// FP64 pipeline: the reference's FP64 corner differences on the stored
// octant (free space) or quadrant (image) of all three components, then the
// parity-reduced transform of pipeline2.cuh in FP64 (real octant lines, two
// per complex FFT, about 8x less transform work than the full L grid).
// Returns false (nothing issued) where that transform does not apply
// (transform lengths above 256).
// dd (free space only): the x+y and z transforms in double-FP32 (k4_*<L,
// dreal>), the spectrum stored as dreal; *fmt reports the format written.
static int build_green_fp64_reduced(sc_mesh* m, bool image, double offz, cudaStream_t s, bool* done, bool dd,
                                    int* fmt) {
    *done = false;
    *fmt = 0;
    NativeWork& w = m->nw;
    // (the process-wide Stockham-only setting keeps the full-grid build too)
    if (fft_engine() != 0 || w.log2L[0] > 8 || w.log2L[1] > 8 || w.log2L[2] > 8) return SC_OK;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const double2* tw = ctx->tw64;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    const int Hy = Ly / 2 + 1, Hz = Lz / 2 + 1;
    const int ez0 = image ? -(nz - 1) : 0;
    const int zc = nz - ez0;
    const int64_t ncorner = (int64_t)(nx + 1) * (ny + 1) * (zc + 1);
    const int64_t gcs = (int64_t)nx * ny * zc;
    const int64_t t1max = (int64_t)Hx * ny * (2 * nz - 1), t2max = (int64_t)Hx * Hy * (2 * nz - 1);
    // scratch (shared by the free-space and image builds, which run one
    // after the other on one stream in FP64): corners | octant | x, y outputs
    const int64_t need = 3 * ((int64_t)(nx + 1) * (ny + 1) * 2 * nz) + 3 * (int64_t)nx * ny * (2 * nz - 1) +
                         3 * (t1max + t2max);
    if (w.fnear_cap < need) {
        w.fnear_cap = 0;
        SC_CUDA(dev_realloc(&w.fnear, sizeof(double) * need));
        w.fnear_cap = need;
    }
    if (image && !w.gimg) SC_CUDA(dev_alloc(&w.gimg, sizeof(double2) * 3 * (int64_t)Hx * Hy * Lz));
    double* F = w.fnear;
    double* G = F + 3 * ((int64_t)(nx + 1) * (ny + 1) * 2 * nz);
    double* T1 = G + 3 * (int64_t)nx * ny * (2 * nz - 1);
    double* T2 = T1 + 3 * t1max;
    k_igf_corners3<<<(unsigned)((3 * ncorner + 127) / 128), 128, 0, s>>>(F, nx, ny, nz, ez0, m->delta[0], m->delta[1],
                                                                        m->delta[2], m->gamma, image ? offz : 0.0);
    SC_LAUNCH_CHECK("k_igf_corners3");
    const int64_t t1cs = (int64_t)Hx * ny * zc, t2cs = (int64_t)Hx * Hy * zc;
    const int64_t plane = (int64_t)Hx * Hy;
    void* dst = image ? w.gimg : w.gfree;
    if (dd && !image && SC_PAIRED_GREEN && dd_green_applies(w.log2L[0], w.log2L[1], w.log2L[2], nx, ny, nz)) {
        // double-FP32: the octant split as it is placed, then the paired
        // transforms on the FP32 units (dreal buffers: 8 bytes, as double)
        dreal* Gd = reinterpret_cast<dreal*>(G);
        launch_pdl(k_igf_place_oct<dreal>, (unsigned)((3 * gcs + 127) / 128), 128, 0, s, (const double*)F, Gd, nx, ny,
                   nz, ez0, kFpei / ((double)Lx * Ly * Lz));
        SC_LAUNCH_CHECK("k_igf_place_oct");
        if (!launch_dd_green(w.log2L[0], w.log2L[2], Gd, reinterpret_cast<dreal*>(T2), (dreal*)dst, nx, ny, nz, Hx,
                             gcs, t2cs, m->gamma, (const ddc*)ctx->twdd, s))
            return fail(SC_ERR_CUDA, "double-FP32 Green transform did not launch");
        SC_LAUNCH_CHECK("double-FP32 Green transform");
        m->launches += 3;
        *fmt = 1;
        *done = true;
        return SC_OK;
    }
    launch_pdl(k_igf_place_oct<double>, (unsigned)((3 * gcs + 127) / 128), 128, 0, s, (const double*)F, G, nx, ny, nz,
               ez0, kFpei / ((double)Lx * Ly * Lz));
    SC_LAUNCH_CHECK("k_igf_place_oct");
    bool ok = SC_PAIRED_GREEN &&
              launch_green_xy_field<double>(w.log2L[0], w.log2L[1], G, T2, nx, ny, zc, Hx, gcs, t2cs, tw, s);
    if (ok) {
        SC_LAUNCH_CHECK("k4_green_xy");
        m->launches += 3;
    } else if ((ok = launch3_green_xy<double>(w.log2L[0], w.log2L[1], G, T2, nx, ny, zc, Hx, gcs, t2cs, tw, s))) {
        SC_LAUNCH_CHECK("k3_green_xy");
        m->launches += 3;
    } else {
        ok = launch3_green_x<double>(w.log2L[0], G, T1, nx, ny * zc, Hx, gcs, t1cs, tw, s) &&
             launch3_green_col<double>(false, w.log2L[1], T1, T2, Hx, zc, ny, 1, Hx, (int64_t)Hx * ny, t1cs, Hx,
                                       plane, t2cs, tw, s);
        if (!ok) return fail(SC_ERR_UNSUPPORTED, "FP64 Green x/y pass: transform length out of range");
        SC_LAUNCH_CHECK("green x/y passes");
        m->launches += 4;
    }
    const bool zok = (!image && SC_PAIRED_GREEN)
                         ? launch_green_z_field<double>(w.log2L[2], T2, (double*)dst, (int)plane, nz, plane, t2cs, plane,
                                                        plane * Hz, m->gamma, tw, s)
                         : launch3_green_col<double>(image, w.log2L[2], T2, dst, (int)plane, 1, nz, 2, plane, 0, t2cs,
                                                     plane, 0, plane * Hz, tw, s);
    if (!zok) return fail(SC_ERR_UNSUPPORTED, "FP64 Green z pass: transform length out of range");
    SC_LAUNCH_CHECK("green z pass");
    if (image) w.img_half = true;
    *done = true;
    return SC_OK;
}

template <>
int build_green_any<double>(sc_mesh* m, bool image, double offz, cudaStream_t s, bool dd, int* fmt) {
    bool done = false;
    SC_TRY(build_green_fp64_reduced(m, image, offz, s, &done, dd, fmt));
    if (done) return SC_OK;
    SC_TRY(build_green<double>(m, image, offz, s));
    m->launches += 18;
    return SC_OK;
}

// fmt < 0: either format
static bool key_matches(const GreenKey& k, const sc_mesh* m, double offz, int fmt = -1) {
    return k.valid && k.delta[0] == m->delta[0] && k.delta[1] == m->delta[1] && k.delta[2] == m->delta[2] &&
           k.gamma == m->gamma && k.offset_z == offz && (fmt < 0 || k.fmt == fmt);
}
static void set_key(GreenKey& k, const sc_mesh* m, double offz, int fmt) {
    for (int d = 0; d < 3; ++d) k.delta[d] = m->delta[d];
    k.gamma = m->gamma;
    k.offset_z = offz;
    k.fmt = fmt;
    k.valid = true;
}

// Whether the free-space spectrum is wanted in double-FP32: FP64 meshes in
// double-FP32 mode, solves in free space (the FP64 image z pass reads the
// FP64 one), every length within the register kernels, the caller's z pass
// able to take it (dd_ok).
static bool green_dd_wanted(const sc_mesh* m, int at_cathode, bool dd_ok) {
    if (!dd_ok || at_cathode || m->precision != SC_PREC_FP64 || !m->df32) return false;
    const NativeWork& w = m->nw;
    const int eng = w.engine >= 0 ? w.engine : fft_engine();
    return eng == 0 && w.log2L[0] > 0 && w.log2L[0] <= 8 && w.log2L[1] <= 8 && w.log2L[2] <= 8;
}

// Build (or reuse) the compressed Green spectra the solve needs.
// Builds the free-space (image = false) or image spectrum unless the cached
// one matches the geometry.
// dd: build the free-space spectrum in double-FP32 (green_dd_wanted); the
// double-FP32 z pass takes a cached FP64 one as well, the FP64 z passes
// only that
template <typename T>
static int ensure_green_part(sc_mesh* m, bool image, cudaStream_t s, bool dd = false) {
    NativeWork& w = m->nw;
    const double offz = image ? 2 * m->lo[2] + (m->hi[2] - m->lo[2]) : 0.0;  // free_space.jl:39
    GreenKey& key = image ? w.key_img : w.key_free;
    if (m->green_cache && key_matches(key, m, offz, dd && !image ? -1 : 0)) return SC_OK;
    StageScope st(m->timer, SC_STAGE_GREEN, s);
    int fmt = 0;
    SC_TRY(build_green_any<T>(m, image, offz, s, dd && !image, &fmt));
    set_key(key, m, offz, fmt);
    m->green_epoch++;
    return SC_OK;
}

template <typename T>
static int ensure_green_t(sc_mesh* m, int at_cathode, cudaStream_t s, bool dd_ok = true) {
    SC_TRY(ensure_green_part<T>(m, false, s, green_dd_wanted(m, at_cathode, dd_ok)));
    if (at_cathode) SC_TRY(ensure_green_part<T>(m, true, s));
    return SC_OK;
}

bool native_green_stale(const sc_mesh* m, int at_cathode, bool dd_ok) {
    const NativeWork& w = m->nw;
    const double offz = 2 * m->lo[2] + (m->hi[2] - m->lo[2]);  // free_space.jl:39
    const int need = green_dd_wanted(m, at_cathode, dd_ok) ? -1 : 0;
    if (!(m->green_cache && key_matches(w.key_free, m, 0.0, need))) return true;
    return at_cathode && !(m->green_cache && key_matches(w.key_img, m, offz));
}

int native_ensure_green(sc_mesh* m, int at_cathode, cudaStream_t s, bool dd_ok) {
    if (m->precision == SC_PREC_MIXED) {
        SC_TRY(alloc_work<float>(m));
        return ensure_green_t<float>(m, at_cathode, s);
    }
    SC_TRY(alloc_work<double>(m));
    return ensure_green_t<double>(m, at_cathode, s, dd_ok);
}

// inverse y and x as one pass (k2_inv_yx) where it applies
#ifndef SC_FUSED_FWD_XY
#define SC_FUSED_FWD_XY 1
#endif
#ifndef SC_FUSED_INV_YX
#define SC_FUSED_INV_YX 1
#endif

template <typename T>
static int solve_t(sc_mesh* m, int at_cathode, cudaStream_t s, cudaEvent_t green_ready) {
    using T2 = typename Cplx<T>::T2;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const T2* tw = twiddles<T>(ctx);
    SC_TRY(alloc_work<T>(m));
    NativeWork& w = m->nw;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    (void)Lx;
    // green_ready: the spectra are being built on another stream (native_green_async)
#ifndef SC_FUSED_FWD_WITH_GREEN
#define SC_FUSED_FWD_WITH_GREEN 0  // the fused forward x+y pass beside a concurrent Green build
#endif
    if (!green_ready) SC_TRY(ensure_green_t<T>(m, at_cathode, s));
    m->launches += 5;
    T2* A = (T2*)w.A;
    T2* B = (T2*)w.B;
    T2* C = (T2*)w.C;
    T2* D = (T2*)w.D;
    const int rows = ny * nz;
    // FP32 with transforms of at most 256 points: register two-step kernels
    // (unless this mesh's autotuned or the process-wide choice says Stockham)
    const int eng = w.engine >= 0 ? w.engine : fft_engine();
    const bool two = std::is_same<T, float>::value && eng == 0;
    // FP64 meshes in double-FP32 mode where all three lengths fit the
    // register kernels: the x and y passes in double-FP32 (A, D and, in free
    // space, B hold double-FP32 values), and the z pass too in free space
    const bool dd = std::is_same<T, double>::value && m->df32 && eng == 0 && w.log2L[0] <= 8 &&
                    w.log2L[1] <= 8 && w.log2L[2] <= 8;
    const ddc* twdd = (const ddc*)ctx->twdd;
    const int lgWy = w.lgW >= 0 ? w.lgW : pick_cols(w.log2L[1]);
    // The fused forward pass runs one CTA per z plane, each a long chain of
    // FFT rounds: it pays only with the GPU to itself.  Beside a concurrent
    // Green build the kick went from 0.138 to 0.145 ms, and inside a batch
    // from 6.10 to 6.43 ms; alone, the Green-cached kick went from 0.110 to
    // 0.108 ms and the tracking step from 0.134 to 0.131 ms.
    bool fwd_fused = false;
    if (two && SC_FUSED_FWD_XY && (!green_ready || m->green_ahead || SC_FUSED_FWD_WITH_GREEN) &&
        !m->beside_others) {
        StageScope st(m->timer, SC_STAGE_FWD_X, s);
        fwd_fused = launch2_fwd_xy(w.log2L[0], w.log2L[1], (const float*)m->rho, (float2*)B, nx, ny, nz, Hx,
                                   (const float2*)tw, s, m->fused_smem_cap);
        if (fwd_fused) {
            SC_LAUNCH_CHECK("k2_fwd_xy");
            m->launches -= 1;  // one launch for the two passes
        }
    }
    if (!fwd_fused) {
        StageScope st(m->timer, SC_STAGE_FWD_X, s);
        if (dd) {
            if (!launch2_dd_fwd_x(w.log2L[0], (const double*)m->rho, (ddc*)A, nx, rows, Hx, twdd, s))
                return fail(SC_ERR_CUDA, "double-FP32 forward x pass did not launch");
        } else if (!(two && launch2_fwd_x(w.log2L[0], (const float*)m->rho, (float2*)A, nx, rows, Hx, (const float2*)tw,
                                          s)))
            SC_TRY(run_fwd_x<T>((const T*)m->rho, A, nx, rows, w, tw, s));
        SC_LAUNCH_CHECK("fwd_x");
    }
    if (!fwd_fused) {
        // y: A (Hx x ny x nz) -> B (Hx x Ly x nz)
        StageScope st(m->timer, SC_STAGE_FWD_Y, s);
        if (dd) {
            // with the image the z pass stays FP64: B widened to FP64
            const bool ok = at_cathode ? launch2_dd_col<false>(w.log2L[1], (const ddc*)A, (double2*)B, Hx, nz, 1, ny, Ly,
                                                               Hx, (int64_t)Hx * ny, 0, Hx, (int64_t)Hx * Ly, 0, twdd, s)
                                       : launch2_dd_col<false>(w.log2L[1], (const ddc*)A, (ddc*)B, Hx, nz, 1, ny, Ly, Hx,
                                                               (int64_t)Hx * ny, 0, Hx, (int64_t)Hx * Ly, 0, twdd, s);
            if (!ok) return fail(SC_ERR_CUDA, "double-FP32 forward y pass did not launch");
        } else if (!(two && launch2_col(false, w.log2L[1], (const float2*)A, (float2*)B, Hx, ny, Ly, Hx, (int64_t)Hx * ny,
                                 0, Hx, (int64_t)Hx * Ly, 0, nz, 1, (const float2*)tw, s)))
            SC_TRY(run_col<false, T>(A, B, Hx, Ly, w.log2L[1], ny, Ly, Hx, (int64_t)Hx * ny, 0, Hx, (int64_t)Hx * Ly,
                                     0, nz, 1, tw, s, lgWy));
        SC_LAUNCH_CHECK("fwd_y");
    }
    bool c_dd = false;  // the z pass left C in double-FP32
    // z + Green + inverse z
    {
        if (green_ready) SC_CUDA(cudaStreamWaitEvent(s, green_ready, 0));
        StageScope st(m->timer, SC_STAGE_ZPASS, s);
        const GreenView gv = make_green_view(w, at_cathode ? 1 : 0);
        if (two && launch2_zpass(w.log2L[2], (const float2*)B, (float2*)C, Hx, Ly, nz, gv, (const float2*)tw, s)) {
            SC_LAUNCH_CHECK("k2_zpass");
            goto zdone;
        }
        // FP64 in free space, on request: the z pass in double-FP32, its
        // output kept in double-FP32 for the inverse passes
        if (dd && launch2_dd_zpass(w.log2L[2], (const ddc*)B, (ddc*)C, Hx, Ly, nz, gv, w.key_free.fmt, twdd, s)) {
            c_dd = true;
            SC_LAUNCH_CHECK("k2_dd_zpass");
            goto zdone;
        }
        {
        int lgW = w.lgW >= 0 ? w.lgW : pick_cols(w.log2L[2]);
        while (lgW > 0 && sizeof(T2) * 3 * ((size_t)1 << lgW) * Lz > 200 * 1024) --lgW;  // shared-memory cap
        const int W = 1 << lgW;
        const size_t smem = sizeof(T2) * 3 * W * Lz;
        SC_TRY(set_smem(k_zpass<T>, smem));
        dim3 grid((Hx + W - 1) / W, Ly);
        k_zpass<T><<<grid, 256, smem, s>>>(B, C, Hx, Ly, nz, Lz, w.log2L[2], lgW, gv, tw);
        SC_LAUNCH_CHECK("k_zpass");
        }
    zdone:;
    }
    {
        // inverse y: C (3 x Hx x Ly x nz) -> D (3 x Hx x ny x nz)
        StageScope st(m->timer, SC_STAGE_INV_Y, s);
        if (two && SC_FUSED_INV_YX &&
            launch2_inv_yx(w.log2L[0], w.log2L[1], (const float2*)C, (float4*)m->efield, nx, ny, nz, Hx,
                           (const float2*)tw, s, m->fused_smem_cap)) {
            SC_LAUNCH_CHECK("k2_inv_yx");
            m->launches -= 1;  // one launch for the two passes
            return SC_OK;
        }
        if (dd) {
            const bool ok = c_dd ? launch2_dd_col<true>(w.log2L[1], (const ddc*)C, (ddc*)D, Hx, nz, 3, Ly, ny, Hx,
                                                        (int64_t)Hx * Ly, (int64_t)Hx * Ly * nz, Hx, (int64_t)Hx * ny,
                                                        (int64_t)Hx * ny * nz, twdd, s)
                                 : launch2_dd_col<true>(w.log2L[1], (const double2*)C, (ddc*)D, Hx, nz, 3, Ly, ny, Hx,
                                                        (int64_t)Hx * Ly, (int64_t)Hx * Ly * nz, Hx, (int64_t)Hx * ny,
                                                        (int64_t)Hx * ny * nz, twdd, s);
            if (!ok) return fail(SC_ERR_CUDA, "double-FP32 inverse y pass did not launch");
            SC_LAUNCH_CHECK("k2_dd_col");
        } else if (!(two && launch2_col(true, w.log2L[1], (const float2*)C, (float2*)D, Hx, Ly, ny, Hx, (int64_t)Hx * Ly,
                                 (int64_t)Hx * Ly * nz, Hx, (int64_t)Hx * ny, (int64_t)Hx * ny * nz, nz, 3,
                                 (const float2*)tw, s)))
            SC_TRY(run_col<true, T>(C, D, Hx, Ly, w.log2L[1], Ly, ny, Hx, (int64_t)Hx * Ly, (int64_t)Hx * Ly * nz, Hx,
                                    (int64_t)Hx * ny, (int64_t)Hx * ny * nz, nz, 3, tw, s, lgWy));
        SC_LAUNCH_CHECK("inv_y");
    }
    {
        // inverse x -> packed efield
        StageScope st(m->timer, SC_STAGE_INV_X, s);
        if (two && launch2_inv_x(w.log2L[0], (const float2*)D, (float4*)m->efield, nx, rows, Hx, (int64_t)Hx * rows,
                                 (const float2*)tw, s)) {
            SC_LAUNCH_CHECK("k2_inv_x");
            return SC_OK;
        }
        if (dd) {
            if (!launch2_dd_inv_x(w.log2L[0], (const ddc*)D, (dnode4*)m->efield, nx, rows, Hx, (int64_t)Hx * rows, twdd,
                                  s))
                return fail(SC_ERR_CUDA, "double-FP32 inverse x pass did not launch");
            SC_LAUNCH_CHECK("k2_dd_inv_x");
            return SC_OK;
        }
        const int lgP = pick_rows(w.log2L[0]);
        const int P = 1 << lgP;
        const size_t smem = sizeof(T2) * 5 * P * w.L[0];
        SC_TRY(set_smem(k_inv_x<T>, smem));
        const int pairs = (rows + 1) / 2;
        k_inv_x<T><<<(pairs + P - 1) / P, 256, smem, s>>>(D, (typename Vec4<T>::V*)m->efield, nx, rows, w.L[0],
                                                           w.log2L[0], Hx, lgP, (int64_t)Hx * rows, tw);
        SC_LAUNCH_CHECK("k_inv_x");
    }
    return SC_OK;
}

// ----------------------------------------------------------- autotuner
// Choices per (GPU name, precision, Lx, Ly, Lz): engine 0 = register
// two-step, 1 = Stockham with 2^lgW columns per CTA.
struct TuneKey {
    std::string gpu;
    int prec, L0, L1, L2;
    bool operator<(const TuneKey& o) const {
        if (gpu != o.gpu) return gpu < o.gpu;
        if (prec != o.prec) return prec < o.prec;
        if (L0 != o.L0) return L0 < o.L0;
        if (L1 != o.L1) return L1 < o.L1;
        return L2 < o.L2;
    }
};
static std::mutex g_tune_mu;
static std::map<TuneKey, std::pair<int, int>> g_tune;
static bool g_tune_loaded = false;

static std::string gpu_name(int dev) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "unknown";
    std::string n(p.name);
    for (char& c : n)
        if (c == ' ') c = '_';
    return n;
}

static void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = getenv("SC_AUTOTUNE_FILE");
    if (!path) return;
    FILE* f = fopen(path, "r");
    if (!f) return;
    char name[256];
    int prec, l0, l1, l2, eng, lg;
    while (fscanf(f, "%255s %d %d %d %d %d %d", name, &prec, &l0, &l1, &l2, &eng, &lg) == 7)
        g_tune[TuneKey{name, prec, l0, l1, l2}] = {eng, lg};
    fclose(f);
}

bool tuned_choice(int device, int precision, const int L[3], int* engine, int* lgW) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load_locked();
    auto it = g_tune.find(TuneKey{gpu_name(device), precision, L[0], L[1], L[2]});
    if (it == g_tune.end()) return false;
    *engine = it->second.first;
    *lgW = it->second.second;
    return true;
}

static int autotune(sc_mesh* m, cudaStream_t s, int* choice) {
    if (m->precision == SC_PREC_PLAIN64)
        return fail(SC_ERR_UNSUPPORTED, "the autotuner tunes the hand-written pipelines (precision fp64 or mixed)");
    NativeWork& w = m->nw;
    const bool keep_cache = m->green_cache;
    m->green_cache = true;
    std::vector<std::pair<int, int>> cand;
    if (m->precision == SC_PREC_MIXED && w.L[0] <= 256 && w.L[1] <= 256 && w.L[2] <= 256) cand.push_back({0, -1});
    for (int lg = 2; lg <= 5; ++lg) cand.push_back({1, lg});
    cudaEvent_t a, b;
    SC_CUDA(cudaEventCreate(&a));
    SC_CUDA(cudaEventCreate(&b));
    float best = 1e30f;
    std::pair<int, int> pick = cand[0];
    int st = SC_OK;
    for (auto c : cand) {
        w.engine = c.first;
        w.lgW = c.second;
        for (int r = 0; r < 2 && st == SC_OK; ++r) st = native_solve(m, 0, s);
        if (st != SC_OK) break;
        cudaEventRecord(a, s);
        for (int r = 0; r < 5 && st == SC_OK; ++r) st = native_solve(m, 0, s);
        cudaEventRecord(b, s);
        if (st != SC_OK) break;
        if (cudaEventSynchronize(b) != cudaSuccess) {
            st = cuda_fail(cudaGetLastError(), "autotune timing");
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) {
            best = ms;
            pick = c;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    m->green_cache = keep_cache;
    w.engine = pick.first;
    w.lgW = pick.second;
    if (st != SC_OK) return st;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        tune_load_locked();
        TuneKey k{gpu_name(m->device), m->precision, w.L[0], w.L[1], w.L[2]};
        g_tune[k] = pick;
        if (const char* path = getenv("SC_AUTOTUNE_FILE")) {
            if (FILE* f = fopen(path, "a")) {
                fprintf(f, "%s %d %d %d %d %d %d\n", k.gpu.c_str(), k.prec, k.L0, k.L1, k.L2, pick.first,
                        pick.second);
                fclose(f);
            }
        }
    }
    if (choice) *choice = pick.first == 0 ? 0 : pick.second;
    return SC_OK;
}

int native_autotune(sc_mesh* m, cudaStream_t s, int* choice) { return autotune(m, s, choice); }

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
    int eng = -1, lg = -1;
    if (tuned_choice(m->device, m->precision, w.L, &eng, &lg)) {
        w.engine = eng;
        w.lgW = lg;
    }
    return SC_OK;
}

int native_solve(sc_mesh* m, int at_cathode, cudaStream_t s, cudaEvent_t green_ready) {
    if (m->precision == SC_PREC_MIXED) return solve_t<float>(m, at_cathode, s, green_ready);
    return solve_t<double>(m, at_cathode, s, green_ready);
}

int native_green_async(sc_mesh* m, int at_cathode, cudaStream_t s, cudaEvent_t* ready, bool dd_ok) {
    *ready = nullptr;
    if (!native_green_stale(m, at_cathode, dd_ok)) return SC_OK;
    // highest priority: the z pass waits for these builds, the deposit on
    // the caller's stream does not
    int least = 0, greatest = 0;
    SC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
#ifndef SC_GREEN_LOW_PRIORITY
#define SC_GREEN_LOW_PRIORITY 0
#endif
    const int prio = SC_GREEN_LOW_PRIORITY ? least : greatest;
    if (!m->side) SC_CUDA(cudaStreamCreateWithPriority(&m->side, cudaStreamNonBlocking, prio));
    if (!m->side2) SC_CUDA(cudaStreamCreateWithPriority(&m->side2, cudaStreamNonBlocking, prio));
    if (!m->ev_fork) SC_CUDA(cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming));
    if (!m->ev_join) SC_CUDA(cudaEventCreateWithFlags(&m->ev_join, cudaEventDisableTiming));
    if (!m->ev_join2) SC_CUDA(cudaEventCreateWithFlags(&m->ev_join2, cudaEventDisableTiming));
    SC_CUDA(cudaEventRecord(m->ev_fork, s));
    SC_CUDA(cudaStreamWaitEvent(m->side, m->ev_fork, 0));
    // the FP32 builds of the two spectra have separate scratch: run them side by side
    int st = SC_OK;
    if (at_cathode && m->precision == SC_PREC_MIXED) {
        SC_TRY(alloc_work<float>(m));
        SC_CUDA(cudaStreamWaitEvent(m->side2, m->ev_fork, 0));
        st = ensure_green_part<float>(m, false, m->side);
        if (st == SC_OK) st = ensure_green_part<float>(m, true, m->side2);
        const cudaError_t e2 = cudaEventRecord(m->ev_join2, m->side2);
        if (st == SC_OK && e2 != cudaSuccess) st = cuda_fail(e2, "cudaEventRecord");
        cudaStreamWaitEvent(m->side, m->ev_join2, 0);
    } else {
        st = native_ensure_green(m, at_cathode, m->side, dd_ok);
    }
    const cudaError_t e = cudaEventRecord(m->ev_join, m->side);
    if (st != SC_OK || e != cudaSuccess) {
        cudaStreamWaitEvent(s, m->ev_join, 0);
        return st != SC_OK ? st : cuda_fail(e, "cudaEventRecord");
    }
    *ready = m->ev_join;
    return SC_OK;
}

// dd: the FP64 mesh's forward passes in double-FP32 (B then holds
// double-FP32 values); the caller checks native_dd_applies
template <typename T>
static int forward_t(sc_mesh* m, cudaStream_t s, bool dd) {
    using T2 = typename Cplx<T>::T2;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const T2* tw = twiddles<T>(ctx);
    SC_TRY(alloc_work<T>(m));
    NativeWork& w = m->nw;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int Ly = w.L[1], Hx = w.Hx;
    const int rows = ny * nz;
    const int eng = w.engine >= 0 ? w.engine : fft_engine();
    const bool two = std::is_same<T, float>::value && eng == 0;
    const int lgWy = w.lgW >= 0 ? w.lgW : pick_cols(w.log2L[1]);
    if (std::is_same<T, double>::value && dd) {
        const ddc* twdd = (const ddc*)ctx->twdd;
        if (!launch2_dd_fwd_x(w.log2L[0], (const double*)m->rho, (ddc*)w.A, nx, rows, Hx, twdd, s) ||
            !launch2_dd_col<false>(w.log2L[1], (const ddc*)w.A, (ddc*)w.B, Hx, nz, 1, ny, Ly, Hx, (int64_t)Hx * ny, 0,
                                   Hx, (int64_t)Hx * Ly, 0, twdd, s))
            return fail(SC_ERR_CUDA, "double-FP32 forward passes did not launch");
        SC_LAUNCH_CHECK("double-FP32 forward x, y");
        m->launches += 2;
        return SC_OK;
    }
    if (two && SC_FUSED_FWD_XY &&
        launch2_fwd_xy(w.log2L[0], w.log2L[1], (const float*)m->rho, (float2*)w.B, nx, ny, nz, Hx, (const float2*)tw,
                       s, m->fused_smem_cap)) {
        SC_LAUNCH_CHECK("k2_fwd_xy");
        m->launches += 1;
        return SC_OK;
    }
    T2* A = (T2*)w.A;
    if (!(two && launch2_fwd_x(w.log2L[0], (const float*)m->rho, (float2*)A, nx, rows, Hx, (const float2*)tw, s)))
        SC_TRY(run_fwd_x<T>((const T*)m->rho, A, nx, rows, w, tw, s));
    SC_LAUNCH_CHECK("fwd_x");
    if (!(two && launch2_col(false, w.log2L[1], (const float2*)A, (float2*)w.B, Hx, ny, Ly, Hx, (int64_t)Hx * ny, 0,
                             Hx, (int64_t)Hx * Ly, 0, nz, 1, (const float2*)tw, s)))
        SC_TRY(run_col<false, T>(A, (T2*)w.B, Hx, Ly, w.log2L[1], ny, Ly, Hx, (int64_t)Hx * ny, 0, Hx,
                                 (int64_t)Hx * Ly, 0, nz, 1, tw, s, lgWy));
    SC_LAUNCH_CHECK("fwd_y");
    m->launches += 2;
    return SC_OK;
}

bool native_dd_applies(const sc_mesh* m) {
    if (m->precision != SC_PREC_FP64 || !m->df32) return false;
    const NativeWork& w = m->nw;
    const int eng = w.engine >= 0 ? w.engine : fft_engine();
    return eng == 0 && w.log2L[0] > 0 && w.log2L[0] <= 8 && w.log2L[1] <= 8 && w.log2L[2] <= 8;
}

int native_forward(sc_mesh* m, cudaStream_t s, bool dd) {
    if (m->precision == SC_PREC_MIXED) return forward_t<float>(m, s, false);
    return forward_t<double>(m, s, dd);
}

int native_release(sc_mesh* m) {
    NativeWork& w = m->nw;
    void* ptrs[] = {w.A,      w.B,     w.C,    w.D,        w.adjE,  w.adjcorner, w.fnear,    w.fnear_img, w.fcorner,
                    w.kgrid,  w.kspec, w.goct, w.goct_img, w.gspec, w.gtmp,      w.gtmp_img, w.gfree,     w.gimg,
                    w.pfree,  w.pimg,  w.pscratch};
    for (void* p : ptrs) cudaFree(p);
    int L[3] = {w.L[0], w.L[1], w.L[2]};
    int lg[3] = {w.log2L[0], w.log2L[1], w.log2L[2]};
    int Hx = w.Hx;
    size_t el = w.elem;
    const int eng = w.engine, lgw = w.lgW;
    w = NativeWork();
    w.engine = eng;
    w.lgW = lgw;
    for (int d = 0; d < 3; ++d) {
        w.L[d] = L[d];
        w.log2L[d] = lg[d];
    }
    w.Hx = Hx;
    w.elem = el;
    return SC_OK;
}

// ------------------------------------------------ allocation-free solve
// sc_solve_noalloc: the mixed-precision free-space solve of a caller's rho
// into a caller's packed efield with every intermediate (FFT workspace,
// Green-function build, twiddle table) in one file-scope device array.  It
// serves callers that cannot let a library call cudaMalloc: host codes that
// own all device memory through their own pool, and loops that forbid device
// allocation once they are running.  Grids up to kNaMaxN nodes per axis.
// The array is shared by every call on a device and keeps the last call's
// contents; every buffer a call reads is written earlier in the same call,
// so nothing needs clearing, but calls that overlap on the GPU race.
constexpr int kNaMaxN = 32;                     // nodes per axis
constexpr int kNaMaxL = 64;                     // transform length per axis
constexpr int kNaMaxHx = kNaMaxL / 2 + 1;
constexpr size_t na_up(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kNaA = na_up(sizeof(float2) * kNaMaxHx * kNaMaxN * kNaMaxN);
constexpr size_t kNaB = na_up(sizeof(float2) * kNaMaxHx * kNaMaxL * kNaMaxN);
constexpr size_t kNaC = 3 * kNaB;
constexpr size_t kNaD = 3 * kNaA;
constexpr size_t kNaGoct = na_up(sizeof(float) * 3 * kNaMaxN * kNaMaxN * (2 * kNaMaxN - 1));
constexpr size_t kNaGspec = na_up(sizeof(float2) * 3 * kNaMaxHx * kNaMaxL * kNaMaxL);
constexpr size_t kNaGfree = na_up(sizeof(float) * 3 * kNaMaxHx * (kNaMaxL / 2 + 1) * (kNaMaxL / 2 + 1));
constexpr size_t kNaFnear = na_up(sizeof(double) * 3 * (kNaMaxN + 1) * (kNaMaxN + 1) * (kNaMaxN + 1));
constexpr size_t kNaTw = na_up(sizeof(float2) * kMaxL);
constexpr size_t kNaBytes = kNaA + kNaB + kNaC + kNaD + kNaGoct + kNaGspec + kNaGfree + kNaFnear + kNaTw;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

// Device address of the array on the current device.  It is looked up on
// every call (cheap once the module is loaded on the device) and compared
// with the one seen last on that device: a new address means the array was
// loaded again (a new primary context after cudaDeviceReset), so the
// twiddle table is uploaded again.  The upload is a synchronous copy; it
// happens on the first call on a device and after such a reload only.
static std::mutex g_na_mu;
static void* g_na_base[256] = {};

static int noalloc_base(unsigned char** out) {
    int dev = 0;
    SC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return fail(SC_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (g_na_base[dev] != p) {
        float2 tw[kMaxL];
        for (int k = 0; k < kMaxL; ++k) {
            long double a = -2.0L * 3.141592653589793238462643383279502884L * (long double)k / (long double)kMaxL;
            tw[k] = make_float2((float)(double)cosl(a), (float)(double)sinl(a));
        }
        const size_t off = kNaBytes - kNaTw;
        e = cudaMemcpy((unsigned char*)p + off, tw, sizeof(tw), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, "twiddle upload");
        g_na_base[dev] = p;
    }
    *out = (unsigned char*)p;
    return SC_OK;
}

int native_solve_noalloc(const int32_t* grid, const double* delta, double gamma, const float* rho, float* efield,
                         cudaStream_t s) {
    for (int d = 0; d < 3; ++d) {
        if (grid[d] <= 1) return fail(SC_ERR_INVALID, "All elements of grid_size must be at least 2.");
        if (grid[d] > kNaMaxN)
            return fail(SC_ERR_UNSUPPORTED,
                        "sc_solve_noalloc handles at most %d nodes per axis (grid_size[%d] = %d); its fixed "
                        "scratch is %zu bytes",
                        kNaMaxN, d, grid[d], kNaBytes);
        if (!(delta[d] > 0) || !isfinite(delta[d])) return fail(SC_ERR_INVALID, "delta must be positive and finite");
    }
    if (!(gamma > 0) || !isfinite(gamma)) return fail(SC_ERR_INVALID, "gamma must be a positive finite number");
    unsigned char* base = nullptr;
    SC_TRY(noalloc_base(&base));
    float2* A = (float2*)base;
    float2* B = (float2*)(base + kNaA);
    float2* Cb = (float2*)(base + kNaA + kNaB);
    float2* D = (float2*)(base + kNaA + kNaB + kNaC);
    float* goct = (float*)(base + kNaA + kNaB + kNaC + kNaD);
    float2* S = (float2*)(base + kNaA + kNaB + kNaC + kNaD + kNaGoct);
    float* gfree = (float*)(base + kNaA + kNaB + kNaC + kNaD + kNaGoct + kNaGspec);
    double* fnear = (double*)(base + kNaA + kNaB + kNaC + kNaD + kNaGoct + kNaGspec + kNaGfree);
    const float2* tw = (const float2*)(base + kNaBytes - kNaTw);

    const int nx = grid[0], ny = grid[1], nz = grid[2];
    NativeWork w;  // sizes only; no buffer of it is used
    for (int d = 0; d < 3; ++d) {
        int L = 4;
        while (L < 2 * grid[d] - 1) L *= 2;
        w.L[d] = L;
        w.log2L[d] = ilog2(L);
    }
    w.Hx = w.L[0] / 2 + 1;
    const int Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    const int Hy = Ly / 2 + 1, Hz = Lz / 2 + 1;

    // Green function: the same kernels as the mesh path (free space)
    OctantGeom g;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.image = 0;
    g.dx = delta[0];
    g.dy = delta[1];
    g.dz = delta[2] * gamma;
    g.offw = 0.0;
    g.gamma = gamma;
    g.hmax = 0.5 * fmax(g.dx, fmax(g.dy, g.dz));
    g.scale = kFpei / ((double)Lx * Ly * Lz);
    g.cs = (int64_t)nx * ny * (2 * nz - 1);
    g.ux = (float)(g.dx / g.hmax);
    g.uy = (float)(g.dy / g.hmax);
    g.uz = (float)(g.dz / g.hmax);
    g.uoff = 0.f;
    g.kxy = (float)(g.gamma * g.scale / (8.0 * g.hmax * g.hmax));
    g.kz = (float)(g.scale / (8.0 * g.hmax * g.hmax));
    {
        const double reach = kNearRatio * g.hmax;
        g.nbx = (int)fmin((double)nx, floor(reach / g.dx) + 2.0);
        g.nby = (int)fmin((double)ny, floor(reach / g.dy) + 2.0);
        g.bz0 = 0;
        g.bz1 = (int)fmin((double)nz, ceil(reach / g.dz) + 2.0);
    }
    g.fnear = fnear;
    const int64_t nfar = 3 * (int64_t)(g.nbx + 1) * (g.nby + 1) * (g.bz1 - g.bz0 + 1);
    k_igf_near_F<<<(nfar + 31) / 32, 32, 0, s>>>(fnear, g);
    SC_LAUNCH_CHECK("k_igf_near_F");
    const int64_t cells = (int64_t)nx * ny * nz;
    k_igf_octant<<<(cells + 255) / 256, 256, 0, s>>>(goct, g);
    SC_LAUNCH_CHECK("k_igf_octant");
    const int64_t scs = (int64_t)Hx * Ly * Lz;
    {
        const int lgP = pick_rows(w.log2L[0]);
        const int P = 1 << lgP;
        const size_t smem = sizeof(float2) * 2 * P * Lx + sizeof(int) * 6 * P;
        const int rows = (2 * ny - 1) * (2 * nz - 1);
        dim3 gr(((rows + 1) / 2 + P - 1) / P, 3);
        k_green_x<<<gr, 256, smem, s>>>(goct, S, nx, ny, nz, 0, Lx, w.log2L[0], Ly, Lz, Hx, lgP, g.cs, scs, tw);
        SC_LAUNCH_CHECK("k_green_x");
    }
    {
        const int lgW = pick_cols(w.log2L[1]);
        const int W = 1 << lgW;
        dim3 gr((Hx + W - 1) / W, 2 * nz - 1, 3);
        k_green_y<<<gr, 256, sizeof(float2) * 2 * W * Ly, s>>>(S, ny, nz, Ly, w.log2L[1], Lz, Hx, lgW, scs, tw);
        SC_LAUNCH_CHECK("k_green_y");
    }
    {
        const int lgW = pick_cols(w.log2L[2]);
        const int W = 1 << lgW;
        dim3 gr((Hx + W - 1) / W, Hy, 3);
        k_green_z<<<gr, 256, sizeof(float2) * 2 * W * Lz, s>>>(S, gfree, nz, 0, Ly, Lz, w.log2L[2], Hx, lgW, scs,
                                                               (int64_t)Hx * Hy * Hz, tw);
        SC_LAUNCH_CHECK("k_green_z");
    }
    // convolution passes, as the mesh path's solve_t<float>
    const int rows = ny * nz;
    {
        const int lgP = pick_rows(w.log2L[0]);
        const int P = 1 << lgP;
        k_fwd_x<float><<<((rows + 1) / 2 + P - 1) / P, 256, sizeof(float2) * 2 * P * Lx, s>>>(
            rho, A, nx, rows, Lx, w.log2L[0], Hx, lgP, tw);
        SC_LAUNCH_CHECK("k_fwd_x");
    }
    {
        const int lgW = pick_cols(w.log2L[1]);
        const int W = 1 << lgW;
        dim3 gr((Hx + W - 1) / W, nz, 1);
        k_col_fft<false, float><<<gr, 256, sizeof(float2) * 2 * W * Ly, s>>>(
            A, B, Hx, lgW, Ly, w.log2L[1], ny, Ly, Hx, (int64_t)Hx * ny, 0, Hx, (int64_t)Hx * Ly, 0, tw);
        SC_LAUNCH_CHECK("k_col_fft");
    }
    {
        GreenView gv{};
        gv.gfree = gfree;
        gv.gimg = nullptr;
        gv.Hx = Hx;
        gv.Hy = Hy;
        gv.Hz = Hz;
        gv.Ly = Ly;
        gv.Lz = Lz;
        gv.cs_free = (int64_t)Hx * Hy * Hz;
        gv.cs_img = 0;
        gv.image = 0;
        const int lgW = pick_cols(w.log2L[2]);
        const int W = 1 << lgW;
        dim3 gr((Hx + W - 1) / W, Ly);
        k_zpass<float><<<gr, 256, sizeof(float2) * 3 * W * Lz, s>>>(B, Cb, Hx, Ly, nz, Lz, w.log2L[2], lgW, gv, tw);
        SC_LAUNCH_CHECK("k_zpass");
    }
    {
        const int lgW = pick_cols(w.log2L[1]);
        const int W = 1 << lgW;
        dim3 gr((Hx + W - 1) / W, nz, 3);
        k_col_fft<true, float><<<gr, 256, sizeof(float2) * 2 * W * Ly, s>>>(
            Cb, D, Hx, lgW, Ly, w.log2L[1], Ly, ny, Hx, (int64_t)Hx * Ly, (int64_t)Hx * Ly * nz, Hx, (int64_t)Hx * ny,
            (int64_t)Hx * ny * nz, tw);
        SC_LAUNCH_CHECK("k_col_fft");
    }
    {
        const int lgP = pick_rows(w.log2L[0]);
        const int P = 1 << lgP;
        const size_t smem = sizeof(float2) * 5 * P * Lx;
        SC_CUDA(cudaFuncSetAttribute(k_inv_x<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_inv_x<float><<<((rows + 1) / 2 + P - 1) / P, 256, smem, s>>>(D, (float4*)efield, nx, rows, Lx, w.log2L[0],
                                                                       Hx, lgP, (int64_t)Hx * rows, tw);
        SC_LAUNCH_CHECK("k_inv_x");
    }
    return SC_OK;
}

}  // namespace sc
