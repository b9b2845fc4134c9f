// Hand-written adjoint of the kick (deposit -> solve -> interpolate) for the
// hand-written pipelines: d(loss)/d(x, y, z, q) from the upstream gradients
// dL/dE at the particles and, optionally, dL/dE on the mesh.  The forward
// grids are recomputed, not stored.
//
//   forward:  rho = D(x) q,  E_c = K_c * rho (+ image),  Ep_c(i) = sum W(x_i) E_c
//   adjoint:  Ebar_c = gEgrid_c + sum_i g_c(i) W(x_i)          (scatter)
//             rhobar = sum_c K_c (correlation) Ebar_c (+ image)  (3 forward
//                      transforms, one z pass with the conjugate cached
//                      Green spectra, one inverse transform)
//             dq_i   = sum W(x_i) rhobar
//             dx_i   = sum dW/dx(x_i) [q_i rhobar + sum_c g_c(i) E_c]
// The Green spectrum is the one the forward solve cached: K_c is odd in its
// own axis, so conj(K^_c) = -K^_c in free space; for the image the flipped
// charge's phase is already folded into the stored spectrum and cancels.
#include <type_traits>

#include "cells.cuh"
#include "pipeline2.cuh"

namespace sc {

Axes make_axes(const sc_mesh* m);

template <typename A>
struct ACell;
template <>
struct ACell<float> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, float& f) {
        return cell_df32(x, a, i, f);
    }
    template <typename P>
    __device__ __forceinline__ static float cvt(P v) { return f64_to_f32(v); }
    // 1/delta in FP32 (precomputed: no FP64 conversion per thread)
    __device__ __forceinline__ static float inv(const AxisP& a) { return a.invf; }
};
template <>
struct ACell<double> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, double& f) {
        return cell_dp(x, a, i, f);
    }
    template <typename P>
    __device__ __forceinline__ static double cvt(P v) { return (double)v; }
    __device__ __forceinline__ static double inv(const AxisP& a) { return a.inv; }
};

template <typename T>
__global__ void __launch_bounds__(256) k_adj_init(T* __restrict__ adjE, const typename Vec4<T>::V* __restrict__ gg,
                                                  int64_t N) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    T a = 0, b = 0, c = 0;
    if (gg) {
        const T* g = reinterpret_cast<const T*>(gg) + 4 * i;
        a = g[0];
        b = g[1];
        c = g[2];
    }
    adjE[i] = a;
    adjE[N + i] = b;
    adjE[2 * N + i] = c;
}

// Adjoint of the gather: deposit g_c(i) with the trilinear weights.
template <typename P, typename T>
__global__ void __launch_bounds__(256) k_adj_scatter(const P* __restrict__ px, const P* __restrict__ py,
                                                     const P* __restrict__ pz, const P* __restrict__ gx,
                                                     const P* __restrict__ gy, const P* __restrict__ gz, int64_t n,
                                                     Axes ax, T* __restrict__ adjE, int64_t N) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    int ix, iy, iz;
    T fx, fy, fz;
    if (!(ACell<T>::run(px[p], ax.a[0], ix, fx) & ACell<T>::run(py[p], ax.a[1], iy, fy) &
          ACell<T>::run(pz[p], ax.a[2], iz, fz)))
        return;
    const T g[3] = {gx ? ACell<T>::cvt(gx[p]) : T(0), gy ? ACell<T>::cvt(gy[p]) : T(0),
                    gz ? ACell<T>::cvt(gz[p]) : T(0)};
    const T ux = T(1) - fx, uy = T(1) - fy, uz = T(1) - fz;
    const T w[8] = {ux * uy * uz, fx * uy * uz, ux * fy * uz, fx * fy * uz,
                    ux * uy * fz, fx * uy * fz, ux * fy * fz, fx * fy * fz};
    const int nx = ax.a[0].n, ny = ax.a[1].n;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    const int64_t b = ix + sy * iy + sz * iz;
    const int64_t off[8] = {0, 1, sy, 1 + sy, sz, 1 + sz, sy + sz, 1 + sy + sz};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (g[c] == T(0)) continue;
        T* r = adjE + c * N + b;
#pragma unroll
        for (int k = 0; k < 8; ++k) atomicAdd(r + off[k], g[c] * w[k]);
    }
}

// The same scatter for mixed meshes with the vector deposit's layout: per
// component with an upstream gradient, two 16-byte vector atomics into that
// component's per-cell corner slots (corner + 8N*c), summed onto the nodes
// afterwards by corner_sum_launch.
template <typename P>
__global__ void __launch_bounds__(256) k_adj_scatter_vec(const P* __restrict__ px, const P* __restrict__ py,
                                                         const P* __restrict__ pz, const P* __restrict__ gx,
                                                         const P* __restrict__ gy, const P* __restrict__ gz,
                                                         int64_t n, Axes ax, float4* __restrict__ corner, int64_t N) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    int ix, iy, iz;
    float fx, fy, fz;
    if (!(cell_df32(px[p], ax.a[0], ix, fx) & cell_df32(py[p], ax.a[1], iy, fy) &
          cell_df32(pz[p], ax.a[2], iz, fz)))
        return;
    const P* gp[3] = {gx, gy, gz};
    const float ux = 1.0f - fx, uy = 1.0f - fy, uz = 1.0f - fz;
    const int64_t cell = ix + (int64_t)ax.a[0].n * (iy + (int64_t)ax.a[1].n * iz);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (!gp[c]) continue;
        const float g = f64_to_f32(gp[c][p]);
        float4* r = corner + 2 * (c * N + cell);
        atomicAdd(r, make_float4(g * ux * uy * uz, g * fx * uy * uz, g * ux * fy * uz, g * fx * fy * uz));
        atomicAdd(r + 1, make_float4(g * ux * uy * fz, g * fx * uy * fz, g * ux * fy * fz, g * fx * fy * fz));
    }
}

// z pass of the adjoint: three forward z transforms of Ebar_c, correlation
// with the Green spectra summed over components, one inverse z transform.
template <typename T>
__global__ void __launch_bounds__(256) k_adj_zpass(const typename Cplx<T>::T2* __restrict__ C,
                                                   typename Cplx<T>::T2* __restrict__ B, int Hx, int Ly, int nz,
                                                   int Lz, int logLz, int lgW, GreenView gv,
                                                   const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int W = 1 << lgW;
    const int n = W << logLz;
    T2* acc = reinterpret_cast<T2*>(smraw);
    T2* a = acc + n;
    T2* b = a + n;
    const int kx0 = blockIdx.x << lgW;
    const int ky = blockIdx.y;
    const int64_t plane = (int64_t)Hx * Ly;
    const int kyf = ky <= Ly / 2 ? ky : Ly - ky;
    const T ysign = ky <= Ly / 2 ? T(1) : T(-1);
    const T* gf = reinterpret_cast<const T*>(gv.gfree);
    const T2* gi = reinterpret_cast<const T2*>(gv.gimg);
    const int halfz = Lz >> 1;
    for (int it = threadIdx.x; it < n; it += blockDim.x) acc[it] = Cplx<T>::make(0, 0);
    for (int comp = 0; comp < 3; ++comp) {
        const T2* Cc = C + comp * (plane * nz);
        for (int it = threadIdx.x; it < n; it += blockDim.x) {
            const int z = it >> lgW, kx = kx0 + (it & (W - 1));
            T2 v = Cplx<T>::make(0, 0);
            if (z < nz && kx < Hx) v = Cc[kx + (int64_t)Hx * ky + plane * z];
            a[it] = v;
        }
        __syncthreads();
        const T2* e = smem_fft<false>(a, b, Lz, logLz, lgW, tw);
        const T* gfc = gf + comp * gv.cs_free + (int64_t)gv.Hx * kyf;
        const T2* gic = gi + comp * gv.cs_img + (int64_t)gv.Hx * kyf;
        for (int it = threadIdx.x; it < n; it += blockDim.x) {
            const int kz = it >> lgW, w = it & (W - 1);
            const int kx = kx0 + w;
            if (kx >= Hx) continue;
            const int kzf = kz <= halfz ? kz : Lz - kz;
            T sg = T(1);
            if (comp == 1) sg = ysign;
            if (comp == 2 && kz > halfz) sg = T(-1);
            const T g = sg * gfc[kx + (int64_t)gv.Hx * gv.Hy * kzf];
            const T2 p = e[it];
            // p * conj(i g) = p * (-i g)
            T2 r = acc[it];
            r.x += p.y * g;
            r.y -= p.x * g;
            if (gv.image) {
                const int kzm = (Lz - kz) & (Lz - 1);
                T2 gc = img_at(gic + kx, (int64_t)gv.Hx * gv.Hy, kzm, gv, comp);
                if (comp == 1) {
                    gc.x *= ysign;
                    gc.y *= ysign;
                }
                r = cadd(r, cmulc(e[(kzm << lgW) + w], gc));
            }
            acc[it] = r;
        }
        __syncthreads();
    }
    const T2* res = smem_fft<true>(acc, a, Lz, logLz, lgW, tw);
    for (int it = threadIdx.x; it < (nz << lgW); it += blockDim.x) {
        const int z = it >> lgW, kx = kx0 + (it & (W - 1));
        if (kx < Hx) B[kx + (int64_t)Hx * ky + plane * z] = res[it];
    }
}

template <typename P, typename T>
__device__ __forceinline__ P out_cast(T v) {
    return (P)v;
}
template <>
__device__ __forceinline__ double out_cast<double, float>(float v) {
    return f32_to_f64(v);
}

// Particle gradients from the packed nodes (Ex, Ey, Ez, rhobar).
template <typename P, typename T>
__global__ void __launch_bounds__(256) k_adj_particles(const P* __restrict__ px, const P* __restrict__ py,
                                                       const P* __restrict__ pz, const P* __restrict__ pq,
                                                       const P* __restrict__ gx, const P* __restrict__ gy,
                                                       const P* __restrict__ gz, int64_t n, Axes ax,
                                                       const T* __restrict__ E4, P* __restrict__ dx,
                                                       P* __restrict__ dy, P* __restrict__ dz, P* __restrict__ dq) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    int ix, iy, iz;
    T fx, fy, fz;
    if (!(ACell<T>::run(px[p], ax.a[0], ix, fx) & ACell<T>::run(py[p], ax.a[1], iy, fy) &
          ACell<T>::run(pz[p], ax.a[2], iz, fz))) {
        dx[p] = P(0);
        dy[p] = P(0);
        dz[p] = P(0);
        dq[p] = P(0);
        return;
    }
    const T q = ACell<T>::cvt(pq[p]);
    const T g0 = gx ? ACell<T>::cvt(gx[p]) : T(0), g1 = gy ? ACell<T>::cvt(gy[p]) : T(0),
            g2 = gz ? ACell<T>::cvt(gz[p]) : T(0);
    const int nx = ax.a[0].n, ny = ax.a[1].n;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    const int64_t b = ix + sy * iy + sz * iz;
    const T wx[2] = {T(1) - fx, fx}, wy[2] = {T(1) - fy, fy}, wz[2] = {T(1) - fz, fz};
    T sq = 0, gxs = 0, gys = 0, gzs = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int a0 = k & 1, b0 = (k >> 1) & 1, c0 = k >> 2;
        const T* e = E4 + 4 * (b + a0 + sy * b0 + sz * c0);
        const T ex = e[0], ey = e[1], ez = e[2], rb = e[3];
        const T S = q * rb + g0 * ex + g1 * ey + g2 * ez;
        sq += wx[a0] * wy[b0] * wz[c0] * rb;
        gxs += (a0 ? T(1) : T(-1)) * wy[b0] * wz[c0] * S;
        gys += (b0 ? T(1) : T(-1)) * wx[a0] * wz[c0] * S;
        gzs += (c0 ? T(1) : T(-1)) * wx[a0] * wy[b0] * S;
    }
    dq[p] = out_cast<P, T>(sq);
    dx[p] = out_cast<P, T>(gxs * ACell<T>::inv(ax.a[0]));
    dy[p] = out_cast<P, T>(gys * ACell<T>::inv(ax.a[1]));
    dz[p] = out_cast<P, T>(gzs * ACell<T>::inv(ax.a[2]));
}

template <typename P, typename T>
static int adjoint_t(sc_mesh* m, const P* x, const P* y, const P* z, const P* q, int64_t n, int at_cathode,
                     const P* gex, const P* gey, const P* gez, const void* ggrid, P* dx, P* dy, P* dz, P* dq,
                     cudaStream_t s) {
    using T2 = typename Cplx<T>::T2;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const T2* tw = twiddles<T>(ctx);
    // forward recompute: rho and E for these particles (a Green build, when
    // needed, overlaps the deposit on the mesh's side stream)
    cudaEvent_t ready = nullptr;
    // (the FP64 adjoint z pass reads an FP64 free-space spectrum)
    if (n > 0)
        SC_TRY(native_green_async(m, at_cathode, s, &ready, false));
    else
        SC_TRY(native_ensure_green(m, at_cathode, s, false));
    const int dmode = m->precision == SC_PREC_MIXED ? SC_DEPOSIT_VECTOR : SC_DEPOSIT_ATOMIC;
    const bool assign = deposit_assigns(m, dmode);
    int st = assign || cudaMemsetAsync(m->rho, 0, sizeof(T) * m->N, s) == cudaSuccess
                 ? SC_OK
                 : cuda_fail(cudaGetLastError(), "memset");
    if (st == SC_OK) st = deposit_launch(m, x, y, z, q, n, sizeof(P) == 8 ? SC_F64 : SC_F32, dmode, s, assign);
    if (st != SC_OK) {
        if (ready) cudaStreamWaitEvent(s, ready, 0);
        return st;
    }
    SC_TRY(native_solve(m, at_cathode, s, ready));
    NativeWork& w = m->nw;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    const int64_t N = m->N;
    if (!w.adjE) SC_CUDA(dev_alloc(&w.adjE, sizeof(T) * 3 * N));
    T* adjE = (T*)w.adjE;
    const Axes ax = make_axes(m);
    k_adj_init<T><<<(N + 255) / 256, 256, 0, s>>>(adjE, (const typename Vec4<T>::V*)ggrid, N);
    SC_LAUNCH_CHECK("k_adj_init");
    if ((gex || gey || gez) && n > 0) {
        if (std::is_same<T, float>::value) {
            const size_t slice = sizeof(float) * 8 * (size_t)N;
            if (!w.adjcorner) SC_CUDA(dev_alloc(&w.adjcorner, 3 * slice));
            const P* g[3] = {gex, gey, gez};
            for (int c = 0; c < 3; ++c)
                if (g[c]) SC_CUDA(cudaMemsetAsync((char*)w.adjcorner + c * slice, 0, slice, s));
            k_adj_scatter_vec<P><<<(n + 255) / 256, 256, 0, s>>>(x, y, z, gex, gey, gez, n, ax,
                                                                 (float4*)w.adjcorner, N);
            SC_LAUNCH_CHECK("k_adj_scatter_vec");
            m->launches += 1;
            for (int c = 0; c < 3; ++c)
                if (g[c]) SC_TRY(corner_sum_launch(m, (const float*)((char*)w.adjcorner + c * slice),
                                                   (float*)(adjE + c * N), s));
        } else {
            k_adj_scatter<P, T><<<(n + 255) / 256, 256, 0, s>>>(x, y, z, gex, gey, gez, n, ax, adjE, N);
            SC_LAUNCH_CHECK("k_adj_scatter");
            m->launches += 1;
        }
    }
    T2* A = (T2*)w.A;
    T2* B = (T2*)w.B;
    T2* C = (T2*)w.C;
    T2* D = (T2*)w.D;
    const int rows = ny * nz;
    const int64_t dcs = (int64_t)Hx * ny * nz;
    const bool two = std::is_same<T, float>::value && fft_engine() == 0;
    // forward x and y of the three components: fused per (z plane,
    // component) where the plane fits (3 nz CTAs), else the separate passes
    if (two && launch2_fwd_xy(w.log2L[0], w.log2L[1], (const float*)adjE, (float2*)C, nx, ny, nz, Hx,
                              (const float2*)tw, s, m->fused_smem_cap, 3, N, (int64_t)Hx * Ly * nz)) {
        SC_LAUNCH_CHECK("k2_fwd_xy");
        m->launches -= 3;  // one launch for the four below
    } else {
        for (int c = 0; c < 3; ++c)
            if (!(two && launch2_fwd_x(w.log2L[0], (const float*)(adjE + c * N), (float2*)(D + c * dcs), nx, rows,
                                       Hx, (const float2*)tw, s)))
                SC_TRY(run_fwd_x<T>(adjE + c * N, D + c * dcs, nx, rows, w, tw, s));
        if (!(two && launch2_col(false, w.log2L[1], (const float2*)D, (float2*)C, Hx, ny, Ly, Hx, (int64_t)Hx * ny,
                                 dcs, Hx, (int64_t)Hx * Ly, (int64_t)Hx * Ly * nz, nz, 3, (const float2*)tw, s)))
            SC_TRY(run_col<false, T>(D, C, Hx, Ly, w.log2L[1], ny, Ly, Hx, (int64_t)Hx * ny, dcs, Hx,
                                     (int64_t)Hx * Ly, (int64_t)Hx * Ly * nz, nz, 3, tw, s));
    }
    if (two && launch2_adj_zpass(w.log2L[2], (const float2*)C, (float2*)B, Hx, Ly, nz,
                                 make_green_view(w, at_cathode ? 1 : 0), (const float2*)tw, s)) {
        SC_LAUNCH_CHECK("k2_adj_zpass");
    } else {
        const GreenView gv = make_green_view(w, at_cathode ? 1 : 0);
        const int lgW = pick_cols(w.log2L[2]);
        const int W = 1 << lgW;
        const size_t smem = sizeof(T2) * 3 * W * Lz;
        SC_TRY(set_smem(k_adj_zpass<T>, smem));
        dim3 grid((Hx + W - 1) / W, Ly);
        k_adj_zpass<T><<<grid, 256, smem, s>>>(C, B, Hx, Ly, nz, Lz, w.log2L[2], lgW, gv, tw);
        SC_LAUNCH_CHECK("k_adj_zpass");
    }
    // inverse y and x of rhobar^ into lane 3 of the packed nodes: fused per z
    // plane where the plane fits, else the separate passes
    if (two && launch2_inv_yx(w.log2L[0], w.log2L[1], (const float2*)B, (float4*)m->efield, nx, ny, nz, Hx,
                              (const float2*)tw, s, m->fused_smem_cap, 1, 3)) {
        SC_LAUNCH_CHECK("k2_inv_yx");
        m->launches -= 1;  // one launch for the two passes
    } else {
        if (!(two && launch2_col(true, w.log2L[1], (const float2*)B, (float2*)A, Hx, Ly, ny, Hx, (int64_t)Hx * Ly,
                                 0, Hx, (int64_t)Hx * ny, 0, nz, 1, (const float2*)tw, s)))
            SC_TRY(run_col<true, T>(B, A, Hx, Ly, w.log2L[1], Ly, ny, Hx, (int64_t)Hx * Ly, 0, Hx, (int64_t)Hx * ny, 0,
                                    nz, 1, tw, s));
        if (two &&
            launch2_inv_x1(w.log2L[0], (const float2*)A, (float*)m->efield, nx, rows, Hx, (const float2*)tw, s)) {
            SC_LAUNCH_CHECK("k2_inv_x1");
        } else {
            const int lgP = pick_rows(w.log2L[0]);
            const int P_ = 1 << lgP;
            const size_t smem = sizeof(T2) * 2 * P_ * Lx;
            SC_TRY(set_smem(k_inv_x1<T>, smem));
            const int pairs = (rows + 1) / 2;
            k_inv_x1<T><<<(pairs + P_ - 1) / P_, 256, smem, s>>>(A, (T*)m->efield, nx, rows, Lx, w.log2L[0], Hx, lgP,
                                                                tw);
            SC_LAUNCH_CHECK("k_inv_x1");
        }
    }
    k_adj_particles<P, T><<<(n + 255) / 256, 256, 0, s>>>(x, y, z, q, gex, gey, gez, n, ax, (const T*)m->efield, dx,
                                                         dy, dz, dq);
    SC_LAUNCH_CHECK("k_adj_particles");
    m->launches += 9;  // init, 3 x fwd_x, fwd_y, z pass, inverse y, inverse x, particles
    return SC_OK;
}

int adjoint_launch(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
                   int at_cathode, const void* gex, const void* gey, const void* gez, const void* ggrid, void* dx,
                   void* dy, void* dz, void* dq, cudaStream_t s) {
    if (m->precision == SC_PREC_PLAIN64)
        return fail(SC_ERR_UNSUPPORTED, "the adjoint needs a hand-written pipeline mesh (precision fp64 or mixed)");
    if (m->precision == SC_PREC_MIXED) {
        if (dtype == SC_F64)
            return adjoint_t<double, float>(m, (const double*)x, (const double*)y, (const double*)z, (const double*)q,
                                            n, at_cathode, (const double*)gex, (const double*)gey, (const double*)gez,
                                            ggrid, (double*)dx, (double*)dy, (double*)dz, (double*)dq, s);
        return adjoint_t<float, float>(m, (const float*)x, (const float*)y, (const float*)z, (const float*)q, n,
                                       at_cathode, (const float*)gex, (const float*)gey, (const float*)gez, ggrid,
                                       (float*)dx, (float*)dy, (float*)dz, (float*)dq, s);
    }
    if (dtype == SC_F64)
        return adjoint_t<double, double>(m, (const double*)x, (const double*)y, (const double*)z, (const double*)q, n,
                                         at_cathode, (const double*)gex, (const double*)gey, (const double*)gez, ggrid,
                                         (double*)dx, (double*)dy, (double*)dz, (double*)dq, s);
    return adjoint_t<float, double>(m, (const float*)x, (const float*)y, (const float*)z, (const float*)q, n,
                                    at_cathode, (const float*)gex, (const float*)gey, (const float*)gez, ggrid,
                                    (float*)dx, (float*)dy, (float*)dz, (float*)dq, s);
}

}  // namespace sc
