// Trilinear field interpolation, src/interpolation.jl:17-128.
//
// gather_plain: the reference's kernel restated: FP64 IEEE-division cell
//   index, 8 weights (:46-53), 24 scalar loads from the component-planar
//   efield (:56-85), same summation order; output in the particle type.
// gather_packed: the hand-written pipelines read the packed (Ex,Ey,Ez,0)
//   node as one 16-byte (FP32) or 32-byte (FP64) load, 8 loads per particle.
// Out-of-range particles get E = 0 and are counted (the reference reads out
// of bounds there).
#include "batch.cuh"
#include "cells.cuh"
#include "dd.cuh"
#include "sc_internal.cuh"

namespace sc {

Axes make_axes(const sc_mesh* m);

template <typename P>
__global__ void __launch_bounds__(256) gather_plain(const P* __restrict__ px, const P* __restrict__ py,
                                                    const P* __restrict__ pz, int64_t n, Axes ax,
                                                    const double* __restrict__ ef, P* __restrict__ ex,
                                                    P* __restrict__ ey, P* __restrict__ ez,
                                                    unsigned long long* __restrict__ oob) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    int ix, iy, iz;
    double dx, dy, dz;
    const bool ok = cell_exact(px[p], ax.a[0], ix, dx) & cell_exact(py[p], ax.a[1], iy, dy) &
                    cell_exact(pz[p], ax.a[2], iz, dz);
    if (!ok) {
        atomicAdd(oob, 1ull);
        ex[p] = P(0);
        ey[p] = P(0);
        ez[p] = P(0);
        return;
    }
    const double w000 = (1 - dx) * (1 - dy) * (1 - dz);
    const double w100 = dx * (1 - dy) * (1 - dz);
    const double w010 = (1 - dx) * dy * (1 - dz);
    const double w110 = dx * dy * (1 - dz);
    const double w001 = (1 - dx) * (1 - dy) * dz;
    const double w101 = dx * (1 - dy) * dz;
    const double w011 = (1 - dx) * dy * dz;
    const double w111 = dx * dy * dz;
    const int nx = ax.a[0].n, ny = ax.a[1].n, nz = ax.a[2].n;
    const int64_t sy = nx, sz = (int64_t)nx * ny, N = sz * nz;
    const int64_t b = ix + sy * iy + sz * iz;
    double out[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double* e = ef + c * N + b;
        // left-to-right sum without FMA contraction, as Julia evaluates it
        double acc = __dmul_rn(e[0], w000);
        acc = __dadd_rn(acc, __dmul_rn(e[1], w100));
        acc = __dadd_rn(acc, __dmul_rn(e[sy], w010));
        acc = __dadd_rn(acc, __dmul_rn(e[1 + sy], w110));
        acc = __dadd_rn(acc, __dmul_rn(e[sz], w001));
        acc = __dadd_rn(acc, __dmul_rn(e[1 + sz], w101));
        acc = __dadd_rn(acc, __dmul_rn(e[sy + sz], w011));
        out[c] = __dadd_rn(acc, __dmul_rn(e[1 + sy + sz], w111));
    }
    ex[p] = (P)out[0];
    ey[p] = (P)out[1];
    ez[p] = (P)out[2];
}

template <typename T>
struct Packed;
template <>
struct Packed<float> {
    using V = float4;
};
template <>
struct Packed<double> {
    using V = dnode4;
};

// One 32-byte load (sm_100+) of a 32-byte aligned FP64 node, read-only path.
__device__ __forceinline__ dnode4 ldg4(const dnode4* p) {
    dnode4 r;
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];" : "=d"(r.x), "=d"(r.y), "=d"(r.z), "=d"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

template <typename P, typename A>
__device__ __forceinline__ P to_out(A v);
template <>
__device__ __forceinline__ float to_out<float, float>(float v) { return v; }
template <>
__device__ __forceinline__ double to_out<double, float>(float v) { return f32_to_f64(v); }
template <>
__device__ __forceinline__ float to_out<float, double>(double v) { return (float)v; }
template <>
__device__ __forceinline__ double to_out<double, double>(double v) { return v; }

template <typename A>
struct GCell;
template <>
struct GCell<float> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, float& f) {
        return cell_df32(x, a, i, f);
    }
};
template <>
struct GCell<double> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, double& f) {
        return cell_dp(x, a, i, f);
    }
};

// Particles per thread of the packed gather: positions of all of them are
// loaded first, then all their 8 node loads are issued before the sums.
#ifndef SC_GATH_PT
#define SC_GATH_PT 2
#endif
#ifndef SC_GATH_MINB
#define SC_GATH_MINB 1
#endif
constexpr int kGathPerThread = SC_GATH_PT;

// Body of one CTA: particles blk * 256 * kGathPerThread + ... of the bunch.
// wait_after_positions: wait for the preceding grid (programmatic launch)
// after the position loads rather than before the body; for callers whose
// positions no preceding grid writes.
template <typename P, typename A>
__device__ __forceinline__ void gather_packed_body(const P* __restrict__ px, const P* __restrict__ py,
                                                   const P* __restrict__ pz, int64_t n, const Axes& ax,
                                                   const typename Packed<A>::V* __restrict__ ef, P* __restrict__ ex,
                                                   P* __restrict__ ey, P* __restrict__ ez,
                                                   unsigned long long* __restrict__ oob, int64_t blk,
                                                   bool wait_after_positions = false) {
    using V = typename Packed<A>::V;
    const int64_t base = blk * (blockDim.x * kGathPerThread) + threadIdx.x;
    P x[kGathPerThread], y[kGathPerThread], z[kGathPerThread];
#pragma unroll
    for (int k = 0; k < kGathPerThread; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        const bool in = p < n;
        x[k] = in ? __ldg(px + p) : P(0);
        y[k] = in ? __ldg(py + p) : P(0);
        z[k] = in ? __ldg(pz + p) : P(0);
    }
    if (wait_after_positions) pdl_wait();
    const int nx = ax.a[0].n, ny = ax.a[1].n;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    const int64_t off[8] = {0, 1, sy, 1 + sy, sz, 1 + sz, sy + sz, 1 + sy + sz};
    A w[kGathPerThread][8];
    V v[kGathPerThread][8];
    bool ok[kGathPerThread];
#pragma unroll
    for (int k = 0; k < kGathPerThread; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        int ix = 0, iy = 0, iz = 0;
        A dx = 0, dy = 0, dz = 0;
        ok[k] = p < n && (GCell<A>::run(x[k], ax.a[0], ix, dx) & GCell<A>::run(y[k], ax.a[1], iy, dy) &
                          GCell<A>::run(z[k], ax.a[2], iz, dz));
        const A ux = A(1) - dx, uy = A(1) - dy, uz = A(1) - dz;
        // interpolation.jl:46-53
        w[k][0] = ux * uy * uz;
        w[k][1] = dx * uy * uz;
        w[k][2] = ux * dy * uz;
        w[k][3] = dx * dy * uz;
        w[k][4] = ux * uy * dz;
        w[k][5] = dx * uy * dz;
        w[k][6] = ux * dy * dz;
        w[k][7] = dx * dy * dz;
        const V* e = ef + (ok[k] ? (ix + sy * iy + sz * iz) : 0);
#pragma unroll
        for (int c = 0; c < 8; ++c) v[k][c] = ok[k] ? ldg4(e + off[c]) : V{};
    }
    unsigned skipped = 0;
#pragma unroll
    for (int k = 0; k < kGathPerThread; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        if (p >= n) break;
        A sx = 0, sy_ = 0, sz_ = 0;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            sx += v[k][c].x * w[k][c];
            sy_ += v[k][c].y * w[k][c];
            sz_ += v[k][c].z * w[k][c];
        }
        if (!ok[k]) {
            ++skipped;
            sx = sy_ = sz_ = A(0);
        }
        ex[p] = to_out<P, A>(sx);
        ey[p] = to_out<P, A>(sy_);
        ez[p] = to_out<P, A>(sz_);
    }
    if (skipped) atomicAdd(oob, (unsigned long long)skipped);
}

template <typename P, typename A>
__global__ void __launch_bounds__(256, SC_GATH_MINB) gather_packed(const P* __restrict__ px, const P* __restrict__ py,
                                                     const P* __restrict__ pz, int64_t n, Axes ax,
                                                     const typename Packed<A>::V* __restrict__ ef,
                                                     P* __restrict__ ex, P* __restrict__ ey, P* __restrict__ ez,
                                                     unsigned long long* __restrict__ oob, int early) {
    // the field (and, unless `early`, possibly the positions) come from preceding grids
    if (!early) pdl_wait();
    gather_packed_body<P, A>(px, py, pz, n, ax, ef, ex, ey, ez, oob, blockIdx.x, early != 0);
}

// FP64 meshes in double-FP32 mode (sc_mesh_set_fp64_arithmetic): the
// packed gather with the cell fractions (cell_dd), the weights and the sums
// in double-FP32 (dd.cuh), so that the FP64 units see only the output's one
// addition per component.  The FP64 node values are split with integer
// operations.  Ex and Ey of a corner share the paired FP32 instructions, and
// so do Ez of two corners.
template <typename P>
__device__ __forceinline__ P dd_out(float h, float l);
template <>
__device__ __forceinline__ double dd_out<double>(float h, float l) {
    return dd_widen(h) + dd_widen(l);
}
template <>
__device__ __forceinline__ float dd_out<float>(float h, float l) {
    return h + l;
}

// One particle per thread, two CTAs per SM: the double-FP32 sums are
// longer dependent chains than gather_packed's, so more warps hide them.
constexpr int kGathDdPerThread = 1;
template <typename P>
__global__ void __launch_bounds__(256, 2) gather_dd(const P* __restrict__ px, const P* __restrict__ py,
                                                   const P* __restrict__ pz, int64_t n, Axes ax,
                                                   const dnode4* __restrict__ ef, P* __restrict__ ex,
                                                   P* __restrict__ ey, P* __restrict__ ez,
                                                   unsigned long long* __restrict__ oob, int early) {
    constexpr int K = kGathDdPerThread;
    if (!early) pdl_wait();
    const int64_t base = blockIdx.x * (int64_t)(blockDim.x * K) + threadIdx.x;
    P x[K], y[K], z[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        const bool in = p < n;
        x[k] = in ? __ldg(px + p) : P(0);
        y[k] = in ? __ldg(py + p) : P(0);
        z[k] = in ? __ldg(pz + p) : P(0);
    }
    if (early) pdl_wait();
    const int nx = ax.a[0].n, ny = ax.a[1].n;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    const int64_t off[8] = {0, 1, sy, 1 + sy, sz, 1 + sz, sy + sz, 1 + sy + sz};
    float2 w[K][8];
    dnode4 v[K][8];
    bool ok[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        int ix = 0, iy = 0, iz = 0;
        float2 dx = make_float2(0.f, 0.f), dy = dx, dz = dx;
        ok[k] = p < n && (cell_dd(x[k], ax.a[0], ix, dx.x, dx.y) & cell_dd(y[k], ax.a[1], iy, dy.x, dy.y) &
                          cell_dd(z[k], ax.a[2], iz, dz.x, dz.y));
        const float2 ux = ddr_one_minus(dx), uy = ddr_one_minus(dy), uz = ddr_one_minus(dz);
        // interpolation.jl:46-53, as (x y) products times the z factor
        const float2 q0 = ddr_mul(ux, uy), q1 = ddr_mul(dx, uy), q2 = ddr_mul(ux, dy), q3 = ddr_mul(dx, dy);
        w[k][0] = ddr_mul(q0, uz);
        w[k][1] = ddr_mul(q1, uz);
        w[k][2] = ddr_mul(q2, uz);
        w[k][3] = ddr_mul(q3, uz);
        w[k][4] = ddr_mul(q0, dz);
        w[k][5] = ddr_mul(q1, dz);
        w[k][6] = ddr_mul(q2, dz);
        w[k][7] = ddr_mul(q3, dz);
        const dnode4* e = ef + (ok[k] ? (ix + sy * iy + sz * iz) : 0);
#pragma unroll
        for (int c = 0; c < 8; ++c) v[k][c] = ok[k] ? ldg4(e + off[c]) : dnode4{};
    }
    unsigned skipped = 0;
    const ddc zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        if (p >= n) break;
        ddc axy = zero, az = zero;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            ddc e;
            dd_split(v[k][c].x, e.h.x, e.l.x);
            dd_split(v[k][c].y, e.h.y, e.l.y);
            axy = dd_add(axy, dd_scale(e, w[k][c].x, w[k][c].y));
        }
#pragma unroll
        for (int c = 0; c < 8; c += 2) {
            ddc e;
            dd_split(v[k][c].z, e.h.x, e.l.x);
            dd_split(v[k][c + 1].z, e.h.y, e.l.y);
            float2 pp, pe;
            dd_prod2(e.h, e.l, make_float2(w[k][c].x, w[k][c + 1].x), make_float2(w[k][c].y, w[k][c + 1].y), pp, pe);
            az = dd_add(az, dd_renorm(pp, pe));
        }
        // Ez: the two lanes' sums added
        const float zs = az.h.x + az.h.y;
        const float zb = zs - az.h.x;
        const float ze = ((az.h.x - (zs - zb)) + (az.h.y - zb)) + (az.l.x + az.l.y);
        const float zh = zs + ze, zl = ze - (zh - zs);
        if (!ok[k]) {
            ++skipped;
            ex[p] = ey[p] = ez[p] = P(0);
            continue;
        }
        ex[p] = dd_out<P>(axy.h.x, axy.l.x);
        ey[p] = dd_out<P>(axy.h.y, axy.l.y);
        ez[p] = dd_out<P>(zh, zl);
    }
    if (skipped) atomicAdd(oob, (unsigned long long)skipped);
}

// Staged batch kick (batch.cuh): the gather of a group of bunches in one launch.
// (three CTAs per SM, as the single-mesh gather's 80 registers allow; the
// table lookup would otherwise push it to 128 and two)
template <typename P>
__global__ void __launch_bounds__(256, 3) kb_gather(const BunchDesc* __restrict__ tab,
                                                               const CtaRef* __restrict__ map) {
    const CtaRef r = map[blockIdx.x];
    const BunchDesc& b = tab[r.item];
    const Axes ax = b.ax;
    pdl_wait();
    gather_packed_body<P, float>((const P*)b.x, (const P*)b.y, (const P*)b.z, b.n, ax, b.efield, (P*)b.ex, (P*)b.ey,
                                 (P*)b.ez, b.oob, r.local);
}

int batch_gather_particles_per_cta() { return 256 * kGathPerThread; }

int batch_gather_launch(const BunchDesc* tab, const CtaRef* map, int64_t ctas, int dtype, cudaStream_t s) {
    if (ctas == 0) return SC_OK;
    if (dtype == SC_F64)
        launch_pdl(kb_gather<double>, (unsigned)ctas, 256, 0, s, tab, map);
    else
        launch_pdl(kb_gather<float>, (unsigned)ctas, 256, 0, s, tab, map);
    SC_LAUNCH_CHECK("kb_gather");
    return SC_OK;
}

int gather_launch(sc_mesh* m, const void* x, const void* y, const void* z, int64_t n, int dtype, void* ex,
                  void* ey, void* ez, cudaStream_t s, bool early) {
    const int e = early ? 1 : 0;
    const Axes ax = make_axes(m);
    const int64_t blocks = (n + 255) / 256;
    if (m->precision == SC_PREC_PLAIN64) {
        if (dtype == SC_F64)
            gather_plain<double><<<blocks, 256, 0, s>>>((const double*)x, (const double*)y, (const double*)z, n, ax,
                                                       (const double*)m->efield, (double*)ex, (double*)ey,
                                                       (double*)ez, m->oob);
        else
            gather_plain<float><<<blocks, 256, 0, s>>>((const float*)x, (const float*)y, (const float*)z, n, ax,
                                                      (const double*)m->efield, (float*)ex, (float*)ey, (float*)ez,
                                                      m->oob);
        SC_LAUNCH_CHECK("gather_plain");
        m->launches += 1;
        return SC_OK;
    }
    const int64_t gblocks = (n + 256 * kGathPerThread - 1) / (256 * kGathPerThread);
    if (m->precision == SC_PREC_MIXED) {
        if (dtype == SC_F64)
            launch_pdl(gather_packed<double, float>, (unsigned)gblocks, 256, 0, s, (const double*)x, (const double*)y,
                                                               (const double*)z, n, ax, (const float4*)m->efield,
                                                               (double*)ex, (double*)ey, (double*)ez, m->oob, e);
        else
            launch_pdl(gather_packed<float, float>, (unsigned)gblocks, 256, 0, s, (const float*)x, (const float*)y, (const float*)z, n,
                                                              ax, (const float4*)m->efield, (float*)ex, (float*)ey,
                                                              (float*)ez, m->oob, e);
    } else if (m->df32) {
        const unsigned dblocks = (unsigned)((n + 256 * kGathDdPerThread - 1) / (256 * kGathDdPerThread));
        if (dtype == SC_F64)
            launch_pdl(gather_dd<double>, dblocks, 256, 0, s, (const double*)x, (const double*)y,
                       (const double*)z, n, ax, (const dnode4*)m->efield, (double*)ex, (double*)ey, (double*)ez,
                       m->oob, e);
        else
            launch_pdl(gather_dd<float>, dblocks, 256, 0, s, (const float*)x, (const float*)y,
                       (const float*)z, n, ax, (const dnode4*)m->efield, (float*)ex, (float*)ey, (float*)ez, m->oob,
                       e);
    } else {
        if (dtype == SC_F64)
            launch_pdl(gather_packed<double, double>, (unsigned)gblocks, 256, 0, s, (const double*)x, (const double*)y,
                                                                (const double*)z, n, ax, (const dnode4*)m->efield,
                                                                (double*)ex, (double*)ey, (double*)ez, m->oob, e);
        else
            launch_pdl(gather_packed<float, double>, (unsigned)gblocks, 256, 0, s, (const float*)x, (const float*)y, (const float*)z,
                                                               n, ax, (const dnode4*)m->efield, (float*)ex,
                                                               (float*)ey, (float*)ez, m->oob, e);
    }
    SC_LAUNCH_CHECK("gather_packed");
    m->launches += 1;
    return SC_OK;
}

}  // namespace sc
