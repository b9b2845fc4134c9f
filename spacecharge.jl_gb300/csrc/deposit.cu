// Cloud-in-Cell charge deposition, src/deposition.jl:28-158.
//
// deposit_plain: the reference's GPU kernel restated (one thread per
//   particle, FP64 IEEE-division cell index, 8 FP64 atomics with the
//   reference's weight products), plus a bounds check.
// deposit_atomic: the hand-written pipelines.  Same cell index (bit-exact,
//   see cells.cuh), weights in the mesh type, warp-aggregated atomics: lanes
//   of a warp that fall in the same cell add their 8 corner charges with
//   shuffles first, then one lane issues the 8 atomics.
#include "cells.cuh"
#include "sc_internal.cuh"

namespace sc {

Axes make_axes(const sc_mesh* m) {
    Axes ax;
    for (int d = 0; d < 3; ++d) ax.a[d] = make_axis(m->lo[d], m->delta[d], m->n[d]);
    return ax;
}

// ----------------------------------------------------------------- plain
template <typename P>
__global__ void __launch_bounds__(256) deposit_plain(const P* __restrict__ px, const P* __restrict__ py,
                                                     const P* __restrict__ pz, const P* __restrict__ pq,
                                                     int64_t n, Axes ax, double* __restrict__ rho,
                                                     unsigned long long* __restrict__ oob) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    int ix, iy, iz;
    double dx, dy, dz;
    const bool ok = cell_exact(px[p], ax.a[0], ix, dx) & cell_exact(py[p], ax.a[1], iy, dy) &
                    cell_exact(pz[p], ax.a[2], iz, dz);
    if (!ok) {
        atomicAdd(oob, 1ull);
        return;
    }
    // deposition.jl:54-61
    const double wx0 = 1 - dx, wx1 = dx, wy0 = 1 - dy, wy1 = dy, wz0 = 1 - dz, wz1 = dz;
    const double charge = (double)pq[p];
    const int nx = ax.a[0].n, ny = ax.a[1].n;
    const int64_t b = ix + (int64_t)nx * (iy + (int64_t)ny * iz);
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    // deposition.jl:67-74, same products and association
    atomicAdd(rho + b, charge * wx0 * wy0 * wz0);
    atomicAdd(rho + b + 1, charge * wx1 * wy0 * wz0);
    atomicAdd(rho + b + sy, charge * wx0 * wy1 * wz0);
    atomicAdd(rho + b + 1 + sy, charge * wx1 * wy1 * wz0);
    atomicAdd(rho + b + sz, charge * wx0 * wy0 * wz1);
    atomicAdd(rho + b + 1 + sz, charge * wx1 * wy0 * wz1);
    atomicAdd(rho + b + sy + sz, charge * wx0 * wy1 * wz1);
    atomicAdd(rho + b + 1 + sy + sz, charge * wx1 * wy1 * wz1);
}

// ------------------------------------------------- hand-written pipelines
template <typename A>
struct CellCalc;

template <>
struct CellCalc<float> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, float& f) {
        return cell_df32(x, a, i, f);
    }
    template <typename P>
    __device__ __forceinline__ static float charge(P q) { return f64_to_f32(q); }
};

template <>
struct CellCalc<double> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, double& f) {
        return cell_dp(x, a, i, f);
    }
    template <typename P>
    __device__ __forceinline__ static double charge(P q) { return (double)q; }
};

template <typename P, typename A>
__global__ void __launch_bounds__(256) deposit_atomic(const P* __restrict__ px, const P* __restrict__ py,
                                                      const P* __restrict__ pz, const P* __restrict__ pq,
                                                      int64_t n, Axes ax, A* __restrict__ rho,
                                                      unsigned long long* __restrict__ oob) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const unsigned full = 0xffffffffu;
    const unsigned active = __ballot_sync(full, p < n);
    if (p >= n) return;
    int ix = 0, iy = 0, iz = 0;
    A fx = 0, fy = 0, fz = 0;
    const bool ok = CellCalc<A>::run(px[p], ax.a[0], ix, fx) & CellCalc<A>::run(py[p], ax.a[1], iy, fy) &
                    CellCalc<A>::run(pz[p], ax.a[2], iz, fz);
    const int nx = ax.a[0].n, ny = ax.a[1].n;
    // key of the lower corner node; -1 for skipped particles
    const long long key = ok ? (long long)ix + (long long)nx * (iy + (long long)ny * iz) : -1ll;
    const unsigned okmask = __ballot_sync(active, ok);
    if (!ok) {
        if ((threadIdx.x & 31) == __ffs(active & ~okmask) - 1) atomicAdd(oob, (unsigned long long)__popc(active & ~okmask));
        return;
    }
    const A q = CellCalc<A>::charge(pq[p]);
    const A wx0 = A(1) - fx, wy0 = A(1) - fy, wz0 = A(1) - fz;
    A c[8];
    c[0] = q * wx0 * wy0 * wz0;
    c[1] = q * fx * wy0 * wz0;
    c[2] = q * wx0 * fy * wz0;
    c[3] = q * fx * fy * wz0;
    c[4] = q * wx0 * wy0 * fz;
    c[5] = q * fx * wy0 * fz;
    c[6] = q * wx0 * fy * fz;
    c[7] = q * fx * fy * fz;
    // Warp aggregation: lanes with the same cell reduce before the atomics.
    const unsigned peers = __match_any_sync(okmask, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    if (__popc(peers) > 1) {
        // sum over the peer group with a lane-ordered scan of the group
        unsigned rest = peers & ~(1u << leader);
        // each peer sends its contributions to the leader by a rotating shuffle
        // over the group members (group sizes are small in practice)
        A acc[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] = c[k];
        while (rest) {
            const int src = __ffs(rest) - 1;
            rest &= rest - 1;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const A v = __shfl_sync(peers, c[k], src);
                if (lane == leader) acc[k] += v;
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) c[k] = acc[k];
    }
    if (lane != leader) return;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    A* r = rho + key;
    atomicAdd(r, c[0]);
    atomicAdd(r + 1, c[1]);
    atomicAdd(r + sy, c[2]);
    atomicAdd(r + 1 + sy, c[3]);
    atomicAdd(r + sz, c[4]);
    atomicAdd(r + 1 + sz, c[5]);
    atomicAdd(r + sy + sz, c[6]);
    atomicAdd(r + 1 + sy + sz, c[7]);
}

// sc_cell_index: bins with the same arithmetic the mesh's deposit uses.
template <typename P, typename A>
__global__ void __launch_bounds__(256) cell_index_kernel(const P* __restrict__ px, const P* __restrict__ py,
                                                         const P* __restrict__ pz, int64_t n, Axes ax, int plain,
                                                         int32_t* __restrict__ idx, double* __restrict__ frac) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const P v[3] = {px[p], py[p], pz[p]};
    int i[3];
    double f[3];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (plain) {
            ok &= cell_exact(v[d], ax.a[d], i[d], f[d]);
        } else {
            A fa;
            ok &= CellCalc<A>::run(v[d], ax.a[d], i[d], fa);
            f[d] = (double)fa;
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        idx[3 * p + d] = ok ? i[d] : -1;
        frac[3 * p + d] = ok ? f[d] : 0.0;
    }
}

int cell_index_launch(sc_mesh* m, const void* x, const void* y, const void* z, int64_t n, int dtype,
                      int32_t* idx, double* frac, cudaStream_t s) {
    const Axes ax = make_axes(m);
    const int64_t blocks = (n + 255) / 256;
    const int plain = m->precision == SC_PREC_PLAIN64;
    if (m->precision == SC_PREC_MIXED) {
        if (dtype == SC_F64)
            cell_index_kernel<double, float><<<blocks, 256, 0, s>>>((const double*)x, (const double*)y,
                                                                   (const double*)z, n, ax, 0, idx, frac);
        else
            cell_index_kernel<float, float><<<blocks, 256, 0, s>>>((const float*)x, (const float*)y,
                                                                  (const float*)z, n, ax, 0, idx, frac);
    } else {
        if (dtype == SC_F64)
            cell_index_kernel<double, double><<<blocks, 256, 0, s>>>((const double*)x, (const double*)y,
                                                                    (const double*)z, n, ax, plain, idx, frac);
        else
            cell_index_kernel<float, double><<<blocks, 256, 0, s>>>((const float*)x, (const float*)y,
                                                                   (const float*)z, n, ax, plain, idx, frac);
    }
    SC_LAUNCH_CHECK("cell_index_kernel");
    return SC_OK;
}

int deposit_sorted_launch(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n,
                          int dtype, int mode, cudaStream_t s);

int deposit_launch(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
                   int mode, cudaStream_t s) {
    const Axes ax = make_axes(m);
    const int64_t blocks = (n + 255) / 256;
    if (m->precision == SC_PREC_PLAIN64) {
        if (dtype == SC_F64)
            deposit_plain<double><<<blocks, 256, 0, s>>>((const double*)x, (const double*)y, (const double*)z,
                                                        (const double*)q, n, ax, (double*)m->rho, m->oob);
        else
            deposit_plain<float><<<blocks, 256, 0, s>>>((const float*)x, (const float*)y, (const float*)z,
                                                       (const float*)q, n, ax, (double*)m->rho, m->oob);
        SC_LAUNCH_CHECK("deposit_plain");
        return SC_OK;
    }
    if (mode != SC_DEPOSIT_ATOMIC) return deposit_sorted_launch(m, x, y, z, q, n, dtype, mode, s);
    if (m->precision == SC_PREC_MIXED) {
        if (dtype == SC_F64)
            deposit_atomic<double, float><<<blocks, 256, 0, s>>>((const double*)x, (const double*)y,
                                                                (const double*)z, (const double*)q, n, ax,
                                                                (float*)m->rho, m->oob);
        else
            deposit_atomic<float, float><<<blocks, 256, 0, s>>>((const float*)x, (const float*)y, (const float*)z,
                                                               (const float*)q, n, ax, (float*)m->rho, m->oob);
    } else {
        if (dtype == SC_F64)
            deposit_atomic<double, double><<<blocks, 256, 0, s>>>((const double*)x, (const double*)y,
                                                                 (const double*)z, (const double*)q, n, ax,
                                                                 (double*)m->rho, m->oob);
        else
            deposit_atomic<float, double><<<blocks, 256, 0, s>>>((const float*)x, (const float*)y,
                                                                (const float*)z, (const float*)q, n, ax,
                                                                (double*)m->rho, m->oob);
    }
    SC_LAUNCH_CHECK("deposit_atomic");
    return SC_OK;
}

}  // namespace sc
