// Cloud-in-Cell charge deposition, src/deposition.jl:28-158.
//
// deposit_plain: the reference's GPU kernel restated (one thread per
//   particle, FP64 IEEE-division cell index, 8 FP64 atomics with the
//   reference's weight products), plus a bounds check.
// deposit_atomic: the hand-written pipelines' unsorted deposit.  Same cell
//   index (bit-exact, see cells.cuh), weights in the mesh type, several
//   particles per thread with their loads in flight together, 8 atomics each.
// deposit_vector: mixed meshes; 2 vector atomics per particle into per-cell
//   corner slots, then a pass that sums each node's 8 slots.
#include "batch.cuh"
#include "cells.cuh"
#include "dd.cuh"
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

// Particles per thread of the atomic deposit: all their loads are issued
// before any arithmetic, so each thread keeps several requests in flight.
#ifndef SC_DEP_PT
#define SC_DEP_PT 4
#endif
constexpr int kDepPerThread = SC_DEP_PT;

// Body of one CTA: particles blk * 256 * kDepPerThread + ... of the bunch.
template <typename P, typename A>
__device__ __forceinline__ void deposit_atomic_body(const P* __restrict__ px, const P* __restrict__ py,
                                                    const P* __restrict__ pz, const P* __restrict__ pq, int64_t n,
                                                    const Axes& ax, A* __restrict__ rho,
                                                    unsigned long long* __restrict__ oob, int64_t blk) {
    const int64_t base = blk * (blockDim.x * kDepPerThread) + threadIdx.x;
    P x[kDepPerThread], y[kDepPerThread], z[kDepPerThread], qq[kDepPerThread];
#pragma unroll
    for (int k = 0; k < kDepPerThread; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        const bool in = p < n;
        x[k] = in ? __ldg(px + p) : P(0);
        y[k] = in ? __ldg(py + p) : P(0);
        z[k] = in ? __ldg(pz + p) : P(0);
        qq[k] = in ? __ldg(pq + p) : P(0);
    }
    const int nx = ax.a[0].n, ny = ax.a[1].n;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    unsigned skipped = 0;
#pragma unroll
    for (int k = 0; k < kDepPerThread; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        if (p >= n) break;
        int ix = 0, iy = 0, iz = 0;
        A fx = 0, fy = 0, fz = 0;
        const bool ok = CellCalc<A>::run(x[k], ax.a[0], ix, fx) & CellCalc<A>::run(y[k], ax.a[1], iy, fy) &
                        CellCalc<A>::run(z[k], ax.a[2], iz, fz);
        if (!ok) {
            ++skipped;
            continue;
        }
        const A q = CellCalc<A>::charge(qq[k]);
        const A wx0 = A(1) - fx, wy0 = A(1) - fy, wz0 = A(1) - fz;
        A* r = rho + (ix + sy * iy + sz * iz);
        // deposition.jl:67-74 corner order and products
        atomicAdd(r, q * wx0 * wy0 * wz0);
        atomicAdd(r + 1, q * fx * wy0 * wz0);
        atomicAdd(r + sy, q * wx0 * fy * wz0);
        atomicAdd(r + 1 + sy, q * fx * fy * wz0);
        atomicAdd(r + sz, q * wx0 * wy0 * fz);
        atomicAdd(r + 1 + sz, q * fx * wy0 * fz);
        atomicAdd(r + sy + sz, q * wx0 * fy * fz);
        atomicAdd(r + 1 + sy + sz, q * fx * fy * fz);
    }
    if (skipped) atomicAdd(oob, (unsigned long long)skipped);
}

// FP64 meshes in double-FP32 mode (sc_mesh_set_fp64_arithmetic): the
// atomic deposit with the cell fractions (cell_dd), the weights and the
// charge products in double-FP32 (dd.cuh), in the reference's order
// q*wx*wy*wz; each corner's charge is widened to FP64 (one FP64 addition)
// for its FP64 atomic add, which the L2 performs.
template <typename P>
__global__ void __launch_bounds__(256) deposit_dd(const P* __restrict__ px, const P* __restrict__ py,
                                                  const P* __restrict__ pz, const P* __restrict__ pq, int64_t n,
                                                  Axes ax, double* __restrict__ rho,
                                                  unsigned long long* __restrict__ oob) {
    const int64_t base = blockIdx.x * (int64_t)(blockDim.x * kDepPerThread) + threadIdx.x;
    P x[kDepPerThread], y[kDepPerThread], z[kDepPerThread], qq[kDepPerThread];
#pragma unroll
    for (int k = 0; k < kDepPerThread; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        const bool in = p < n;
        x[k] = in ? __ldg(px + p) : P(0);
        y[k] = in ? __ldg(py + p) : P(0);
        z[k] = in ? __ldg(pz + p) : P(0);
        qq[k] = in ? __ldg(pq + p) : P(0);
    }
    const int nx = ax.a[0].n, ny = ax.a[1].n;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    unsigned skipped = 0;
#pragma unroll
    for (int k = 0; k < kDepPerThread; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        if (p >= n) break;
        int ix = 0, iy = 0, iz = 0;
        float2 fx, fy, fz;
        const bool ok = cell_dd(x[k], ax.a[0], ix, fx.x, fx.y) & cell_dd(y[k], ax.a[1], iy, fy.x, fy.y) &
                        cell_dd(z[k], ax.a[2], iz, fz.x, fz.y);
        if (!ok) {
            ++skipped;
            continue;
        }
        float2 q;
        dd_split(qq[k], q.x, q.y);
        const float2 wx0 = ddr_one_minus(fx), wy0 = ddr_one_minus(fy), wz0 = ddr_one_minus(fz);
        const float2 qx0 = ddr_mul(q, wx0), qx1 = ddr_mul(q, fx);
        const float2 q00 = ddr_mul(qx0, wy0), q10 = ddr_mul(qx1, wy0), q01 = ddr_mul(qx0, fy), q11 = ddr_mul(qx1, fy);
        double* r = rho + (ix + sy * iy + sz * iz);
        // deposition.jl:67-74 corner order
        atomicAdd(r, ddr_to(ddr_mul(q00, wz0)));
        atomicAdd(r + 1, ddr_to(ddr_mul(q10, wz0)));
        atomicAdd(r + sy, ddr_to(ddr_mul(q01, wz0)));
        atomicAdd(r + 1 + sy, ddr_to(ddr_mul(q11, wz0)));
        atomicAdd(r + sz, ddr_to(ddr_mul(q00, fz)));
        atomicAdd(r + 1 + sz, ddr_to(ddr_mul(q10, fz)));
        atomicAdd(r + sy + sz, ddr_to(ddr_mul(q01, fz)));
        atomicAdd(r + 1 + sy + sz, ddr_to(ddr_mul(q11, fz)));
    }
    if (skipped) atomicAdd(oob, (unsigned long long)skipped);
}

template <typename P, typename A>
__global__ void __launch_bounds__(256) deposit_atomic(const P* __restrict__ px, const P* __restrict__ py,
                                                      const P* __restrict__ pz, const P* __restrict__ pq,
                                                      int64_t n, Axes ax, A* __restrict__ rho,
                                                      unsigned long long* __restrict__ oob) {
    deposit_atomic_body<P, A>(px, py, pz, pq, n, ax, rho, oob, blockIdx.x);
}

// ------------------------------------------------ vector (mixed meshes)
// The 8 CIC weights of a particle in cell c = (ix, iy, iz) go with two 16-byte
// vector atomics into corner[8c .. 8c+7]: the 4 nodes of the cell's lower z
// face, then the 4 of its upper face, x fastest (one 32-byte sector per cell).
// That is a quarter of the atomic operations of deposit_atomic.
// k_corner_sum then adds, for every node, the entries the (up to) 8 cells
// around it hold for it.  Cells with an index n-1 are never written and stay
// zero from the clear.
template <typename P>
__device__ __forceinline__ void deposit_vector_body(const P* __restrict__ px, const P* __restrict__ py,
                                                    const P* __restrict__ pz, const P* __restrict__ pq, int64_t n,
                                                    const Axes& ax, float4* __restrict__ corner,
                                                    unsigned long long* __restrict__ oob, int64_t blk) {
    const int64_t base = blk * (blockDim.x * kDepPerThread) + threadIdx.x;
    P x[kDepPerThread], y[kDepPerThread], z[kDepPerThread], qq[kDepPerThread];
#pragma unroll
    for (int k = 0; k < kDepPerThread; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        const bool in = p < n;
        x[k] = in ? __ldg(px + p) : P(0);
        y[k] = in ? __ldg(py + p) : P(0);
        z[k] = in ? __ldg(pz + p) : P(0);
        qq[k] = in ? __ldg(pq + p) : P(0);
    }
    const int nx = ax.a[0].n, ny = ax.a[1].n;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    unsigned skipped = 0;
#pragma unroll
    for (int k = 0; k < kDepPerThread; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        if (p >= n) break;
        int ix = 0, iy = 0, iz = 0;
        float fx = 0, fy = 0, fz = 0;
        const bool ok = cell_df32(x[k], ax.a[0], ix, fx) & cell_df32(y[k], ax.a[1], iy, fy) &
                        cell_df32(z[k], ax.a[2], iz, fz);
        if (!ok) {
            ++skipped;
            continue;
        }
        const float q = f64_to_f32(qq[k]);
        const float wx0 = 1.0f - fx, wy0 = 1.0f - fy, wz0 = 1.0f - fz;
        float4* c = corner + 2 * (ix + sy * iy + sz * iz);
        // deposition.jl:67-74 products
        atomicAdd(c, make_float4(q * wx0 * wy0 * wz0, q * fx * wy0 * wz0, q * wx0 * fy * wz0, q * fx * fy * wz0));
        atomicAdd(c + 1, make_float4(q * wx0 * wy0 * fz, q * fx * wy0 * fz, q * wx0 * fy * fz, q * fx * fy * fz));
    }
    if (skipped) atomicAdd(oob, (unsigned long long)skipped);
}

template <typename P>
__global__ void __launch_bounds__(256) deposit_vector(const P* __restrict__ px, const P* __restrict__ py,
                                                      const P* __restrict__ pz, const P* __restrict__ pq,
                                                      int64_t n, Axes ax, float4* __restrict__ corner,
                                                      unsigned long long* __restrict__ oob) {
    deposit_vector_body<P>(px, py, pz, pq, n, ax, corner, oob, blockIdx.x);
}

__device__ __forceinline__ void corner_sum_body(const float* __restrict__ corner, int nx, int ny, int64_t N,
                                                float* __restrict__ rho, int assign, int64_t blk) {
    const int64_t node = blk * blockDim.x + threadIdx.x;
    if (node >= N) return;
    int i, j, k;
    if (N <= 0x7FFFFFFF) {  // 32-bit index arithmetic (every mesh that fits in memory)
        const unsigned u = (unsigned)node, r = u / (unsigned)nx;
        i = (int)(u - r * (unsigned)nx);
        j = (int)(r % (unsigned)ny);
        k = (int)(r / (unsigned)ny);
    } else {
        const int64_t r = node / nx;
        i = (int)(node - r * nx);
        j = (int)(r % ny);
        k = (int)(r / ny);
    }
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
#pragma unroll
        for (int b = 0; b < 2; ++b) {
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                if (i >= a && j >= b && k >= c)
                    s += __ldg(corner + 8 * (node - a - b * sy - c * sz) + 4 * c + 2 * b + a);
            }
        }
    }
    if (assign)
        rho[node] = s;
    else
        rho[node] += s;
}

__global__ void __launch_bounds__(256) k_corner_sum(const float* __restrict__ corner, int nx, int ny, int64_t N,
                                                    float* __restrict__ rho, int assign) {
    pdl_wait();  // the corner slots come from the preceding deposit
    corner_sum_body(corner, nx, ny, N, rho, assign, blockIdx.x);
}

int corner_sum_launch(sc_mesh* m, const float* corner, float* out, cudaStream_t s, bool assign) {
    launch_pdl(k_corner_sum, (unsigned)((m->N + 255) / 256), 256, 0, s, corner, m->n[0], m->n[1], m->N, out,
               assign ? 1 : 0);
    SC_LAUNCH_CHECK("k_corner_sum");
    m->launches += 1;
    return SC_OK;
}

static int corner_clear(sc_mesh* m, cudaStream_t s) {
    const size_t bytes = sizeof(float) * 8 * (size_t)m->N;
    if (!m->corner) SC_CUDA(dev_alloc(&m->corner, bytes));
    // Clearing here rather than in the node sum: the clear writes whole
    // sectors, so the atomics then find every line in L2 instead of
    // fetching it from DRAM.
    SC_CUDA(cudaMemsetAsync(m->corner, 0, bytes, s));
    return SC_OK;
}

static int deposit_vector_add(sc_mesh* m, const Axes& ax, const void* x, const void* y, const void* z,
                              const void* q, int64_t n, int dtype, cudaStream_t s) {
    const int64_t blocks = (n + 256 * kDepPerThread - 1) / (256 * kDepPerThread);
    if (dtype == SC_F64)
        deposit_vector<double><<<blocks, 256, 0, s>>>((const double*)x, (const double*)y, (const double*)z,
                                                     (const double*)q, n, ax, (float4*)m->corner, m->oob);
    else
        deposit_vector<float><<<blocks, 256, 0, s>>>((const float*)x, (const float*)y, (const float*)z,
                                                    (const float*)q, n, ax, (float4*)m->corner, m->oob);
    SC_LAUNCH_CHECK("deposit_vector");
    m->launches += 1;
    return SC_OK;
}

static int deposit_vector_launch(sc_mesh* m, const Axes& ax, const void* x, const void* y, const void* z,
                                 const void* q, int64_t n, int dtype, cudaStream_t s, bool assign) {
    SC_TRY(corner_clear(m, s));
    SC_TRY(deposit_vector_add(m, ax, x, y, z, q, n, dtype, s));
    return corner_sum_launch(m, (const float*)m->corner, (float*)m->rho, s, assign);
}

bool deposit_assigns(const sc_mesh* m, int mode) {
    return mode == SC_DEPOSIT_VECTOR && m->precision == SC_PREC_MIXED;
}

// Deposit in chunks (sc_kick_host): the atomic and vector modes accumulate,
// so chunks can be deposited as their particles arrive.
bool deposit_chunkable(const sc_mesh* m, int mode) {
    return m->precision == SC_PREC_PLAIN64 || mode == SC_DEPOSIT_ATOMIC || mode == SC_DEPOSIT_VECTOR;
}

int deposit_chunk_begin(sc_mesh* m, int mode, cudaStream_t s) {
    if (deposit_assigns(m, mode)) return corner_clear(m, s);  // the node sum assigns rho
    SC_CUDA(cudaMemsetAsync(m->rho, 0, field_elem_bytes(m->precision) * m->N, s));
    return SC_OK;
}

int deposit_chunk_add(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
                      int mode, cudaStream_t s) {
    if (n == 0) return SC_OK;
    if (mode == SC_DEPOSIT_VECTOR && m->precision == SC_PREC_MIXED)
        return deposit_vector_add(m, make_axes(m), x, y, z, q, n, dtype, s);
    return deposit_launch(m, x, y, z, q, n, dtype, SC_DEPOSIT_ATOMIC, s);
}

int deposit_chunk_finish(sc_mesh* m, int mode, cudaStream_t s) {
    if (deposit_assigns(m, mode)) return corner_sum_launch(m, (const float*)m->corner, (float*)m->rho, s, true);
    return SC_OK;
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
                   int mode, cudaStream_t s, bool assign) {
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
        m->launches += 1;
        return SC_OK;
    }
    if (mode == SC_DEPOSIT_TILED) return deposit_tiled_launch(m, x, y, z, q, n, dtype, s);
    if (mode == SC_DEPOSIT_VECTOR && m->precision == SC_PREC_MIXED)
        return deposit_vector_launch(m, ax, x, y, z, q, n, dtype, s, assign);
    if (mode == SC_DEPOSIT_SORTED || mode == SC_DEPOSIT_DETERMINISTIC)
        return deposit_sorted_launch(m, x, y, z, q, n, dtype, mode, s);
    const int64_t ablocks = (n + 256 * kDepPerThread - 1) / (256 * kDepPerThread);
    if (m->precision == SC_PREC_MIXED) {
        if (dtype == SC_F64)
            deposit_atomic<double, float><<<ablocks, 256, 0, s>>>((const double*)x, (const double*)y,
                                                                (const double*)z, (const double*)q, n, ax,
                                                                (float*)m->rho, m->oob);
        else
            deposit_atomic<float, float><<<ablocks, 256, 0, s>>>((const float*)x, (const float*)y, (const float*)z,
                                                               (const float*)q, n, ax, (float*)m->rho, m->oob);
    } else if (m->df32) {
        if (dtype == SC_F64)
            deposit_dd<double><<<ablocks, 256, 0, s>>>((const double*)x, (const double*)y, (const double*)z,
                                                      (const double*)q, n, ax, (double*)m->rho, m->oob);
        else
            deposit_dd<float><<<ablocks, 256, 0, s>>>((const float*)x, (const float*)y, (const float*)z,
                                                     (const float*)q, n, ax, (double*)m->rho, m->oob);
    } else {
        if (dtype == SC_F64)
            deposit_atomic<double, double><<<ablocks, 256, 0, s>>>((const double*)x, (const double*)y,
                                                                 (const double*)z, (const double*)q, n, ax,
                                                                 (double*)m->rho, m->oob);
        else
            deposit_atomic<float, double><<<ablocks, 256, 0, s>>>((const float*)x, (const float*)y,
                                                                (const float*)z, (const float*)q, n, ax,
                                                                (double*)m->rho, m->oob);
    }
    SC_LAUNCH_CHECK("deposit_atomic");
    m->launches += 1;
    return SC_OK;
}


// ------------------------------------------------------- staged batch kick
// One launch per stage over a group of bunches (batch.cuh): each CTA finds
// its bunch and its CTA index within the bunch in the launch's CtaRef table
// and runs the single-mesh kernel's body on that bunch.
__global__ void __launch_bounds__(256) kb_clear(const ClearSeg* __restrict__ segs, const CtaRef* __restrict__ map) {
    const CtaRef r = map[blockIdx.x];
    const ClearSeg g = segs[r.item];
    const int64_t lo = (int64_t)r.local * kClearChunk;
    const int64_t hi = lo + kClearChunk < g.n ? lo + kClearChunk : g.n;
    pdl_wait();  // the previous call's readers of these buffers came before
    // the buffers come from cudaMalloc (256-byte aligned) and chunks are
    // multiples of 4 floats, so whole float4 groups start aligned
    const int64_t nv = (hi - lo) / 4;
    float4* p4 = reinterpret_cast<float4*>(g.p + lo);
    for (int64_t i = threadIdx.x; i < nv; i += blockDim.x) p4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t i = lo + 4 * nv + threadIdx.x; i < hi; i += blockDim.x) g.p[i] = 0.f;
}

template <typename P>
__global__ void __launch_bounds__(256) kb_deposit(const BunchDesc* __restrict__ tab, const CtaRef* __restrict__ map) {
    const CtaRef r = map[blockIdx.x];
    const BunchDesc& b = tab[r.item];
    const Axes ax = b.ax;
    pdl_wait();  // rho or the corner slots were cleared by the preceding launch
    if (b.corner)
        deposit_vector_body<P>((const P*)b.x, (const P*)b.y, (const P*)b.z, (const P*)b.q, b.n, ax, b.corner, b.oob,
                               r.local);
    else
        deposit_atomic_body<P, float>((const P*)b.x, (const P*)b.y, (const P*)b.z, (const P*)b.q, b.n, ax, b.rho,
                                      b.oob, r.local);
}

__global__ void __launch_bounds__(256) kb_corner_sum(const BunchDesc* __restrict__ tab,
                                                     const CtaRef* __restrict__ map) {
    const CtaRef r = map[blockIdx.x];
    const BunchDesc& b = tab[r.item];
    pdl_wait();
    corner_sum_body(reinterpret_cast<const float*>(b.corner), b.nx, b.ny, (int64_t)b.nx * b.ny * b.nz, b.rho, 1,
                    r.local);
}

int batch_clear_launch(const ClearSeg* segs, const CtaRef* map, int64_t ctas, cudaStream_t s) {
    if (ctas == 0) return SC_OK;
    launch_pdl(kb_clear, (unsigned)ctas, 256, 0, s, segs, map);
    SC_LAUNCH_CHECK("kb_clear");
    return SC_OK;
}

int batch_deposit_particles_per_cta() { return 256 * kDepPerThread; }

int batch_deposit_launch(const BunchDesc* tab, const CtaRef* map, int64_t ctas, int dtype, cudaStream_t s) {
    if (ctas == 0) return SC_OK;
    if (dtype == SC_F64)
        launch_pdl(kb_deposit<double>, (unsigned)ctas, 256, 0, s, tab, map);
    else
        launch_pdl(kb_deposit<float>, (unsigned)ctas, 256, 0, s, tab, map);
    SC_LAUNCH_CHECK("kb_deposit");
    return SC_OK;
}

int batch_corner_sum_launch(const BunchDesc* tab, const CtaRef* map, int64_t ctas, cudaStream_t s) {
    if (ctas == 0) return SC_OK;
    launch_pdl(kb_corner_sum, (unsigned)ctas, 256, 0, s, tab, map);
    SC_LAUNCH_CHECK("kb_corner_sum");
    return SC_OK;
}

int corner_alloc(sc_mesh* m) {
    if (!m->corner) SC_CUDA(dev_alloc(&m->corner, sizeof(float) * 8 * (size_t)m->N));
    return SC_OK;
}

}  // namespace sc
