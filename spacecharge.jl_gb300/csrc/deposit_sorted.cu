// Sort-then-deposit CIC scatter (SC_DEPOSIT_SORTED / SC_DEPOSIT_DETERMINISTIC).
//
//   k_bin      : exact cell index (the reference's floor((x-min)/delta),
//                deposition.jl:39-46), a ticket within the cell from an
//                integer atomic on its counter, and the particle's
//                (fx, fy, fz, q) packed for the next passes;
//   scan       : exclusive prefix sum of the per-cell counts;
//   k_scatter  : particle -> its slot offset[cell] + ticket (cell order);
//   k_dep_seg  : one thread per sorted particle; lanes of a warp holding the
//                same cell reduce their 8 corner charges with a segmented
//                shuffle scan, and only the first lane of each segment issues
//                the 8 atomics.
//
// SC_DEPOSIT_DETERMINISTIC converts every corner charge to 64-bit fixed
// point before any addition (scale 2^k with k from an FP64 reduction of
// sum |q|, so the total stays below 2^62), adds with integer shuffles and
// integer atomics, and converts the grid back to the mesh type.  Integer
// addition is associative, so rho is bitwise the same for any atomic order,
// any launch configuration and any run; the rounding of each contribution to
// 2^-k (~1e-19 of the total charge) is below the FP32/FP64 rounding of rho.
#include <math.h>

#include "cells.cuh"
#include "sc_internal.cuh"

namespace sc {

Axes make_axes(const sc_mesh* m);

template <typename A>
struct SCell;
template <>
struct SCell<float> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, float& f) {
        return cell_df32(x, a, i, f);
    }
    template <typename P>
    __device__ __forceinline__ static float cvt(P v) { return f64_to_f32(v); }
};
template <>
struct SCell<double> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, double& f) {
        return cell_dp(x, a, i, f);
    }
    template <typename P>
    __device__ __forceinline__ static double cvt(P v) { return (double)v; }
};

template <typename A>
struct Pack4 {
    A fx, fy, fz, q;
};

template <typename P, typename A>
__global__ void __launch_bounds__(256) k_bin(const P* __restrict__ px, const P* __restrict__ py,
                                             const P* __restrict__ pz, const P* __restrict__ pq, int64_t n, Axes ax,
                                             int* __restrict__ key, int* __restrict__ ticket,
                                             Pack4<A>* __restrict__ pdat, int* __restrict__ count,
                                             unsigned long long* __restrict__ oob) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    int ix, iy, iz;
    Pack4<A> d;
    const bool ok = SCell<A>::run(px[p], ax.a[0], ix, d.fx) & SCell<A>::run(py[p], ax.a[1], iy, d.fy) &
                    SCell<A>::run(pz[p], ax.a[2], iz, d.fz);
    d.q = SCell<A>::cvt(pq[p]);
    if (!ok) {
        key[p] = -1;
        atomicAdd(oob, 1ull);
        return;
    }
    const int k = ix + ax.a[0].n * (iy + ax.a[1].n * iz);
    key[p] = k;
    ticket[p] = atomicAdd(count + k, 1);
    pdat[p] = d;
}

// ---------------------------------------------------------------- scan
// Three-phase exclusive scan of n ints (n <= 2^31): per-block scans, a scan
// of the block totals (one block, looping), and the add-back.
__device__ __forceinline__ int block_excl_scan(int v, int* sm, int& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sm[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int s = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sm[lane] = s;
    }
    __syncthreads();
    const int before = warp ? sm[warp - 1] : 0;
    total = sm[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(1024) k_scan_blocks(const int* __restrict__ in, int* __restrict__ out,
                                                      int* __restrict__ sums, int64_t n) {
    __shared__ int sm[32];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    int total;
    const int e = block_excl_scan(v, sm, total);
    if (i < n) out[i] = e;
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int* __restrict__ sums, int nb) {
    __shared__ int sm[32];
    int carry = 0;
    for (int base = 0; base < nb; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        int total;
        const int e = block_excl_scan(v, sm, total);
        if (i < nb) sums[i] = e + carry;
        carry += total;
    }
}

__global__ void __launch_bounds__(1024) k_scan_add(int* __restrict__ out, const int* __restrict__ sums, int64_t n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
}

template <typename A>
__global__ void __launch_bounds__(256) k_scatter(const int* __restrict__ key, const int* __restrict__ ticket,
                                                 const Pack4<A>* __restrict__ pdat, const int* __restrict__ offset,
                                                 int* __restrict__ skey, Pack4<A>* __restrict__ sdat, int64_t n) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int k = key[p];
    if (k < 0) return;
    const int pos = offset[k] + ticket[p];
    skey[pos] = k;
    sdat[pos] = pdat[p];
}

// Accumulator of the segmented sums: A for the plain sorted deposit,
// int64 fixed point for the deterministic one.
template <typename A, bool DET>
struct Acc;
template <typename A>
struct Acc<A, false> {
    using V = A;
    __device__ __forceinline__ static V from(A v, int) { return v; }
    __device__ __forceinline__ static void add(A* rho, long long*, int64_t i, V v) { atomicAdd(rho + i, v); }
};
// round(v * 2^k) to nearest, ties to even, for FP32 v with |v| 2^k < 2^62,
// with integer operations only (the FP64 route costs three instructions on
// the slow FP64 pipe per corner); equal to __double2ll_rn((double)v * 2^k).
__device__ __forceinline__ long long f32_to_fixed(float v, int k) {
    const unsigned u = __float_as_uint(v);
    const int be = (int)((u >> 23) & 0xFF);
    const long long m = be ? (long long)((u & 0x7FFFFFu) | 0x800000u) : (long long)(u & 0x7FFFFFu);
    const int sh = (be ? be : 1) - 150 + k;  // |v| 2^k = m 2^sh
    long long r;
    if (sh >= 0) {
        r = m << sh;  // sh < 38 since m 2^sh < 2^62
    } else if (sh > -40) {
        const int s = -sh;
        r = m >> s;
        const long long rem = m & ((1LL << s) - 1), half = 1LL << (s - 1);
        if (rem > half || (rem == half && (r & 1))) r += 1;
    } else {
        r = 0;  // m < 2^24: below half a unit
    }
    return (u >> 31) ? -r : r;
}

template <typename A>
struct Acc<A, true> {
    using V = long long;
    __device__ __forceinline__ static V from(A v, int k) { return __double2ll_rn(ldexp((double)v, k)); }
    __device__ __forceinline__ static void add(A*, long long* fx, int64_t i, V v) {
        atomicAdd(reinterpret_cast<unsigned long long*>(fx + i), (unsigned long long)v);
    }
};
template <>
__device__ __forceinline__ long long Acc<float, true>::from(float v, int k) { return f32_to_fixed(v, k); }

// fixed-point exponent: sum|q| * 2^k lies in [2^61, 2^62)
__device__ __forceinline__ int fixed_exponent(double qsum) { return qsum > 0 ? 61 - ilogb(qsum) : 0; }

template <typename A, bool DET>
__global__ void __launch_bounds__(256) k_dep_seg(const int* __restrict__ skey, const Pack4<A>* __restrict__ sdat,
                                                 const int* __restrict__ last_off, const int* __restrict__ last_cnt,
                                                 int nx, int ny, A* __restrict__ rho, long long* __restrict__ fixed,
                                                 const double* __restrict__ qsum) {
    using V = typename Acc<A, DET>::V;
    // particles skipped as out of range are not in the sorted array: it is
    // dense in [0, offset[N-1] + count[N-1])
    const int64_t nsorted = (int64_t)*last_off + *last_cnt;
    const int scale = DET ? fixed_exponent(*qsum) : 0;  // the fixed-point exponent k
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool in = i < nsorted;
    const int k = in ? skey[i] : -1 - lane;  // distinct dummy keys past the end
    V c[8];
    if (in) {
        const Pack4<A> d = sdat[i];
        const A wx0 = A(1) - d.fx, wy0 = A(1) - d.fy, wz0 = A(1) - d.fz;
        // deposition.jl:67-74 corner order and products
        c[0] = Acc<A, DET>::from(d.q * wx0 * wy0 * wz0, scale);
        c[1] = Acc<A, DET>::from(d.q * d.fx * wy0 * wz0, scale);
        c[2] = Acc<A, DET>::from(d.q * wx0 * d.fy * wz0, scale);
        c[3] = Acc<A, DET>::from(d.q * d.fx * d.fy * wz0, scale);
        c[4] = Acc<A, DET>::from(d.q * wx0 * wy0 * d.fz, scale);
        c[5] = Acc<A, DET>::from(d.q * d.fx * wy0 * d.fz, scale);
        c[6] = Acc<A, DET>::from(d.q * wx0 * d.fy * d.fz, scale);
        c[7] = Acc<A, DET>::from(d.q * d.fx * d.fy * d.fz, scale);
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) c[j] = V(0);
    }
    // segmented suffix sums: lanes of one cell are contiguous in cell order
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int ko = __shfl_down_sync(0xffffffffu, k, o);
        const bool same = (lane + o < 32) && ko == k;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const V v = __shfl_down_sync(0xffffffffu, c[j], o);
            if (same) c[j] += v;
        }
    }
    const int kp = __shfl_up_sync(0xffffffffu, k, 1);
    const bool head = in && (lane == 0 || kp != k);
    if (!head) return;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    const int64_t off[8] = {0, 1, sy, 1 + sy, sz, 1 + sz, sy + sz, 1 + sy + sz};
#pragma unroll
    for (int j = 0; j < 8; ++j) Acc<A, DET>::add(rho, fixed, k + off[j], c[j]);
}

// sum |q| in FP64 (the fixed-point scale of the deterministic deposit), in
// a fixed order: each block's partial to out[1 + block], then k_abs_final
// adds the partials in block order into out[0].  A floating-point atomic
// here would make the sum, and with it the exponent near a power of two,
// depend on the block order.
constexpr int kAbsBlocks = 2 * 152;

template <typename P>
__global__ void __launch_bounds__(256) k_abs_sum(const P* __restrict__ q, int64_t n, double* __restrict__ out) {
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += fabs((double)q[i]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double sm[8];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
        out[1 + blockIdx.x] = t;
    }
}

// One warp: lane l adds partials l, l + 32, ... in order, then a fixed
// butterfly combines the lanes, so the order never depends on scheduling.
__global__ void k_abs_final(double* __restrict__ out, int nblocks) {
    const int lane = threadIdx.x & 31;
    double t = 0;
    for (int b = lane; b < nblocks; b += 32) t += out[1 + b];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) out[0] = t;
}

// fixed point -> rho (adds to the existing rho, which `clear` has zeroed or
// the caller keeps for accumulation)
template <typename A>
__global__ void __launch_bounds__(256) k_fixed_to_rho(const long long* __restrict__ fixed, const double* __restrict__ qsum,
                                                      A* __restrict__ rho, int64_t N) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N) return;
    rho[i] += (A)ldexp((double)fixed[i], -fixed_exponent(*qsum));
}

struct SortWork {
    int64_t cap_n = 0, cap_N = 0;
    int *key = nullptr, *ticket = nullptr, *skey = nullptr;
    int *count = nullptr, *offset = nullptr, *sums = nullptr;
    void *pdat = nullptr, *sdat = nullptr;
    long long* fixed = nullptr;
    double* qsum = nullptr;
};

template <typename P, typename A>
static int sorted_t(sc_mesh* m, const P* x, const P* y, const P* z, const P* q, int64_t n, bool det, cudaStream_t s) {
    SortWork* w = reinterpret_cast<SortWork*>(m->sortwork);
    if (!w) {
        w = new SortWork();
        m->sortwork = w;
    }
    const int64_t N = m->N;
    // capacity 0 until every buffer of the set is in place: a failed
    // allocation leaves the set to be reallocated by the next call
    if (w->cap_n < n) {
        w->cap_n = 0;
        SC_CUDA(dev_realloc(&w->key, sizeof(int) * n));
        SC_CUDA(dev_realloc(&w->ticket, sizeof(int) * n));
        SC_CUDA(dev_realloc(&w->skey, sizeof(int) * n));
        SC_CUDA(dev_realloc(&w->pdat, sizeof(Pack4<double>) * n));
        SC_CUDA(dev_realloc(&w->sdat, sizeof(Pack4<double>) * n));
        w->cap_n = n;
    }
    if (w->cap_N < N) {
        const int64_t nb = (N + 1023) / 1024;
        w->cap_N = 0;
        SC_CUDA(dev_realloc(&w->count, sizeof(int) * N));
        SC_CUDA(dev_realloc(&w->offset, sizeof(int) * N));
        SC_CUDA(dev_realloc(&w->sums, sizeof(int) * nb));
        SC_CUDA(dev_realloc(&w->fixed, sizeof(long long) * N));
        SC_CUDA(dev_realloc(&w->qsum, sizeof(double) * (1 + kAbsBlocks)));
        w->cap_N = N;
    }
    const Axes ax = make_axes(m);
    const int64_t blocks = (n + 255) / 256;
    SC_CUDA(cudaMemsetAsync(w->count, 0, sizeof(int) * N, s));
    k_bin<P, A><<<blocks, 256, 0, s>>>(x, y, z, q, n, ax, w->key, w->ticket, (Pack4<A>*)w->pdat, w->count, m->oob);
    SC_LAUNCH_CHECK("k_bin");
    const int64_t nb = (N + 1023) / 1024;
    k_scan_blocks<<<nb, 1024, 0, s>>>(w->count, w->offset, w->sums, N);
    SC_LAUNCH_CHECK("k_scan_blocks");
    k_scan_sums<<<1, 1024, 0, s>>>(w->sums, (int)nb);
    SC_LAUNCH_CHECK("k_scan_sums");
    k_scan_add<<<nb, 1024, 0, s>>>(w->offset, w->sums, N);
    SC_LAUNCH_CHECK("k_scan_add");
    k_scatter<A><<<blocks, 256, 0, s>>>(w->key, w->ticket, (const Pack4<A>*)w->pdat, w->offset, w->skey,
                                        (Pack4<A>*)w->sdat, n);
    SC_LAUNCH_CHECK("k_scatter");
    const int* last_off = w->offset + N - 1;
    const int* last_cnt = w->count + N - 1;
    if (!det) {
        k_dep_seg<A, false><<<blocks, 256, 0, s>>>(w->skey, (const Pack4<A>*)w->sdat, last_off, last_cnt, m->n[0],
                                                    m->n[1], (A*)m->rho, nullptr, nullptr);
        SC_LAUNCH_CHECK("k_dep_seg");
        m->launches += 6;
        return SC_OK;
    }
    k_abs_sum<P><<<kAbsBlocks, 256, 0, s>>>(q, n, w->qsum);
    SC_LAUNCH_CHECK("k_abs_sum");
    k_abs_final<<<1, 32, 0, s>>>(w->qsum, kAbsBlocks);
    SC_LAUNCH_CHECK("k_abs_final");
    SC_CUDA(cudaMemsetAsync(w->fixed, 0, sizeof(long long) * N, s));
    k_dep_seg<A, true><<<blocks, 256, 0, s>>>(w->skey, (const Pack4<A>*)w->sdat, last_off, last_cnt, m->n[0], m->n[1],
                                               (A*)m->rho, w->fixed, w->qsum);
    SC_LAUNCH_CHECK("k_dep_seg");
    k_fixed_to_rho<A><<<(N + 255) / 256, 256, 0, s>>>(w->fixed, w->qsum, (A*)m->rho, N);
    SC_LAUNCH_CHECK("k_fixed_to_rho");
    m->launches += 9;
    return SC_OK;
}

int deposit_sorted_launch(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n,
                          int dtype, int mode, cudaStream_t s) {
    if (m->precision == SC_PREC_PLAIN64)
        return fail(SC_ERR_UNSUPPORTED, "sorted deposit modes need a hand-written pipeline mesh (fp64 or mixed)");
    if (n > (int64_t)0x7fffffff) return fail(SC_ERR_UNSUPPORTED, "sorted deposit supports at most 2^31-1 particles");
    const bool det = mode == SC_DEPOSIT_DETERMINISTIC;
    if (m->precision == SC_PREC_MIXED) {
        if (dtype == SC_F64)
            return sorted_t<double, float>(m, (const double*)x, (const double*)y, (const double*)z, (const double*)q,
                                           n, det, s);
        return sorted_t<float, float>(m, (const float*)x, (const float*)y, (const float*)z, (const float*)q, n, det,
                                      s);
    }
    if (dtype == SC_F64)
        return sorted_t<double, double>(m, (const double*)x, (const double*)y, (const double*)z, (const double*)q, n,
                                        det, s);
    return sorted_t<float, double>(m, (const float*)x, (const float*)y, (const float*)z, (const float*)q, n, det, s);
}

void sorted_release(sc_mesh* m) {
    SortWork* w = reinterpret_cast<SortWork*>(m->sortwork);
    if (!w) return;
    void* ptrs[] = {w->key, w->ticket, w->skey, w->count, w->offset, w->sums, w->pdat, w->sdat, w->fixed, w->qsum};
    for (void* p : ptrs) cudaFree(p);
    delete w;
    m->sortwork = nullptr;
}

}  // namespace sc
