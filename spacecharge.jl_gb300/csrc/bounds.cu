// extrema(particles_x/y/z) for the particle-bounds Mesh3D constructor
// (src/mesh.jl:120-122): one device reduction, then a 48-byte copy to the
// host (CUDA.jl's `extrema` on CuArrays does the same round trip).
#include <atomic>
#include <chrono>
#include <mutex>

#include "cells.cuh"
#include "sc_internal.cuh"

namespace sc {

// FP64 min/max run on the slow FP64 pipe (1/64 of the FP32 rate here): the
// reduction compares order keys instead, 64-bit integers that sort as the
// doubles do (-0 just below +0).  A NaN (either sign) lands beyond +-inf, so
// any NaN makes the maximum or the minimum non-finite, which the host check
// rejects, as the explicit NaN flag of an FP64 reduction would.
__device__ __forceinline__ unsigned long long order_key(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_order_key(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    return __longlong_as_double((long long)b);
}
__device__ __forceinline__ double widen(double v) { return v; }
__device__ __forceinline__ double widen(float v) { return f32_to_f64(v); }

template <typename P>
__global__ void __launch_bounds__(256) minmax_partials(const P* __restrict__ x, const P* __restrict__ y,
                                                       const P* __restrict__ z, int64_t n,
                                                       unsigned long long* __restrict__ partials) {
    unsigned long long mn[3] = {~0ull, ~0ull, ~0ull};
    unsigned long long mx[3] = {0ull, 0ull, 0ull};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    // four elements per coordinate in flight per thread: the loop is bound by
    // load latency, not by the integer compares
    for (; i + 3 * stride < n; i += 4 * stride) {
        P v[3][4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v[0][u] = __ldg(x + i + u * stride);
            v[1][u] = __ldg(y + i + u * stride);
            v[2][u] = __ldg(z + i + u * stride);
        }
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const unsigned long long k = order_key(widen(v[d][u]));
                mn[d] = min(mn[d], k);
                mx[d] = max(mx[d], k);
            }
    }
    for (; i < n; i += stride) {
        const unsigned long long k[3] = {order_key(widen(x[i])), order_key(widen(y[i])), order_key(widen(z[i]))};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            mn[d] = min(mn[d], k[d]);
            mx[d] = max(mx[d], k[d]);
        }
    }
    __shared__ unsigned long long red[6][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = min(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = max(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
        if (lane == 0) {
            red[d][warp] = mn[d];
            red[3 + d][warp] = mx[d];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        unsigned long long r = red[k][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = k < 3 ? min(r, red[k][w]) : max(r, red[k][w]);
        partials[blockIdx.x * 6 + k] = r;
    }
}

// One warp per extremum (6 warps): each lane reduces a stride of the block
// partials, then the warp reduces its lanes.
// out[6], read as an unsigned 64-bit word, is set to `seq` once the six
// extrema are visible to the host.
__global__ void __launch_bounds__(192) minmax_final(const unsigned long long* __restrict__ partials, int nblocks,
                                                    double* __restrict__ out, unsigned long long seq) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long r = k < 3 ? ~0ull : 0ull;
    for (int b = lane; b < nblocks; b += 32) r = k < 3 ? min(r, partials[b * 6 + k]) : max(r, partials[b * 6 + k]);
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, r, o);
        r = k < 3 ? min(r, v) : max(r, v);
    }
    if (lane == 0) {
        out[k] = from_order_key(r);
        __threadfence_system();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence_system();
        *reinterpret_cast<volatile unsigned long long*>(out + 6) = seq;
    }
}

int bounds_reduce(const void* x, const void* y, const void* z, int64_t n, int dtype, double mins[3],
                  double maxs[3], cudaStream_t s) {
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    // The partials buffer is per device and the call synchronises, so
    // concurrent callers are serialised here.
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    int blocks = (int)((n + 255) / 256);
    if (blocks > ctx->partial_blocks) blocks = ctx->partial_blocks;
    if (blocks < 1) blocks = 1;
    if (dtype == SC_F64)
        minmax_partials<double><<<blocks, 256, 0, s>>>((const double*)x, (const double*)y, (const double*)z, n,
                                                      reinterpret_cast<unsigned long long*>(ctx->partials));
    else
        minmax_partials<float><<<blocks, 256, 0, s>>>((const float*)x, (const float*)y, (const float*)z, n,
                                                     reinterpret_cast<unsigned long long*>(ctx->partials));
    SC_LAUNCH_CHECK("minmax_partials");
    // The final kernel writes the extrema straight into page-locked host
    // memory, then a sequence number after them.  The host spins on that
    // word for up to 20 ms (it returns as soon as the kernel has written it,
    // without the latency of a stream synchronisation), and otherwise
    // synchronises the stream, which also reports any error.
    const unsigned long long seq = ++ctx->ext_seq;
    minmax_final<<<1, 192, 0, s>>>(reinterpret_cast<const unsigned long long*>(ctx->partials), blocks,
                                   ctx->ext_dev, seq);
    SC_LAUNCH_CHECK("minmax_final");
    const volatile unsigned long long* flag = reinterpret_cast<volatile unsigned long long*>(ctx->ext_host + 6);
    const auto t0 = std::chrono::steady_clock::now();
    while (*flag != seq && std::chrono::steady_clock::now() - t0 < std::chrono::milliseconds(20)) {
    }
    std::atomic_thread_fence(std::memory_order_acquire);
    if (*flag != seq) SC_CUDA(cudaStreamSynchronize(s));
    if (*flag != seq) return fail(SC_ERR_CUDA, "bounds reduction: extrema not written");
    const volatile double* h = ctx->ext_host;
    for (int d = 0; d < 3; ++d) {
        mins[d] = h[d];
        maxs[d] = h[3 + d];
    }
    return SC_OK;
}

}  // namespace sc
