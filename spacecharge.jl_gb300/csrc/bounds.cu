// extrema(particles_x/y/z) for the particle-bounds Mesh3D constructor
// (src/mesh.jl:147-149): one device reduction, then a 48-byte copy to the
// host (CUDA.jl's `extrema` on CuArrays does the same round trip).
#include <float.h>

#include <mutex>

#include "sc_internal.cuh"

namespace sc {

template <typename P>
__global__ void __launch_bounds__(256) minmax_partials(const P* __restrict__ x, const P* __restrict__ y,
                                                       const P* __restrict__ z, int64_t n,
                                                       double* __restrict__ partials) {
    double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX};
    double mx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    // NaN is carried as "not finite" by the host check; fmin/fmax skip it,
    // so flag it explicitly through +inf.
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v[3] = {(double)x[i], (double)y[i], (double)z[i]};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double a = v[d] == v[d] ? v[d] : __longlong_as_double(0x7ff0000000000000LL);
            mn[d] = fmin(mn[d], a);
            mx[d] = fmax(mx[d], a);
        }
    }
    __shared__ double red[6][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = fmin(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = fmax(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
        if (lane == 0) {
            red[d][warp] = mn[d];
            red[3 + d][warp] = mx[d];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        double r = red[k][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = k < 3 ? fmin(r, red[k][w]) : fmax(r, red[k][w]);
        partials[blockIdx.x * 6 + k] = r;
    }
}

__global__ void minmax_final(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
    const int k = threadIdx.x;
    if (k >= 6) return;
    double r = partials[k];
    for (int b = 1; b < nblocks; ++b) r = k < 3 ? fmin(r, partials[b * 6 + k]) : fmax(r, partials[b * 6 + k]);
    out[k] = r;
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
                                                      ctx->partials);
    else
        minmax_partials<float><<<blocks, 256, 0, s>>>((const float*)x, (const float*)y, (const float*)z, n,
                                                     ctx->partials);
    SC_LAUNCH_CHECK("minmax_partials");
    double* out = ctx->partials + 6 * ctx->partial_blocks;
    minmax_final<<<1, 32, 0, s>>>(ctx->partials, blocks, out);
    SC_LAUNCH_CHECK("minmax_final");
    double h[6];
    SC_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, s));
    SC_CUDA(cudaStreamSynchronize(s));
    for (int d = 0; d < 3; ++d) {
        mins[d] = h[d];
        maxs[d] = h[3 + d];
    }
    return SC_OK;
}

}  // namespace sc
