// Beside the kick (no counterpart in the reference): the bunch's magnetic
// field at the particles, and particle-layout adapters at the API boundary
// (array-of-structs records, FP32 positions relative to an FP64 point).
#include "sc_internal.cuh"

namespace sc {

// B = (beta / c) z x E for a bunch moving along +z: Bx = -beta Ey / c,
// By = beta Ex / c (Bz = 0).
template <typename P>
__global__ void __launch_bounds__(256) k_magnetic(const P* __restrict__ ex, const P* __restrict__ ey, int64_t n,
                                                  double k, P* __restrict__ bx, P* __restrict__ by) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = (double)ex[i], y = (double)ey[i];
    bx[i] = (P)(-k * y);
    by[i] = (P)(k * x);
}

template <typename P>
__global__ void __launch_bounds__(256) k_aos_to_soa(const P* __restrict__ aos, int64_t n, int stride, int ox,
                                                    int oy, int oz, int oq, P* __restrict__ x, P* __restrict__ y,
                                                    P* __restrict__ z, P* __restrict__ q) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const P* r = aos + i * stride;
    x[i] = r[ox];
    y[i] = r[oy];
    z[i] = r[oz];
    q[i] = r[oq];
}

template <typename P>
__global__ void __launch_bounds__(256) k_soa_to_aos(const P* __restrict__ ex, const P* __restrict__ ey,
                                                    const P* __restrict__ ez, int64_t n, int stride, int ox, int oy,
                                                    int oz, P* __restrict__ aos) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    P* r = aos + i * stride;
    r[ox] = ex[i];
    r[oy] = ey[i];
    r[oz] = ez[i];
}

// x = ref + r, one FP64 rounding (the FP32 offset converts exactly)
__global__ void __launch_bounds__(256) k_rel_to_abs(const float* __restrict__ rx, const float* __restrict__ ry,
                                                    const float* __restrict__ rz, int64_t n, double x0, double y0,
                                                    double z0, double* __restrict__ x, double* __restrict__ y,
                                                    double* __restrict__ z) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = x0 + (double)rx[i];
    y[i] = y0 + (double)ry[i];
    z[i] = z0 + (double)rz[i];
}

}  // namespace sc

using namespace sc;

static int check_layout(int64_t n, int stride, const int32_t* offs, int count) {
    if (n < 0) return fail(SC_ERR_INVALID, "negative particle count");
    if (!offs) return fail(SC_ERR_INVALID, "offsets are NULL");
    if (stride <= 0) return fail(SC_ERR_INVALID, "record stride must be positive");
    for (int k = 0; k < count; ++k)
        if (offs[k] < 0 || offs[k] >= stride)
            return fail(SC_ERR_INVALID, "field offset %d (%d) outside the record of %d elements", k, offs[k], stride);
    return SC_OK;
}

extern "C" {

int sc_magnetic_field(const sc_mesh* m, const void* ex, const void* ey, int64_t n, int dtype, void* bx, void* by,
                      void* stream) {
    if (!m) return fail(SC_ERR_INVALID, "mesh is NULL");
    if (dtype != SC_F32 && dtype != SC_F64) return fail(SC_ERR_INVALID, "dtype must be SC_F32 or SC_F64");
    if (n < 0) return fail(SC_ERR_INVALID, "negative particle count");
    if (n == 0) return SC_OK;
    if (!ex || !ey || !bx || !by) return fail(SC_ERR_INVALID, "field pointer is NULL");
    const double beta = sqrt(1.0 - 1.0 / (m->gamma * m->gamma));
    const double k = beta / kClight;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t blocks = (n + 255) / 256;
    if (dtype == SC_F64)
        k_magnetic<double><<<blocks, 256, 0, s>>>((const double*)ex, (const double*)ey, n, k, (double*)bx,
                                                 (double*)by);
    else
        k_magnetic<float><<<blocks, 256, 0, s>>>((const float*)ex, (const float*)ey, n, k, (float*)bx, (float*)by);
    SC_LAUNCH_CHECK("k_magnetic");
    return SC_OK;
}

int sc_aos_to_soa(const void* aos, int64_t n, int stride, const int32_t offs[4], int dtype, void* x, void* y,
                  void* z, void* q, void* stream) {
    SC_TRY(check_layout(n, stride, offs, 4));
    if (dtype != SC_F32 && dtype != SC_F64) return fail(SC_ERR_INVALID, "dtype must be SC_F32 or SC_F64");
    if (n == 0) return SC_OK;
    if (!aos || !x || !y || !z || !q) return fail(SC_ERR_INVALID, "particle pointer is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t blocks = (n + 255) / 256;
    if (dtype == SC_F64)
        k_aos_to_soa<double><<<blocks, 256, 0, s>>>((const double*)aos, n, stride, offs[0], offs[1], offs[2], offs[3],
                                                   (double*)x, (double*)y, (double*)z, (double*)q);
    else
        k_aos_to_soa<float><<<blocks, 256, 0, s>>>((const float*)aos, n, stride, offs[0], offs[1], offs[2], offs[3],
                                                  (float*)x, (float*)y, (float*)z, (float*)q);
    SC_LAUNCH_CHECK("k_aos_to_soa");
    return SC_OK;
}

int sc_soa_to_aos(const void* ex, const void* ey, const void* ez, int64_t n, int dtype, int stride,
                  const int32_t offs[3], void* aos, void* stream) {
    SC_TRY(check_layout(n, stride, offs, 3));
    if (dtype != SC_F32 && dtype != SC_F64) return fail(SC_ERR_INVALID, "dtype must be SC_F32 or SC_F64");
    if (n == 0) return SC_OK;
    if (!aos || !ex || !ey || !ez) return fail(SC_ERR_INVALID, "field pointer is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t blocks = (n + 255) / 256;
    if (dtype == SC_F64)
        k_soa_to_aos<double><<<blocks, 256, 0, s>>>((const double*)ex, (const double*)ey, (const double*)ez, n, stride,
                                                   offs[0], offs[1], offs[2], (double*)aos);
    else
        k_soa_to_aos<float><<<blocks, 256, 0, s>>>((const float*)ex, (const float*)ey, (const float*)ez, n, stride,
                                                  offs[0], offs[1], offs[2], (float*)aos);
    SC_LAUNCH_CHECK("k_soa_to_aos");
    return SC_OK;
}

int sc_relative_to_absolute(const float* rx, const float* ry, const float* rz, int64_t n, const double ref[3],
                            double* x, double* y, double* z, void* stream) {
    if (n < 0) return fail(SC_ERR_INVALID, "negative particle count");
    if (n == 0) return SC_OK;
    if (!rx || !ry || !rz || !ref || !x || !y || !z) return fail(SC_ERR_INVALID, "particle pointer is NULL");
    k_rel_to_abs<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(rx, ry, rz, n, ref[0], ref[1], ref[2], x, y, z);
    SC_LAUNCH_CHECK("k_rel_to_abs");
    return SC_OK;
}

}  // extern "C"
