// The plain FP64 GPU path: SpaceCharge.jl's solve! restated in CUDA
// (src/solvers/free_space.jl:14-101, src/green_functions.jl:41-112) with the
// same schedule the reference runs through CUDA.jl: zero-pad rho into a
// complex 2nx x 2ny x 2nz array, one forward complex FFT, then per component
// an IGF point evaluation + 8-point difference, a forward FFT of it, the
// spectral product, an inverse FFT and the window extraction scaled by FPEI.
// 7 complex-to-complex cuFFT Z2Z transforms per solve (14 with the cathode),
// all in FP64.  It is the FP64 parity anchor and the baseline that the
// hand-written mixed-precision pipeline is measured against.
#include "sc_internal.cuh"

namespace sc {

// src/green_functions.jl:35-38
__device__ __forceinline__ double field_green(double x, double y, double z) {
    const double r = sqrt(x * x + y * y + z * z);
    return x * atan((y * z) / (r * x)) - z * log(r + y) + y * log((r - z) / (r + z)) / 2;
}

// src/green_functions.jl:13-22 (the reference defines it and never calls it):
// the antiderivative of 1/r, zero at r = 0.
__device__ __forceinline__ double potential_green(double x, double y, double z) { return potential_green_n(x, y, z); }

// green_functions.jl:69-101: F * factor at every point of the doubled grid.
// icomp 4 is the scalar potential: potential_green with the transverse
// factor gamma/(dx dy dz), which gives the lab-frame potential gamma*phi'.
__global__ void __launch_bounds__(256) plain_green_point(double2* __restrict__ g, int isize, int jsize, int ksize,
                                                         double dx, double dy, double dz_lab, double gamma,
                                                         int icomp, double offx, double offy, double offz) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)isize * jsize * ksize;
    if (t >= total) return;
    const int i = (int)(t % isize);
    const int j = (int)((t / isize) % jsize);
    const int k = (int)(t / ((int64_t)isize * jsize));
    const double dz = dz_lab * gamma;  // :73
    const double factor = (icomp == 1 || icomp == 2 || icomp == 4) ? gamma / (dx * dy * dz)  // :76-80
                                                                   : 1.0 / (dx * dy * dz);
    const double umin = (double)(1 - isize) * dx / 2 + offx;  // :82-84
    const double vmin = (double)(1 - jsize) * dy / 2 + offy;
    const double wmin = (double)(1 - ksize) * dz / 2 + offz * gamma;
    const double u = (double)i * dx + umin;  // :86-88
    const double v = (double)j * dy + vmin;
    const double w = (double)k * dz + wmin;
    double val;
    if (icomp == 1)
        val = field_green(u, v, w) * factor;
    else if (icomp == 2)
        val = field_green(v, w, u) * factor;
    else if (icomp == 3)
        val = field_green(w, u, v) * factor;
    else
        val = potential_green(u, v, w) * factor;
    g[t] = make_double2(val, 0.0);
}

// green_functions.jl:103-112 fused with the copy-back of :64-66: the output
// holds the 8-point difference below the last plane of each axis and the
// raw point values on it, exactly the array the reference then transforms.
__global__ void __launch_bounds__(256) plain_green_diff(const double2* __restrict__ f, double2* __restrict__ out,
                                                        int isize, int jsize, int ksize) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)isize * jsize * ksize;
    if (t >= total) return;
    const int i = (int)(t % isize);
    const int j = (int)((t / isize) % jsize);
    const int k = (int)(t / ((int64_t)isize * jsize));
    if (i == isize - 1 || j == jsize - 1 || k == ksize - 1) {
        out[t] = f[t];
        return;
    }
    const int64_t sj = isize, sk = (int64_t)isize * jsize;
    auto F = [&](int a, int b, int c) { return f[t + a + b * sj + c * sk].x; };
    const double v = F(1, 1, 1) - F(0, 1, 1) - F(1, 0, 1) - F(1, 1, 0) - F(0, 0, 0) + F(0, 0, 1) + F(0, 1, 0) +
                     F(1, 0, 0);
    out[t] = make_double2(v, 0.0);
}

// free_space.jl:68-69 (and :34 for the image: -rho[:, :, end:-1:1]); rho of
// the mesh type (the potential solve pads FP32 meshes' rho too)
template <typename T>
__global__ void __launch_bounds__(256) plain_pad(const T* __restrict__ rho, double2* __restrict__ c, int nx,
                                                 int ny, int nz, int image) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)8 * nx * ny * nz;
    if (t >= total) return;
    const int i = (int)(t % (2 * nx));
    const int j = (int)((t / (2 * nx)) % (2 * ny));
    const int k = (int)(t / ((int64_t)4 * nx * ny));
    double v = 0.0;
    if (i < nx && j < ny && k < nz) {
        const int ks = image ? nz - 1 - k : k;
        v = (double)rho[i + (int64_t)nx * (j + (int64_t)ny * ks)];
        if (image) v = -v;
    }
    c[t] = make_double2(v, 0.0);
}

// free_space.jl:92: temp = crho .* cgrn
__global__ void __launch_bounds__(256) plain_mul(const double2* __restrict__ a, double2* __restrict__ b,
                                                 int64_t total) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    const double2 x = a[t], y = b[t];
    b[t] = make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
}

// free_space.jl:98-99 (ifft normalisation 1/(8N) folded in first, as the
// normalised inverse plan produces it), with `accumulate` for the image
// superposition of :45.
__global__ void __launch_bounds__(256) plain_extract(const double2* __restrict__ c, double* __restrict__ ef,
                                                     int nx, int ny, int nz, int comp, double inv_total,
                                                     int accumulate) {
    const int64_t N = (int64_t)nx * ny * nz;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= N) return;
    const int i = (int)(t % nx);
    const int j = (int)((t / nx) % ny);
    const int k = (int)(t / ((int64_t)nx * ny));
    const int64_t src = (i + nx - 1) + (int64_t)(2 * nx) * ((j + ny - 1) + (int64_t)(2 * ny) * (k + nz - 1));
    const double v = kFpei * (c[src].x * inv_total);
    double* o = ef + comp * N + t;
    *o = accumulate ? *o + v : v;
}

static int plain_workspace(sc_mesh* m, cudaStream_t s) {
    PlainWork& w = m->pw;
    if (w.plan_ok) return SC_OK;
    const size_t total = (size_t)8 * m->N;
    if (!w.crho) SC_CUDA(dev_alloc(&w.crho, sizeof(double2) * total));
    if (!w.cgrn) SC_CUDA(dev_alloc(&w.cgrn, sizeof(double2) * total));
    if (!w.tmp) SC_CUDA(dev_alloc(&w.tmp, sizeof(double2) * total));
    // cuFFT dims are slowest-first: (2nz, 2ny, 2nx) for x-fastest storage.
    cufftResult r = cufftPlan3d(&w.plan, 2 * m->n[2], 2 * m->n[1], 2 * m->n[0], CUFFT_Z2Z);
    if (r != CUFFT_SUCCESS) return fail(SC_ERR_CUDA, "cufftPlan3d failed (%d)", (int)r);
    w.plan_ok = true;
    (void)s;
    return SC_OK;
}

static int fft(sc_mesh* m, double2* data, int dir, cudaStream_t s) {
    cufftResult r = cufftSetStream(m->pw.plan, s);
    if (r == CUFFT_SUCCESS) r = cufftExecZ2Z(m->pw.plan, (cufftDoubleComplex*)data, (cufftDoubleComplex*)data, dir);
    if (r != CUFFT_SUCCESS) return fail(SC_ERR_CUDA, "cufftExecZ2Z failed (%d)", (int)r);
    return SC_OK;
}

// free_space.jl:56-101 for one offset; `image` selects the flipped,
// negated charge of :34 and accumulation into efield (:45).
static int plain_solve_freespace(sc_mesh* m, double offz, int image, cudaStream_t s) {
    PlainWork& w = m->pw;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int64_t total = (int64_t)8 * m->N;
    const int64_t gb = (total + 255) / 256;
    StageTimer& tm = m->timer;
    StageScope st(tm, SC_STAGE_PLAIN_FFT, s);
    plain_pad<double><<<gb, 256, 0, s>>>((const double*)m->rho, w.crho, nx, ny, nz, image);
    SC_LAUNCH_CHECK("plain_pad");
    SC_TRY(fft(m, w.crho, CUFFT_FORWARD, s));
    m->launches += 2 + 3 * 6;
    for (int comp = 1; comp <= 3; ++comp) {
        if (tm.enabled) tm.begin(SC_STAGE_GREEN, s);
        plain_green_point<<<gb, 256, 0, s>>>(w.cgrn, 2 * nx, 2 * ny, 2 * nz, m->delta[0], m->delta[1],
                                             m->delta[2], m->gamma, comp, 0.0, 0.0, offz);
        SC_LAUNCH_CHECK("plain_green_point");
        plain_green_diff<<<gb, 256, 0, s>>>(w.cgrn, w.tmp, 2 * nx, 2 * ny, 2 * nz);
        SC_LAUNCH_CHECK("plain_green_diff");
        if (tm.enabled) tm.begin(SC_STAGE_PLAIN_FFT, s);
        SC_TRY(fft(m, w.tmp, CUFFT_FORWARD, s));
        plain_mul<<<gb, 256, 0, s>>>(w.crho, w.tmp, total);
        SC_LAUNCH_CHECK("plain_mul");
        SC_TRY(fft(m, w.tmp, CUFFT_INVERSE, s));
        plain_extract<<<(m->N + 255) / 256, 256, 0, s>>>(w.tmp, (double*)m->efield, nx, ny, nz, comp - 1,
                                                          1.0 / (double)total, image);
        SC_LAUNCH_CHECK("plain_extract");
    }
    return SC_OK;
}

// window extraction of the potential into a mesh-type array (free_space.jl:98-99)
template <typename T>
__global__ void __launch_bounds__(256) plain_extract_phi(const double2* __restrict__ c, T* __restrict__ phi, int nx,
                                                         int ny, int nz, double inv_total, int accumulate) {
    const int64_t N = (int64_t)nx * ny * nz;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= N) return;
    const int i = (int)(t % nx);
    const int j = (int)((t / nx) % ny);
    const int k = (int)(t / ((int64_t)nx * ny));
    const int64_t src = (i + nx - 1) + (int64_t)(2 * nx) * ((j + ny - 1) + (int64_t)(2 * ny) * (k + nz - 1));
    const double v = kFpei * (c[src].x * inv_total);
    phi[t] = accumulate ? (T)((double)phi[t] + v) : (T)v;
}

static int plain_potential_freespace(sc_mesh* m, double offz, int image, void* phi, cudaStream_t s) {
    PlainWork& w = m->pw;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int64_t total = (int64_t)8 * m->N;
    const int64_t gb = (total + 255) / 256;
    const bool f32 = m->precision == SC_PREC_MIXED;
    if (f32)
        plain_pad<float><<<gb, 256, 0, s>>>((const float*)m->rho, w.crho, nx, ny, nz, image);
    else
        plain_pad<double><<<gb, 256, 0, s>>>((const double*)m->rho, w.crho, nx, ny, nz, image);
    SC_LAUNCH_CHECK("plain_pad");
    SC_TRY(fft(m, w.crho, CUFFT_FORWARD, s));
    plain_green_point<<<gb, 256, 0, s>>>(w.cgrn, 2 * nx, 2 * ny, 2 * nz, m->delta[0], m->delta[1], m->delta[2],
                                         m->gamma, 4, 0.0, 0.0, offz);
    SC_LAUNCH_CHECK("plain_green_point");
    plain_green_diff<<<gb, 256, 0, s>>>(w.cgrn, w.tmp, 2 * nx, 2 * ny, 2 * nz);
    SC_LAUNCH_CHECK("plain_green_diff");
    SC_TRY(fft(m, w.tmp, CUFFT_FORWARD, s));
    plain_mul<<<gb, 256, 0, s>>>(w.crho, w.tmp, total);
    SC_LAUNCH_CHECK("plain_mul");
    SC_TRY(fft(m, w.tmp, CUFFT_INVERSE, s));
    const double inv = 1.0 / (double)total;
    if (f32)
        plain_extract_phi<float><<<(m->N + 255) / 256, 256, 0, s>>>(w.tmp, (float*)phi, nx, ny, nz, inv, image);
    else
        plain_extract_phi<double><<<(m->N + 255) / 256, 256, 0, s>>>(w.tmp, (double*)phi, nx, ny, nz, inv, image);
    SC_LAUNCH_CHECK("plain_extract_phi");
    m->launches += 6;
    return SC_OK;
}

// Scalar potential from the mesh's rho: the field solve's schedule in FP64
// with cuFFT for every mesh precision (free_space.jl:14-101 with the
// potential Green function; the image as in :19-46).
int plain_potential(sc_mesh* m, int at_cathode, void* phi, cudaStream_t s) {
    SC_TRY(plain_workspace(m, s));
    SC_TRY(plain_potential_freespace(m, 0.0, 0, phi, s));
    if (at_cathode) {
        const double offz = 2 * m->lo[2] + (m->hi[2] - m->lo[2]);
        SC_TRY(plain_potential_freespace(m, offz, 1, phi, s));
    }
    return SC_OK;
}

int plain_solve(sc_mesh* m, int at_cathode, cudaStream_t s) {
    SC_TRY(plain_workspace(m, s));
    SC_TRY(plain_solve_freespace(m, 0.0, 0, s));
    if (at_cathode) {
        // free_space.jl:39: offset_z = 2*zmin + (zmax - zmin)
        const double offz = 2 * m->lo[2] + (m->hi[2] - m->lo[2]);
        SC_TRY(plain_solve_freespace(m, offz, 1, s));
    }
    return SC_OK;
}

int plain_release(sc_mesh* m) {
    PlainWork& w = m->pw;
    if (w.plan_ok) cufftDestroy(w.plan);
    cudaFree(w.crho);
    cudaFree(w.cgrn);
    cudaFree(w.tmp);
    w = PlainWork();
    return SC_OK;
}

}  // namespace sc
