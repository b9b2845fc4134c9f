// Tracking steps of a bunch in its own field (sc_track; no counterpart in the
// reference, which stops at the kick).  Each step: optionally refit the mesh
// bounds to the particles (the particle constructor's arithmetic,
// mesh.jl:95-174), kick, B = (beta/c) z x E, and one relativistic Boris step
// (J. P. Boris 1970; Birdsall & Langdon section 15-4) of u = gamma*beta:
//   u- = u + a E,  a = qm dt / (2c)
//   t = qm dt / (2 gamma(u-)) B,  s = 2 t / (1 + |t|^2)
//   u' = u- + u- x t,  u+ = u- + u' x s,  u_new = u+ + a E
//   x += c dt u_new / gamma(u_new)
// FP64 meshes push in FP64 throughout.  Mixed meshes keep u and x in the
// particle type and form the increments (both half kicks with the rotation,
// and the drift) in FP32: each is small next to the value it is added to, so
// FP32 keeps it to ~1e-7 of itself, and one FP64 add per coordinate keeps a
// relativistic u exact to the step.  FP64 arithmetic, conversions included,
// runs at 1/64 of the FP32 rate on this GPU: the mixed push converts between
// FP64 and FP32 with integer operations (f64_to_f32, f32_to_f64) and issues
// only the two FP64 adds per coordinate that the FP64 state needs.
#include <algorithm>
#include <type_traits>

#include "cells.cuh"
#include "sc_internal.cuh"

namespace sc {

template <typename P>
__global__ void __launch_bounds__(256) k_boris64(P* __restrict__ x, P* __restrict__ y, P* __restrict__ z,
                                                 P* __restrict__ ux, P* __restrict__ uy, P* __restrict__ uz,
                                                 const P* __restrict__ ex, const P* __restrict__ ey,
                                                 const P* __restrict__ ez, int64_t n, double a, double qmdt2,
                                                 double kb, double cdt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double Ex = (double)ex[i], Ey = (double)ey[i], Ez = (double)ez[i];
    const double bx = -kb * Ey, by = kb * Ex;
    const double umx = (double)ux[i] + a * Ex, umy = (double)uy[i] + a * Ey, umz = (double)uz[i] + a * Ez;
    const double g = sqrt(1.0 + umx * umx + umy * umy + umz * umz);
    const double tb = qmdt2 / g;
    const double tx = tb * bx, ty = tb * by;
    const double upx = umx - umz * ty, upy = umy + umz * tx, upz = umz + (umx * ty - umy * tx);
    const double s = 2.0 / (1.0 + tx * tx + ty * ty);
    const double sx = s * tx, sy = s * ty;
    const double nx = umx - upz * sy + a * Ex, ny = umy + upz * sx + a * Ey, nz = umz + (upx * sy - upy * sx) + a * Ez;
    const double f = cdt / sqrt(1.0 + nx * nx + ny * ny + nz * nz);
    x[i] = (P)((double)x[i] + f * nx);
    y[i] = (P)((double)y[i] + f * ny);
    z[i] = (P)((double)z[i] + f * nz);
    ux[i] = (P)nx;
    uy[i] = (P)ny;
    uz[i] = (P)nz;
}

template <typename P>
__global__ void __launch_bounds__(256) k_boris_mixed(P* __restrict__ x, P* __restrict__ y, P* __restrict__ z,
                                                     P* __restrict__ ux, P* __restrict__ uy, P* __restrict__ uz,
                                                     const P* __restrict__ ex, const P* __restrict__ ey,
                                                     const P* __restrict__ ez, int64_t n, float a, float qmdt2,
                                                     float kb, float cdt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float Ex = f64_to_f32(ex[i]), Ey = f64_to_f32(ey[i]), Ez = f64_to_f32(ez[i]);
    const float bx = -kb * Ey, by = kb * Ex;
    const float hx = a * Ex, hy = a * Ey, hz = a * Ez;  // half electric kick
    const P ux0 = ux[i], uy0 = uy[i], uz0 = uz[i];
    const float wx = f64_to_f32(ux0), wy = f64_to_f32(uy0), wz = f64_to_f32(uz0);
    const float fx = wx + hx, fy = wy + hy, fz = wz + hz;  // u-
    const float tb = qmdt2 / sqrtf(1.0f + fx * fx + fy * fy + fz * fz);
    const float tx = tb * bx, ty = tb * by;
    const float px = fx - fz * ty, py = fy + fz * tx, pz = fz + (fx * ty - fy * tx);  // u'
    const float s = 2.0f / (1.0f + tx * tx + ty * ty);
    const float sx = s * tx, sy = s * ty;
    // u_new - u = 2 a E + (u' x s)
    const float dx = hx + (-pz * sy + hx), dy = hy + (pz * sx + hy), dz = hz + ((px * sy - py * sx) + hz);
    const float gx = wx + dx, gy = wy + dy, gz = wz + dz;  // u_new to FP32 rounding, for the drift
    const float f = cdt / sqrtf(1.0f + gx * gx + gy * gy + gz * gz);
    if (std::is_same<P, double>::value) {
        x[i] = (P)((double)x[i] + f32_to_f64(f * gx));
        y[i] = (P)((double)y[i] + f32_to_f64(f * gy));
        z[i] = (P)((double)z[i] + f32_to_f64(f * gz));
        ux[i] = (P)((double)ux0 + f32_to_f64(dx));
        uy[i] = (P)((double)uy0 + f32_to_f64(dy));
        uz[i] = (P)((double)uz0 + f32_to_f64(dz));
    } else {  // FP32 state: the FP32 add rounds as the FP64 add then FP32 store would
        x[i] = (P)((float)x[i] + f * gx);
        y[i] = (P)((float)y[i] + f * gy);
        z[i] = (P)((float)z[i] + f * gz);
        ux[i] = (P)((float)ux0 + dx);
        uy[i] = (P)((float)uy0 + dy);
        uz[i] = (P)((float)uz0 + dz);
    }
}

static int push_launch(sc_mesh* m, void* x, void* y, void* z, void* ux, void* uy, void* uz, const void* ex,
                       const void* ey, const void* ez, int64_t n, int dtype, double dt, double qm, cudaStream_t s) {
    const double beta = sqrt(1.0 - 1.0 / (m->gamma * m->gamma));
    const double a = qm * dt / (2.0 * kClight), qmdt2 = qm * dt / 2.0, kb = beta / kClight, cdt = kClight * dt;
    const int64_t blocks = (n + 255) / 256;
    const bool mixed = m->precision == SC_PREC_MIXED;
#define SC_PUSH(P)                                                                                                \
    if (mixed)                                                                                                    \
        k_boris_mixed<P><<<blocks, 256, 0, s>>>((P*)x, (P*)y, (P*)z, (P*)ux, (P*)uy, (P*)uz, (const P*)ex,        \
                                                (const P*)ey, (const P*)ez, n, (float)a, (float)qmdt2, (float)kb, \
                                                (float)cdt);                                                      \
    else                                                                                                          \
        k_boris64<P><<<blocks, 256, 0, s>>>((P*)x, (P*)y, (P*)z, (P*)ux, (P*)uy, (P*)uz, (const P*)ex,            \
                                            (const P*)ey, (const P*)ez, n, a, qmdt2, kb, cdt);
    if (dtype == SC_F64) {
        SC_PUSH(double)
    } else {
        SC_PUSH(float)
    }
#undef SC_PUSH
    SC_LAUNCH_CHECK("k_boris");
    m->launches += 1;
    return SC_OK;
}

}  // namespace sc

using namespace sc;

extern "C" {

int sc_track(sc_mesh* m, void* x, void* y, void* z, void* ux, void* uy, void* uz, const void* q, int64_t n,
             int dtype, double dt, double qm, int steps, int refit, int at_cathode, void* stream) {
    if (!m) return fail(SC_ERR_INVALID, "mesh is NULL");
    if (dtype != SC_F32 && dtype != SC_F64) return fail(SC_ERR_INVALID, "dtype must be SC_F32 or SC_F64");
    if (n < 0) return fail(SC_ERR_INVALID, "Particle coordinate and charge arrays must have the same length.");
    if (steps < 0) return fail(SC_ERR_INVALID, "steps must be non-negative");
    if (!(dt >= 0) || !isfinite(dt) || !isfinite(qm)) return fail(SC_ERR_INVALID, "dt and qm must be finite, dt >= 0");
    if (n == 0 || steps == 0) return SC_OK;
    if (!x || !y || !z || !ux || !uy || !uz || !q) return fail(SC_ERR_INVALID, "particle pointer is NULL");
    DeviceGuard g(m->device);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t elem = dtype == SC_F64 ? 8 : 4;
    if (m->track_cap < n || m->track_elem != elem) {
        cudaFree(m->trackE);
        m->trackE = nullptr;
        m->track_cap = 0;
        SC_CUDA(dev_alloc(&m->trackE, 3 * elem * (size_t)n));
        m->track_cap = n;
        m->track_elem = elem;
    }
    char* e = (char*)m->trackE;
    void* ex = e;
    void* ey = e + elem * (size_t)n;
    void* ez = e + 2 * elem * (size_t)n;
    for (int step = 0; step < steps; ++step) {
        if (refit) {
            // the particle constructor's bounds for the moved bunch (synchronises, as extrema does)
            double lo[3], hi[3], dl[3];
            SC_TRY(sc_auto_bounds(m->n, x, y, z, n, dtype, lo, hi, dl, stream));
            SC_TRY(mesh_set_geometry(m, lo, hi, dl));
            SC_TRY(kick_issue(m, x, y, z, q, n, dtype, at_cathode, ex, ey, ez, s));
        } else {
            SC_TRY(sc_kick(m, x, y, z, q, n, dtype, at_cathode, ex, ey, ez, stream));
        }
        SC_TRY(push_launch(m, x, y, z, ux, uy, uz, ex, ey, ez, n, dtype, dt, qm, s));
    }
    return SC_OK;
}

}  // extern "C"
