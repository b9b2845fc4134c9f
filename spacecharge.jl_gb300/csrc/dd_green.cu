// FP64 meshes in double-FP32 mode: the transform of the free-space Green
// function (the paired k4_green_xy and k4_green_col kernels of pipeline2.cuh
// with dreal values), in a translation unit of its own with only the
// instantiations the double-FP32 build uses.
#include "pipeline2.cuh"

namespace sc {

bool dd_green_applies(int logLx, int logLy, int logLz, int nx, int ny, int nz) {
    return logLx == logLy && (logLx == 6 || logLx == 7) && logLz >= 6 && logLz <= 8 && 2 * nx == (1 << logLx) &&
           2 * ny == (1 << logLy) && 2 * nz == (1 << logLz);
}

// The x+y pass as launch_green_xy_field runs it for these lengths (L = 64:
// 256 threads with the slice staged; L = 128: 256 threads, not staged), then
// the z pass as launch_green_z_field (nh = L/2).
bool launch_dd_green(int logLxy, int logLz, dreal* G, dreal* T2, dreal* out, int nx, int ny, int nz, int Hx,
                     int64_t gcs, int64_t t2cs, double gamma, const ddc* tw, cudaStream_t s, int solo) {
    const int Hy = (1 << logLxy) / 2 + 1, Hz = (1 << logLz) / 2 + 1;
    const int64_t plane = (int64_t)Hx * Hy;
    const size_t planes = 2 * sizeof(dreal) * (size_t)ny * Hx;
    const size_t slice = 2 * sizeof(dreal) * (size_t)nx * ny + 16;
    const int g16 = ((uintptr_t)G % 16 == 0 && (sizeof(dreal) * (size_t)nx * ny) % 16 == 0 &&
                     (sizeof(dreal) * (size_t)gcs) % 16 == 0) ? 1 : 0;
    const dim3 gxy(nz, solo ? 1 : 2);
    if (logLxy == 6) {
        constexpr int LL = 64;
        const size_t sm = sizeof(ddc) * (256 / F2<LL>::NT) * F2<LL>::S + planes + slice;
        if (sm > 100 * 1024 || set_smem(k4_green_xy<LL, dreal, 256, true, true>, sm) != SC_OK) return false;
        launch_pdl(k4_green_xy<LL, dreal, 256, true, true>, gxy, 256, sm, s, G, T2, nx, ny, Hx, gcs, t2cs, GreenNear{},
                   g16, solo, tw);
    } else if (logLxy == 7) {
        constexpr int LL = 128;
        const size_t sm = sizeof(ddc) * (256 / F2<LL>::NT) * F2<LL>::S + planes;
        if (sm > 100 * 1024 || set_smem(k4_green_xy<LL, dreal, 256, false, true>, sm) != SC_OK) return false;
        launch_pdl(k4_green_xy<LL, dreal, 256, false, true>, gxy, 256, sm, s, G, T2, nx, ny, Hx, gcs, t2cs,
                   GreenNear{}, g16, solo, tw);
    } else {
        return false;
    }
    const dreal s2(exp2(rint(log2(gamma > 1.0 ? gamma : 1.0))));  // a power of two: exact scaling
    const dim3 gz((unsigned)((plane + 2 * kColW - 1) / (2 * kColW)), solo ? 1 : 2);
#define SC_KDG(LL)                                                                                          \
    {                                                                                                       \
        const size_t sm = sizeof(ddc) * kColW * F2<LL>::S;                                                  \
        if (set_smem(k4_green_col<LL, dreal, true>, sm) != SC_OK) return false;                             \
        launch_pdl(k4_green_col<LL, dreal, true>, gz, kColW * F2<LL>::NT, sm, s, (const dreal*)T2, out,     \
                   (int)plane, nz, plane, t2cs, plane, plane * Hz, s2, solo, tw);                           \
    }
    switch (logLz) {
        case 6: SC_KDG(64); break;
        case 7: SC_KDG(128); break;
        case 8: SC_KDG(256); break;
        default: return false;
    }
#undef SC_KDG
    return true;
}

}  // namespace sc
