// Transform passes of the staged batch kick (batch.cuh): the forward x+y
// transform (one fused pass per plane, or an x pass and a y pass), the z
// pass with the Green multiply, and the fused inverse y+x pass, each as one
// launch over a group of bunches of one grid class (bunches whose transforms
// have the same lengths; their node counts may differ).  Each CTA looks up
// its bunch and its plane, row block or column tile in the launch's CtaRef
// table and runs the single-mesh kernel's body (pipeline2.cuh) there.
#include "batch.cuh"
#include "pipeline2.cuh"

namespace sc {

static_assert(kBatchZCols == kColW, "the batch plans z-pass and column tiles of kColW columns");

// CTA local index = z plane
template <int L>
__global__ void __launch_bounds__(256) kb_fwd_xy(const BunchDesc* __restrict__ tab, const CtaRef* __restrict__ map,
                                                 const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    const CtaRef r = map[blockIdx.x];
    const BunchDesc& b = tab[r.item];
    const int nx = b.nx, ny = b.ny, Hx = b.Hx;
    const float* rho = b.rho;
    float2* B = b.B;
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    const int z = r.local;
    fwd_xy_body<L>(rho + (int64_t)nx * ny * z, B + (int64_t)Hx * L * z, nx, ny, Hx, swt, smraw);
}

// Two-pass forward: x pass (CTA local index = row-pair block) ...
template <int L>
__global__ void __launch_bounds__(256) kb_fwd_x(const BunchDesc* __restrict__ tab, const CtaRef* __restrict__ map,
                                                const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    __shared__ float2 xb[(256 / F2<L>::NT) * F2<L>::S];
    const CtaRef r = map[blockIdx.x];
    const BunchDesc& b = tab[r.item];
    const int nx = b.nx, rows = b.ny * b.nz, Hx = b.Hx;
    const float* rho = b.rho;
    float2* A = b.A;
    stage_twiddles<L>(swt, tw);
    fwd_x_body<L>(rho, A, nx, rows, Hx, r.local, swt, xb);
}

// ... and y pass (CTA local index = tile of kColW of the Hx x nz columns of A)
template <int L>
__global__ void __launch_bounds__(kColW * F2<L>::NT, SC_COL_MINB) kb_fwd_y(const BunchDesc* __restrict__ tab,
                                                                           const CtaRef* __restrict__ map,
                                                                           const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    __shared__ float2 xb[kColW * F2<L>::S];
    const CtaRef r = map[blockIdx.x];
    const BunchDesc& b = tab[r.item];
    const int ny = b.ny, nz = b.nz, Hx = b.Hx;
    const float2* A = b.A;
    float2* B = b.B;
    stage_twiddles<L>(swt, tw);
    col_body<L, false>(A, B, Hx, nz, ny, L, 0, 0, 0, Hx, (int64_t)Hx * ny, 0, Hx, (int64_t)Hx * L, 0, r.local, 0,
                       swt, xb);
}

// CTA local index = column tile
template <int L>
__global__ void __launch_bounds__(kColW * F2<L>::NT, SC_ZPASS_MINB) kb_zpass(const BunchDesc* __restrict__ tab,
                                                                             const CtaRef* __restrict__ map,
                                                                             const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    const CtaRef r = map[blockIdx.x];
    const BunchDesc& b = tab[r.item];
    const GreenView gv = b.gv;
    const float2* B = b.B;
    float2* C = b.C;
    const int Hx = b.Hx, Ly = b.Ly, nz = b.nz;
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    if (2 * nz == L)
        zpass_body<L, true>(B, C, Hx, Ly, nz, gv, r.local, swt, smraw);
    else
        zpass_body<L, false>(B, C, Hx, Ly, nz, gv, r.local, swt, smraw);
}

// CTA local index = 3 * z + component
template <int L>
__global__ void __launch_bounds__(256) kb_inv_yx(const BunchDesc* __restrict__ tab, const CtaRef* __restrict__ map,
                                                 const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    const CtaRef r = map[blockIdx.x];
    const BunchDesc& b = tab[r.item];
    const int nx = b.nx, ny = b.ny, nz = b.nz, Hx = b.Hx;
    const float2* C = b.C;
    float* E4 = reinterpret_cast<float*>(b.efield);
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    const int z = r.local / 3, comp = r.local - 3 * (r.local / 3);
    const int64_t plane = (int64_t)Hx * L;
    float* o = E4 + comp + 4 * (int64_t)nx * ny * z;
    if (2 * nx == L && 2 * ny == L && 2 * (Hx - 1) == L)
        inv_yx_body<L, true>(C + (int64_t)comp * plane * nz + plane * z, o, nx, ny, Hx, swt, smraw);
    else
        inv_yx_body<L, false>(C + (int64_t)comp * plane * nz + plane * z, o, nx, ny, Hx, swt, smraw);
}

// Expands MACRO(L) for the transform length 2^logL; `fallback` otherwise.
#define SC_KB_SWITCH(logL, MACRO, fallback) \
    switch (logL) {                          \
        case 2: MACRO(4); break;             \
        case 3: MACRO(8); break;             \
        case 4: MACRO(16); break;            \
        case 5: MACRO(32); break;            \
        case 6: MACRO(64); break;            \
        case 7: MACRO(128); break;           \
        case 8: MACRO(256); break;           \
        default: fallback;                   \
    }

size_t batch_plane_smem(int logL, int64_t plane) {
    size_t ws = 0;
#define SC_KBW(LL) ws = (size_t)(256 / F2<LL>::NT) * F2<LL>::S;
    SC_KB_SWITCH(logL, SC_KBW, return (size_t)-1)
#undef SC_KBW
    return sizeof(float2) * (ws + (size_t)plane);
}

int64_t batch_fwd_x_ctas(int logL, int64_t rows) {
    int nt = 0;
#define SC_KBNT(LL) nt = F2<LL>::NT;
    SC_KB_SWITCH(logL, SC_KBNT, return 0)
#undef SC_KBNT
    const int64_t pairs = (rows + 1) / 2, P = 256 / nt;
    return (pairs + P - 1) / P;
}

int64_t batch_fwd_y_ctas(int64_t columns) { return (columns + kColW - 1) / kColW; }

static int length_fail(const char* what) { return fail(SC_ERR_UNSUPPORTED, "%s: transform length out of range", what); }

int batch_fwd_xy_launch(int logL, const BunchDesc* tab, const CtaRef* map, int64_t ctas, size_t smem_plane,
                        cudaStream_t s) {
    if (ctas == 0) return SC_OK;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const size_t smem = batch_plane_smem(logL, (int64_t)smem_plane);
#define SC_KBFXY(LL)                                                                                  \
    {                                                                                                 \
        SC_TRY(set_smem(kb_fwd_xy<LL>, smem));                                                        \
        launch_pdl(kb_fwd_xy<LL>, (unsigned)ctas, 256, smem, s, tab, map, (const float2*)ctx->tw32); \
    }
    SC_KB_SWITCH(logL, SC_KBFXY, return length_fail("kb_fwd_xy"))
#undef SC_KBFXY
    SC_LAUNCH_CHECK("kb_fwd_xy");
    return SC_OK;
}

int batch_fwd_x_launch(int logL, const BunchDesc* tab, const CtaRef* map, int64_t ctas, cudaStream_t s) {
    if (ctas == 0) return SC_OK;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
#define SC_KBFX(LL) launch_pdl(kb_fwd_x<LL>, (unsigned)ctas, 256, 0, s, tab, map, (const float2*)ctx->tw32);
    SC_KB_SWITCH(logL, SC_KBFX, return length_fail("kb_fwd_x"))
#undef SC_KBFX
    SC_LAUNCH_CHECK("kb_fwd_x");
    return SC_OK;
}

int batch_fwd_y_launch(int logL, const BunchDesc* tab, const CtaRef* map, int64_t ctas, cudaStream_t s) {
    if (ctas == 0) return SC_OK;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
#define SC_KBFY(LL) \
    launch_pdl(kb_fwd_y<LL>, (unsigned)ctas, kColW * F2<LL>::NT, 0, s, tab, map, (const float2*)ctx->tw32);
    SC_KB_SWITCH(logL, SC_KBFY, return length_fail("kb_fwd_y"))
#undef SC_KBFY
    SC_LAUNCH_CHECK("kb_fwd_y");
    return SC_OK;
}

int batch_inv_yx_launch(int logL, const BunchDesc* tab, const CtaRef* map, int64_t ctas, size_t smem_plane,
                        cudaStream_t s) {
    if (ctas == 0) return SC_OK;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const size_t smem = batch_plane_smem(logL, (int64_t)smem_plane);
#define SC_KBIYX(LL)                                                                                  \
    {                                                                                                 \
        SC_TRY(set_smem(kb_inv_yx<LL>, smem));                                                        \
        launch_pdl(kb_inv_yx<LL>, (unsigned)ctas, 256, smem, s, tab, map, (const float2*)ctx->tw32); \
    }
    SC_KB_SWITCH(logL, SC_KBIYX, return length_fail("kb_inv_yx"))
#undef SC_KBIYX
    SC_LAUNCH_CHECK("kb_inv_yx");
    return SC_OK;
}

int batch_zpass_launch(int logLz, const BunchDesc* tab, const CtaRef* map, int64_t ctas, bool image,
                       cudaStream_t s) {
    if (ctas == 0) return SC_OK;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
#define SC_KBZ(LL)                                                                                             \
    {                                                                                                          \
        const size_t smem = sizeof(float2) * kColW * F2<LL>::S * 2 + sizeof(float) * 3 * (LL / 2 + 1) * kColW + \
                            (image ? sizeof(float2) * (LL / 2 + 1) * kColW : 0);                                  \
        SC_TRY(set_smem(kb_zpass<LL>, smem));                                                                  \
        launch_pdl(kb_zpass<LL>, (unsigned)ctas, kColW * F2<LL>::NT, smem, s, tab, map,                        \
                   (const float2*)ctx->tw32);                                                                  \
    }
    SC_KB_SWITCH(logLz, SC_KBZ, return length_fail("kb_zpass"))
#undef SC_KBZ
    SC_LAUNCH_CHECK("kb_zpass");
    return SC_OK;
}

#undef SC_KB_SWITCH

}  // namespace sc
