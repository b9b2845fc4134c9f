// Scalar potential on the hand-written pipelines (SC_PREC_MIXED and
// SC_PREC_FP64): the step beside the field solve, with the potential
// antiderivative potential_green_function of src/green_functions.jl:13-22
// (defined in the reference, never called there) in place of the field's.
//
//   Green : the cell integrals of 1/r over the stored octant (free space) or
//           quadrant (image), times gamma/(dx dy dz) (the lab-frame potential
//           gamma*phi' of the rest-frame potential), then the parity-reduced
//           transform of pipeline2.cuh with every axis even: one component,
//           real in free space, complex with the flip phase for the image.
//           Mixed meshes: the reference's FP64 8-point difference of the
//           antiderivative near the origin, FP32 Gauss-Legendre quadrature of
//           1/r beyond, with the field build's thresholds (1/r is smoother
//           than its gradient, so the same orders are at least as accurate).
//           FP64 meshes: the FP64 8-point difference everywhere.
//   solve : the field solve's forward x and y transforms of rho, a z pass
//           that multiplies by the one spectrum (+ the image on -kz), the
//           inverse y and x transforms into the spare fourth lane of the
//           packed field nodes, and a copy of that lane to phi.
// Transforms longer than 256 points are not handled here (the caller falls
// back to the FP64 cuFFT schedule of plain.cu).
#include "pipeline2.cuh"

namespace sc {

// Kernel geometry of the potential build (the field build's OctantGeom with
// one component).
struct PotGeom {
    int nx, ny, nz;
    int image;          // dz range [-(nz-1), nz-1] instead of [0, nz-1]
    double dx, dy, dz;  // full cell widths, dz already scaled by gamma
    double offw;        // cathode offset * gamma on the w axis
    double factor;      // gamma / (dx dy dz)
    double scale;       // FPEI / (Lx Ly Lz)
    float ux, uy, uz, uoff;  // widths and offset in units of hmax (half the longest width)
    float kp;           // gamma * scale / (8 hmax): the quadrature's prefactor
    // box of cells (ix < nbx, iy < nby, bz0 <= dz < bz1) holding every near cell
    int nbx, nby, bz0, bz1;
};

constexpr float kPotNear = 6.0f;   // R / hmax below which a cell takes the FP64 difference
constexpr float kPotQ3 = 16.0f;    // 4 points per axis below, 3 below kPotQ2, 2 beyond
constexpr float kPotQ2 = 48.0f;

// corner e (lattice index, ez from bz0 or ez0) of the reference's doubled grid
__device__ __forceinline__ double pot_corner(const PotGeom& g, int ex, int ey, int ez) {
    const double umin = (double)(1 - 2 * g.nx) * g.dx / 2;
    const double vmin = (double)(1 - 2 * g.ny) * g.dy / 2;
    const double wmin = (double)(1 - 2 * g.nz) * g.dz / 2 + g.offw;
    const double u = (double)(ex + g.nx - 1) * g.dx + umin;
    const double v = (double)(ey + g.ny - 1) * g.dy + vmin;
    const double w = (double)(ez + g.nz - 1) * g.dz + wmin;
    return potential_green_n(u, v, w) * g.factor;
}

__device__ __forceinline__ bool pot_near(const PotGeom& g, int ix, int iy, int dz, float& px, float& py, float& pz) {
    px = (float)ix * g.ux;
    py = (float)iy * g.uy;
    pz = fmaf((float)dz, g.uz, g.uoff);
    const float ratio = sqrtf(fmaf(px, px, fmaf(py, py, pz * pz)));
    return ratio < kPotNear && ix < g.nbx && iy < g.nby && dz >= g.bz0 && dz < g.bz1;
}

__device__ __forceinline__ float pot_quad(const PotGeom& g, float cx, float cy, float cz) {
    const float t4[4] = {-0.86113631159405258f, -0.33998104358485626f, 0.33998104358485626f, 0.86113631159405258f};
    const float w4[4] = {0.34785484513745386f, 0.65214515486254614f, 0.65214515486254614f, 0.34785484513745386f};
    const float t3[3] = {-0.77459666924148338f, 0.0f, 0.77459666924148338f};
    const float w3[3] = {0.55555555555555556f, 0.88888888888888889f, 0.55555555555555556f};
    const float t2[2] = {-0.57735026918962576f, 0.57735026918962576f};
    const float w2[2] = {1.0f, 1.0f};
    const float ratio = sqrtf(fmaf(cx, cx, fmaf(cy, cy, cz * cz)));
    const int m = ratio < kPotQ3 ? 4 : ratio < kPotQ2 ? 3 : 2;
    const float* t = m == 4 ? t4 : m == 3 ? t3 : t2;
    const float* w = m == 4 ? w4 : m == 3 ? w3 : w2;
    const float hx = 0.5f * g.ux, hy = 0.5f * g.uy, hz = 0.5f * g.uz;
    float acc = 0.f;
    for (int i = 0; i < m; ++i) {
        const float px = fmaf(hx, t[i], cx);
        for (int j = 0; j < m; ++j) {
            const float py = fmaf(hy, t[j], cy);
            const float wij = w[i] * w[j];
            for (int k = 0; k < m; ++k) {
                const float pz = fmaf(hz, t[k], cz);
                acc = fmaf(wij * w[k], rsqrtf(fmaf(px, px, fmaf(py, py, pz * pz))), acc);
            }
        }
    }
    // the cell average of 1/r times gamma, times FPEI / (Lx Ly Lz)
    return g.kp * acc;
}

// Mixed meshes, one launch, two block roles.  Blocks [0, near_blocks): the
// FP64 antiderivative at the near-box corners, one per thread, into Fn.  The
// other blocks: every far cell by quadrature into G (near cells are left to
// k_pot_near_cells).
__global__ void __launch_bounds__(64) k_pot_split(float* __restrict__ G, double* __restrict__ Fn, PotGeom g,
                                                  int near_blocks) {
    if ((int)blockIdx.x < near_blocks) {
        const int cx = g.nbx + 1, cy = g.nby + 1, cz = g.bz1 - g.bz0 + 1;
        const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
        if (t >= (int64_t)cx * cy * cz) return;
        const int ex = (int)(t % cx), ey = (int)((t / cx) % cy), ez = (int)(t / ((int64_t)cx * cy)) + g.bz0;
        Fn[t] = pot_corner(g, ex, ey, ez);
        return;
    }
    const int zc = g.image ? 2 * g.nz - 1 : g.nz;
    const int64_t t = (blockIdx.x - near_blocks) * (int64_t)blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)g.nx * g.ny * zc;
    if (t >= total) return;
    int ix, iy, iz;
    if (total <= 0x7FFFFFFF) {  // 32-bit index arithmetic
        const unsigned u = (unsigned)t, r = u / (unsigned)g.nx;
        ix = (int)(u - r * (unsigned)g.nx);
        iy = (int)(r % (unsigned)g.ny);
        iz = (int)(r / (unsigned)g.ny);
    } else {
        ix = (int)(t % g.nx);
        iy = (int)((t / g.nx) % g.ny);
        iz = (int)(t / ((int64_t)g.nx * g.ny));
    }
    const int dz = g.image ? iz - (g.nz - 1) : iz;
    float px, py, pz;
    if (pot_near(g, ix, iy, dz, px, py, pz)) return;
    G[t] = pot_quad(g, px, py, pz);
}

// Near cells: the 8-point difference (green_functions.jl:108-111) of the
// corner antiderivatives, one cell per thread.
__global__ void __launch_bounds__(64) k_pot_near_cells(float* __restrict__ G, const double* __restrict__ Fn,
                                                       PotGeom g) {
    pdl_wait();  // the corners come from the preceding k_pot_split
    const int bz = g.bz1 - g.bz0;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)g.nbx * g.nby * bz) return;
    const int ix = (int)(t % g.nbx), iy = (int)((t / g.nbx) % g.nby), dz = (int)(t / ((int64_t)g.nbx * g.nby)) + g.bz0;
    float px, py, pz;
    if (!pot_near(g, ix, iy, dz, px, py, pz)) return;
    const int64_t sy = g.nbx + 1, sz = (int64_t)(g.nbx + 1) * (g.nby + 1);
    const double* f = Fn + ix + sy * iy + sz * (dz - g.bz0);
    auto F = [&](int a, int b, int e) { return f[a + sy * b + sz * e]; };
    const double d = F(1, 1, 1) - F(0, 1, 1) - F(1, 0, 1) - F(1, 1, 0) - F(0, 0, 0) + F(0, 0, 1) + F(0, 1, 0) +
                     F(1, 0, 0);
    const int iz = g.image ? dz + g.nz - 1 : dz;
    G[ix + (int64_t)g.nx * (iy + (int64_t)g.ny * iz)] = (float)(d * g.scale);
}

// FP64 meshes: the antiderivative at every corner of the stored region
// (ez from ez0), then the 8-point difference of every cell.
__global__ void __launch_bounds__(128) k_pot_corners(double* __restrict__ F, PotGeom g, int ez0) {
    const int cx = g.nx + 1, cy = g.ny + 1, cz = g.nz + 1 - ez0;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)cx * cy * cz) return;
    const int ex = (int)(t % cx), ey = (int)((t / cx) % cy), ez = (int)(t / ((int64_t)cx * cy)) + ez0;
    F[t] = pot_corner(g, ex, ey, ez);
}

template <typename OT>  // double, or dreal for the double-FP32 transform
__global__ void __launch_bounds__(128) k_pot_place(const double* __restrict__ F, OT* __restrict__ G, PotGeom g,
                                                   int ez0) {
    pdl_wait();  // the corners come from the preceding k_pot_corners
    const int cx = g.nx + 1, cy = g.ny + 1;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)g.nx * g.ny * (g.nz - ez0)) return;
    const int dx = (int)(t % g.nx), dy = (int)((t / g.nx) % g.ny), dzi = (int)(t / ((int64_t)g.nx * g.ny));
    const int64_t sy = cx, sz = (int64_t)cx * cy;
    const double* f = F + dx + sy * dy + sz * dzi;
    auto Fv = [&](int a, int b, int e) { return f[a + sy * b + sz * e]; };
    const double d = Fv(1, 1, 1) - Fv(0, 1, 1) - Fv(1, 0, 1) - Fv(1, 1, 0) - Fv(0, 0, 0) + Fv(0, 0, 1) +
                     Fv(0, 1, 0) + Fv(1, 0, 0);
    G[t] = OT(d * g.scale);
}

// z pass of the potential: forward z transform of rho^(kx, ky, .), times
// the real potential spectrum (+ rho^ at -kz times the image spectrum),
// inverse transform, z < nz stored into C (one component).  The stored
// spectra are folded to ky <= Ly/2, kz <= Lz/2; the kernel is even along
// every axis, so no sign changes; the half-stored image column of a real
// line gives S(Lz - kz) = conj S(kz).  W columns per CTA, shared-memory
// Stockham transforms (any L).
template <typename T>
__global__ void __launch_bounds__(256) k_zpass_pot(const typename Cplx<T>::T2* __restrict__ B,
                                                   typename Cplx<T>::T2* __restrict__ C, int Hx, int Ly, int nz,
                                                   int Lz, int logLz, int lgW, const T* __restrict__ pf,
                                                   const typename Cplx<T>::T2* __restrict__ pi, int image, int Hy,
                                                   const typename Cplx<T>::T2* __restrict__ tw) {
    using T2 = typename Cplx<T>::T2;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int W = 1 << lgW;
    const int n = W << logLz;
    T2* spec = reinterpret_cast<T2*>(smraw);
    T2* a = spec + n;
    T2* b = a + n;
    const int kx0 = blockIdx.x << lgW;
    const int ky = blockIdx.y;
    const int64_t plane = (int64_t)Hx * Ly;
    const int stages = ((logLz & 3) ? 1 : 0) + (logLz >> 2);
    T2* first = (stages & 1) ? a : spec;
    T2* second = (stages & 1) ? spec : a;
    for (int it = threadIdx.x; it < n; it += blockDim.x) {
        const int z = it >> lgW, kx = kx0 + (it & (W - 1));
        T2 v = Cplx<T>::make(0, 0);
        if (z < nz && kx < Hx) v = B[kx + (int64_t)Hx * ky + plane * z];
        first[it] = v;
    }
    __syncthreads();
    smem_fft<false>(first, second, Lz, logLz, lgW, tw);  // result in spec
    const int kyf = ky <= Ly / 2 ? ky : Ly - ky;
    const int halfz = Lz >> 1;
    const int64_t gstep = (int64_t)Hx * Hy;
    for (int it = threadIdx.x; it < n; it += blockDim.x) {
        const int kz = it >> lgW, w = it & (W - 1);
        const int kx = kx0 + w;
        T2 r = Cplx<T>::make(0, 0);
        if (kx < Hx) {
            const int kzf = kz <= halfz ? kz : Lz - kz;
            const int64_t o = kx + (int64_t)Hx * kyf;
            const T g = pf[o + gstep * kzf];
            const T2 p = spec[it];
            r = Cplx<T>::make(p.x * g, p.y * g);
            if (image) {
                T2 gc = pi[o + gstep * kzf];
                if (kz > halfz) gc.y = -gc.y;
                r = cadd(r, cmul(spec[(((Lz - kz) & (Lz - 1)) << lgW) + w], gc));
            }
        }
        a[it] = r;
    }
    __syncthreads();
    const T2* res = smem_fft<true>(a, b, Lz, logLz, lgW, tw);
    for (int it = threadIdx.x; it < (nz << lgW); it += blockDim.x) {
        const int z = it >> lgW, kx = kx0 + (it & (W - 1));
        if (kx < Hx) C[kx + (int64_t)Hx * ky + plane * z] = res[it];
    }
}

// The same z pass for FP32 and Lz <= 256 on the register two-step transform
// (zpass_body's thread map: kColW columns of the flattened (kx, ky) plane per
// CTA, F2<L>::NT threads per column).  The tile's free-space spectrum
// (Lz/2 + 1 values per column) and, with the image, its half-stored image
// spectrum are copied to shared memory with cp.async while the forward
// transform runs; the forward spectrum stays in shared memory for the image
// term at -kz.  HALF: nz = Lz/2.
template <int L, bool HALF>
__global__ void __launch_bounds__(kColW * F2<L>::NT, SC_ZPASS_MINB)
    k2_zpass_pot(const float2* __restrict__ B, float2* __restrict__ C, int Hx, int Ly, int nz,
                 const float* __restrict__ pf, const float2* __restrict__ pi, int image, int Hy,
                 const float2* __restrict__ tw) {
    using E = F2<L>;
    constexpr int RL = E::R1, HZ = L / 2 + 1;
    __shared__ float2 swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    float2* xb = reinterpret_cast<float2*>(smraw);
    float2* spec = xb + kColW * E::S;
    float2* gis = spec + kColW * E::S;                    // [HZ][kColW] image spectrum
    float* gs = reinterpret_cast<float*>(gis + HZ * kColW);  // [HZ][kColW] free-space spectrum
    const int c = threadIdx.x % kColW, t = threadIdx.x / kColW;
    const int64_t plane = (int64_t)Hx * Ly;
    const int f = blockIdx.x * kColW + c;
    const bool cok = f < plane;
    const int fl = cok ? f : (int)plane - 1;
    const int ky = fl / Hx, kx = fl - ky * Hx;
    const int kyf = ky <= Ly / 2 ? ky : Ly - ky;
    const int64_t gstep = (int64_t)Hx * Hy;
    {
        const int64_t o = kx + (int64_t)Hx * kyf;
        for (int kz = t; kz < HZ; kz += blockDim.x / kColW) {
            cp_async4(gs + kz * kColW + c, pf + o + gstep * kz);
            if (image) cp_async8(gis + kz * kColW + c, pi + o + gstep * kz);
        }
        cp_async_commit();
    }
    float2* col = xb + c * E::S;
    float2* sc = spec + c * E::S;
    float2 v[16];
    if (t < E::R2) {
        const float2* Bc = B + fl;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int z = t + E::R2 * s;
            v[s] = (HALF ? E::R2 * s < L / 2 : z < nz) ? Bc[plane * z] : make_float2(0.f, 0.f);
        }
    }
    E::template fwd<false>(v, col, t, swt);
    if (t < E::R1) {
#pragma unroll
        for (int r = 0; r < E::R2; ++r) sc[t + xoff(RL * r)] = v[r];
    }
    cp_async_wait_all();
    __syncthreads();
    if (t < E::R1) {
        // kz = t + RL*r: folded index kz below L/2, L - kz at or above it
        const float* glo = gs + t * kColW + c;
        const float* ghi = gs + (L - t) * kColW + c;
#pragma unroll
        for (int r = 0; r < E::R2; ++r) {
            const int kz = t + RL * r;
            const bool lower = RL * r < L / 2;
            const float g = lower ? glo[RL * r * kColW] : ghi[-RL * r * kColW];
            const float2 X = v[r];
            float2 o = make_float2(X.x * g, X.y * g);
            if (image) {
                const int kzf = kz <= L / 2 ? kz : L - kz;
                float2 gc = gis[kzf * kColW + c];
                if (kz > L / 2) gc.y = -gc.y;  // S(L - kz) = conj S(kz)
                o = cadd(o, cmul(sc[xsw((L - kz) & (L - 1))], gc));
            }
            v[r] = o;
        }
    }
    E::template inv<true>(v, col, t, swt);
    if (t < E::R2 && cok) {
        float2* Cc = C + f;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int z = t + E::R2 * s;
            if (HALF ? E::R2 * s < L / 2 : z < nz) Cc[plane * z] = v[s];
        }
    }
}

static bool launch2_zpass_pot(int logLz, const float2* B, float2* C, int Hx, int Ly, int nz, const float* pf,
                              const float2* pi, int image, int Hy, const float2* tw, cudaStream_t s) {
#define SC_K2ZP_GO(LL, HALF)                                                                               \
    {                                                                                                      \
        if (set_smem(k2_zpass_pot<LL, HALF>, smem) != SC_OK) return false;                                 \
        k2_zpass_pot<LL, HALF><<<grid, kColW * F2<LL>::NT, smem, s>>>(B, C, Hx, Ly, nz, pf, pi, image, Hy, tw); \
    }
#define SC_K2ZP(LL)                                                                                         \
    {                                                                                                       \
        const size_t smem = sizeof(float2) * kColW * F2<LL>::S * 2 + sizeof(float2) * (LL / 2 + 1) * kColW + \
                            sizeof(float) * (LL / 2 + 1) * kColW;                                           \
        const unsigned grid = (unsigned)(((int64_t)Hx * Ly + kColW - 1) / kColW);                          \
        if (2 * nz == LL)                                                                                   \
            SC_K2ZP_GO(LL, true)                                                                            \
        else                                                                                                \
            SC_K2ZP_GO(LL, false)                                                                           \
    }
    SC_L_SWITCH(logLz, SC_K2ZP)
#undef SC_K2ZP
#undef SC_K2ZP_GO
    return true;
}

template <typename T>
__global__ void __launch_bounds__(256) k_lane3(const T* __restrict__ E4, T* __restrict__ phi, int64_t N) {
    pdl_wait();
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < N) phi[i] = E4[4 * i + 3];
}

// fmt < 0: either format (the double-FP32 z pass reads both)
static bool pot_key_matches(const GreenKey& k, const sc_mesh* m, double offz, int fmt = -1) {
    return k.valid && k.delta[0] == m->delta[0] && k.delta[1] == m->delta[1] && k.delta[2] == m->delta[2] &&
           k.gamma == m->gamma && k.offset_z == offz && (fmt < 0 || k.fmt == fmt);
}

// Builds the compressed potential spectrum (free space, or the image at
// offset offz) unless the cached one matches the geometry.  dd (FP64 meshes
// in double-FP32 mode): the free-space spectrum's transform in double-FP32
// where it applies, stored as dreal; a cached FP64 one serves too.
template <typename T>
static int pot_green(sc_mesh* m, bool image, cudaStream_t s, bool dd = false) {
    using T2 = typename Cplx<T>::T2;
    NativeWork& w = m->nw;
    const double offz = image ? 2 * m->lo[2] + (m->hi[2] - m->lo[2]) : 0.0;  // free_space.jl:39
    GreenKey& key = image ? w.key_pimg : w.key_pfree;
    if (m->green_cache && pot_key_matches(key, m, offz, dd && !image ? -1 : 0)) return SC_OK;
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const T2* tw = twiddles<T>(ctx);
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    const int Hy = Ly / 2 + 1, Hz = Lz / 2 + 1;
    const int zc = image ? 2 * nz - 1 : nz;
    const int ez0 = image ? -(nz - 1) : 0;
    PotGeom g;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.image = image ? 1 : 0;
    g.dx = m->delta[0];
    g.dy = m->delta[1];
    g.dz = m->delta[2] * m->gamma;  // green_functions.jl:73
    g.offw = image ? offz * m->gamma : 0.0;
    g.factor = m->gamma / (g.dx * g.dy * g.dz);
    g.scale = kFpei / ((double)Lx * Ly * Lz);
    const double hmax = 0.5 * fmax(g.dx, fmax(g.dy, g.dz));
    g.ux = (float)(g.dx / hmax);
    g.uy = (float)(g.dy / hmax);
    g.uz = (float)(g.dz / hmax);
    g.uoff = (float)(g.offw / hmax);
    g.kp = (float)(m->gamma * g.scale / (8.0 * hmax));
    {
        const double reach = (double)kPotNear * hmax;
        g.nbx = (int)fmin((double)nx, floor(reach / g.dx) + 2.0);
        g.nby = (int)fmin((double)ny, floor(reach / g.dy) + 2.0);
        g.bz0 = (int)fmax((double)ez0, floor((-reach - g.offw) / g.dz) - 1.0);
        g.bz1 = (int)fmin((double)nz, ceil((reach - g.offw) / g.dz) + 2.0);
        if (g.bz1 <= g.bz0) g.nbx = g.nby = 0, g.bz0 = g.bz1 = 0;
    }
    const bool fp32 = std::is_same<T, float>::value;
    const int64_t cells = (int64_t)nx * ny * zc;
    const int64_t corners = fp32 ? (int64_t)(g.nbx + 1) * (g.nby + 1) * (g.bz1 - g.bz0 + 1)
                                 : (int64_t)(nx + 1) * (ny + 1) * (zc + 1);
    const int64_t t2n = (int64_t)Hx * Hy * zc;
    const int64_t t1n = (int64_t)Hx * ny * zc;
    // scratch: corners (FP64) | octant (T) | x pass (T) | x+y pass (T), 256-byte aligned parts
    auto up = [](int64_t b) { return (b + 255) / 256 * 256; };
    const int64_t o_oct = up(sizeof(double) * corners), o_t1 = o_oct + up(sizeof(T) * cells);
    const int64_t o_t2 = o_t1 + up(sizeof(T) * t1n), need = o_t2 + up(sizeof(T) * t2n);
    if (w.pscratch_cap < need) {
        w.pscratch_cap = 0;
        SC_CUDA(dev_realloc(&w.pscratch, need));
        w.pscratch_cap = need;
    }
    void*& dst = image ? w.pimg : w.pfree;
    if (!dst) SC_CUDA(dev_alloc(&dst, (image ? sizeof(T2) : sizeof(T)) * (int64_t)Hx * Hy * Hz));
    unsigned char* base = (unsigned char*)w.pscratch;
    double* F = (double*)base;
    T* G = (T*)(base + o_oct);
    T* T1 = (T*)(base + o_t1);
    T* Txy = (T*)(base + o_t2);
    if (fp32) {
        const bool has_near = g.nbx > 0 && g.nby > 0 && g.bz1 > g.bz0;
        const int near_blocks = has_near ? (int)((corners + 63) / 64) : 0;
        k_pot_split<<<(unsigned)(near_blocks + (cells + 63) / 64), 64, 0, s>>>((float*)G, F, g, near_blocks);
        SC_LAUNCH_CHECK("k_pot_split");
        if (has_near) {
            const int64_t box = (int64_t)g.nbx * g.nby * (g.bz1 - g.bz0);
            launch_pdl(k_pot_near_cells, (unsigned)((box + 63) / 64), 64, 0, s, (float*)G, (const double*)F, g);
            SC_LAUNCH_CHECK("k_pot_near_cells");
        }
    } else {
        k_pot_corners<<<(unsigned)((corners + 127) / 128), 128, 0, s>>>(F, g, ez0);
        SC_LAUNCH_CHECK("k_pot_corners");
        if (dd && !image && dd_green_applies(w.log2L[0], w.log2L[1], w.log2L[2], nx, ny, nz)) {
            // double-FP32: the octant split as it is placed, then the paired
            // kernels' single-component mode with dreal values
            launch_pdl(k_pot_place<dreal>, (unsigned)((cells + 127) / 128), 128, 0, s, (const double*)F, (dreal*)G, g,
                       ez0);
            SC_LAUNCH_CHECK("k_pot_place");
            if (!launch_dd_green(w.log2L[0], w.log2L[2], (dreal*)G, (dreal*)Txy, (dreal*)dst, nx, ny, nz, Hx, cells,
                                 t2n, 1.0, (const ddc*)ctx->twdd, s, 1))
                return fail(SC_ERR_CUDA, "double-FP32 potential Green transform did not launch");
            SC_LAUNCH_CHECK("double-FP32 potential Green transform");
            m->launches += 3;
            key.delta[0] = m->delta[0];
            key.delta[1] = m->delta[1];
            key.delta[2] = m->delta[2];
            key.gamma = m->gamma;
            key.offset_z = offz;
            key.fmt = 1;
            key.valid = true;
            return SC_OK;
        }
        launch_pdl(k_pot_place<double>, (unsigned)((cells + 127) / 128), 128, 0, s, (const double*)F, (double*)G, g,
                   ez0);
        SC_LAUNCH_CHECK("k_pot_place");
    }
    // parity-reduced transform, every axis even (pipeline2.cuh)
    const int64_t plane = (int64_t)Hx * Hy;
    // the paired kernels' single-component mode where they apply (Lx = Ly):
    // the slice staged in shared memory, constant offsets for power-of-two axes
    if (!launch_green_xy_field<T>(w.log2L[0], w.log2L[1], G, Txy, nx, ny, zc, Hx, cells, t2n, tw, s, GreenNear{}, 1) &&
        !launch3_green_xy<T>(w.log2L[0], w.log2L[1], G, Txy, nx, ny, zc, Hx, cells, t2n, tw, s, 1, -1, -1)) {
        if (!(launch3_green_x<T>(w.log2L[0], G, T1, nx, ny * zc, Hx, cells, t1n, tw, s, 1, -1) &&
              launch3_green_col<T>(false, w.log2L[1], T1, Txy, Hx, zc, ny, -1, Hx, (int64_t)Hx * ny, t1n, Hx, plane, t2n,
                                   tw, s, 1, 0)))
            return fail(SC_ERR_UNSUPPORTED, "potential Green x/y pass: transform length out of range");
    }
    SC_LAUNCH_CHECK("potential Green x/y");
    if (!(!image && launch_green_z_field<T>(w.log2L[2], Txy, (T*)dst, (int)plane, nz, plane, t2n, plane, plane * Hz,
                                            1.0, tw, s, 1)) &&
        !launch3_green_col<T>(image, w.log2L[2], Txy, dst, (int)plane, 1, nz, -1, plane, 0, t2n, plane, 0, plane * Hz,
                              tw, s, 1, 0))
        return fail(SC_ERR_UNSUPPORTED, "potential Green z pass: transform length out of range");
    SC_LAUNCH_CHECK("potential Green z");
    m->launches += 4;
    key.delta[0] = m->delta[0];
    key.delta[1] = m->delta[1];
    key.delta[2] = m->delta[2];
    key.gamma = m->gamma;
    key.offset_z = offz;
    key.fmt = 0;
    key.valid = true;
    return SC_OK;
}

template <typename T>
static int potential_t(sc_mesh* m, int at_cathode, void* phi, cudaStream_t s) {
    using T2 = typename Cplx<T>::T2;
    SC_TRY(alloc_work<T>(m));
    NativeWork& w = m->nw;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int Lx = w.L[0], Ly = w.L[1], Lz = w.L[2], Hx = w.Hx;
    const int Hy = Ly / 2 + 1;
    (void)Lx;
    // The Green spectra do not depend on rho: build them on the mesh's side
    // stream beside the forward x and y transforms, join before the z pass.
    if (!m->side) SC_CUDA(cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking));
    if (!m->ev_fork) SC_CUDA(cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming));
    if (!m->ev_join) SC_CUDA(cudaEventCreateWithFlags(&m->ev_join, cudaEventDisableTiming));
    SC_CUDA(cudaEventRecord(m->ev_fork, s));
    SC_CUDA(cudaStreamWaitEvent(m->side, m->ev_fork, 0));
    // FP64 meshes in double-FP32 mode: every pass but the Green function's
    // antiderivative in double-FP32 (dd_xy.cu, dd_pot.cu, dd_green.cu)
    const bool dd = native_dd_applies(m);
    int st = pot_green<T>(m, false, m->side, dd);
    if (st == SC_OK && at_cathode) st = pot_green<T>(m, true, m->side);
    const cudaError_t ej = cudaEventRecord(m->ev_join, m->side);
    if (st == SC_OK && ej != cudaSuccess) st = cuda_fail(ej, "cudaEventRecord");
    if (st == SC_OK) st = native_forward(m, s, dd);
    cudaStreamWaitEvent(s, m->ev_join, 0);  // joined on every path
    SC_TRY(st);
    DeviceCtx* ctx = nullptr;
    SC_TRY(device_ctx(&ctx));
    const T2* tw = twiddles<T>(ctx);
    T2* C = (T2*)w.C;
    if (dd) {
        const ddc* twdd = (const ddc*)ctx->twdd;
        const int rows = ny * nz;
        if (!launch2_dd_zpass_pot(w.log2L[2], (const ddc*)w.B, (ddc*)C, Hx, Ly, nz, w.pfree, w.key_pfree.fmt,
                                  (const double2*)w.pimg, at_cathode ? 1 : 0, Hy, twdd, s) ||
            !launch2_dd_col<true>(w.log2L[1], (const ddc*)C, (ddc*)w.A, Hx, nz, 1, Ly, ny, Hx, (int64_t)Hx * Ly, 0, Hx,
                                  (int64_t)Hx * ny, 0, twdd, s) ||
            !launch2_dd_inv_x1(w.log2L[0], (const ddc*)w.A, (dnode4*)m->efield, nx, rows, Hx, twdd, s))
            return fail(SC_ERR_CUDA, "double-FP32 potential passes did not launch");
        SC_LAUNCH_CHECK("double-FP32 potential z, y, x");
        m->launches += 3;
        launch_pdl(k_lane3<T>, (unsigned)((m->N + 255) / 256), 256, 0, s, (const T*)m->efield, (T*)phi, m->N);
        SC_LAUNCH_CHECK("k_lane3");
        m->launches += 1;
        return SC_OK;
    }
    const bool two_z = std::is_same<T, float>::value && (w.engine >= 0 ? w.engine : fft_engine()) == 0;
    if (two_z && launch2_zpass_pot(w.log2L[2], (const float2*)w.B, (float2*)C, Hx, Ly, nz, (const float*)w.pfree,
                                   (const float2*)w.pimg, at_cathode ? 1 : 0, Hy, (const float2*)tw, s)) {
        SC_LAUNCH_CHECK("k2_zpass_pot");
    } else {
        int lgW = pick_cols(w.log2L[2]);
        while (lgW > 0 && sizeof(T2) * 3 * ((size_t)1 << lgW) * Lz > 200 * 1024) --lgW;
        const int W = 1 << lgW;
        const size_t smem = sizeof(T2) * 3 * W * Lz;
        SC_TRY(set_smem(k_zpass_pot<T>, smem));
        dim3 grid((Hx + W - 1) / W, Ly);
        k_zpass_pot<T><<<grid, 256, smem, s>>>((const T2*)w.B, C, Hx, Ly, nz, Lz, w.log2L[2], lgW, (const T*)w.pfree,
                                                (const T2*)w.pimg, at_cathode ? 1 : 0, Hy, tw);
        SC_LAUNCH_CHECK("k_zpass_pot");
    }
    // inverse y and x into lane 3 of the packed nodes
    const bool two = std::is_same<T, float>::value && (w.engine >= 0 ? w.engine : fft_engine()) == 0;
    if (two && launch2_inv_yx(w.log2L[0], w.log2L[1], (const float2*)C, (float4*)m->efield, nx, ny, nz, Hx,
                              (const float2*)tw, s, m->fused_smem_cap, 1, 3)) {
        SC_LAUNCH_CHECK("k2_inv_yx");
        m->launches += 1;
    } else {
        T2* A = (T2*)w.A;
        const int rows = ny * nz;
        if (!(two && launch2_col(true, w.log2L[1], (const float2*)C, (float2*)A, Hx, Ly, ny, Hx, (int64_t)Hx * Ly, 0,
                                 Hx, (int64_t)Hx * ny, 0, nz, 1, (const float2*)tw, s)))
            SC_TRY(run_col<true, T>(C, A, Hx, Ly, w.log2L[1], Ly, ny, Hx, (int64_t)Hx * Ly, 0, Hx, (int64_t)Hx * ny, 0,
                                    nz, 1, tw, s));
        if (two && launch2_inv_x1(w.log2L[0], (const float2*)A, (float*)m->efield, nx, rows, Hx, (const float2*)tw, s)) {
            SC_LAUNCH_CHECK("k2_inv_x1");
        } else {
            const int lgP = pick_rows(w.log2L[0]);
            const int P = 1 << lgP;
            const size_t smem = sizeof(T2) * 2 * P * w.L[0];
            SC_TRY(set_smem(k_inv_x1<T>, smem));
            k_inv_x1<T><<<((rows + 1) / 2 + P - 1) / P, 256, smem, s>>>(A, (T*)m->efield, nx, rows, w.L[0], w.log2L[0],
                                                                       Hx, lgP, tw);
            SC_LAUNCH_CHECK("k_inv_x1");
        }
        m->launches += 2;
    }
    launch_pdl(k_lane3<T>, (unsigned)((m->N + 255) / 256), 256, 0, s, (const T*)m->efield, (T*)phi, m->N);
    SC_LAUNCH_CHECK("k_lane3");
    m->launches += 2;
    return SC_OK;
}

int native_potential(sc_mesh* m, int at_cathode, void* phi, cudaStream_t s) {
    const NativeWork& w = m->nw;
    if (w.log2L[0] > 8 || w.log2L[1] > 8 || w.log2L[2] > 8)
        return fail(SC_ERR_UNSUPPORTED, "the native potential solve takes transforms of at most 256 points");
    if (m->precision == SC_PREC_MIXED) return potential_t<float>(m, at_cathode, phi, s);
    return potential_t<double>(m, at_cathode, phi, s);
}

}  // namespace sc
