// FP64 meshes in double-FP32 mode: the scalar potential's z pass and its
// inverse x pass into the spare lane of the packed nodes, in double-FP32
// (dd.cuh).  The forward passes and the inverse y pass are the field solve's
// (dd_xy.cu).
#include "fft2.cuh"
#include "pipeline.cuh"
#include "zstage.cuh"

namespace sc {

// The potential's z pass (the FP32 k2_zpass_pot of potential.cu in
// double-FP32): forward z transform of the double-FP32 rho^(kx, ky, .),
// times the real FP64 potential spectrum (split with integer operations),
// plus rho^ at -kz times the half-stored FP64 image spectrum with the
// cathode, inverse transform, z < nz stored (double-FP32).  The tile's
// spectra are copied to shared memory with cp.async during the forward
// transform; the forward spectrum stays in shared memory for the image
// term.  HALF: nz = L/2.
template <int L, bool HALF, typename TG>
__global__ void __launch_bounds__(kColW * F2<L>::NT, 1)
    k2_dd_zpass_pot(const ddc* __restrict__ B, ddc* __restrict__ C, int Hx, int Ly, int nz,
                    const TG* __restrict__ pf, const double2* __restrict__ pi, int image, int Hy,
                    const ddc* __restrict__ tw) {
    using E = F2<L>;
    constexpr int RL = E::R1, HZ = L / 2 + 1;
    __shared__ ddc swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    ddc* xb = reinterpret_cast<ddc*>(smraw);
    ddc* spec = xb + kColW * E::S;
    double2* gis = reinterpret_cast<double2*>(spec + kColW * E::S);  // [HZ][kColW] image spectrum
    TG* gs = reinterpret_cast<TG*>(gis + HZ * kColW);                 // [HZ][kColW] free-space spectrum
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
            cp_async8(gs + kz * kColW + c, pf + o + gstep * kz);
            if (image) cp_async16(gis + kz * kColW + c, pi + o + gstep * kz);
        }
        cp_async_commit();
    }
    ddc* col = xb + c * E::S;
    ddc* sc = spec + c * E::S;
    ddc v[16];
    if (t < E::R2) {
        const ddc* Bc = B + fl;
        const ddc zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int z = t + E::R2 * s;
            v[s] = (HALF ? E::R2 * s < L / 2 : z < nz) ? Bc[plane * z] : zero;
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
        const TG* glo = gs + t * kColW + c;
        const TG* ghi = gs + (L - t) * kColW + c;
#pragma unroll
        for (int r = 0; r < E::R2; ++r) {
            const int kz = t + RL * r;
            const bool lower = RL * r < L / 2;
            const TG gv = lower ? glo[RL * r * kColW] : ghi[-RL * r * kColW];
            float gh, gl;
            if constexpr (std::is_same<TG, dreal>::value) {
                gh = gv.h;
                gl = gv.l;
            } else {
                dd_split(gv, gh, gl);
            }
            ddc o = dd_scale(v[r], gh, gl);
            if (image) {
                const int kzf = kz <= L / 2 ? kz : L - kz;
                double2 gc = gis[kzf * kColW + c];
                if (kz > L / 2) gc.y = -gc.y;  // S(L - kz) = conj S(kz)
                o = dd_add(o, dd_cmul(sc[xsw((L - kz) & (L - 1))], dd_from(gc)));
            }
            v[r] = o;
        }
    }
    E::template inv<true>(v, col, t, swt);
    if (t < E::R2 && cok) {
        ddc* Cc = C + f;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int z = t + E::R2 * s;
            if (HALF ? E::R2 * s < L / 2 : z < nz) Cc[plane * z] = v[s];
        }
    }
}

// Inverse x of one component into the fourth lane of the packed FP64 nodes
// (k2_dd_inv_x with one component): rows r0 = 2p, r1 = 2p + 1 through one
// complex transform as Xa + i Xb.  HALF: Hx = L/2 + 1 and nx = L/2.
template <int L, bool HALF>
__global__ void __launch_bounds__(256, 1) k2_dd_inv_x1(const ddc* __restrict__ D, dnode4* __restrict__ E4, int nx,
                                                      int rows, int Hx, const ddc* __restrict__ tw) {
    using E = F2<L>;
    __shared__ ddc swt[L];
    stage_twiddles<L>(swt, tw);
    constexpr int P = 256 / E::NT;
    extern __shared__ __align__(16) unsigned char smraw[];
    ddc* xb = reinterpret_cast<ddc*>(smraw);
    const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
    const int r0 = 2 * (blockIdx.x * P + p), r1 = r0 + 1;
    ddc v[16];
    const ddc zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    if (t < E::R1) {
        const ddc* Da = D + (int64_t)r0 * Hx;
        const ddc* Db = Da + Hx;
#pragma unroll
        for (int r = 0; r < E::R2; ++r) {
            const int k = t + E::R1 * r;
            const bool cj = HALF ? (E::R1 * r > L / 2 || (E::R1 * r == L / 2 && t > 0)) : k > L / 2;
            const int kk = HALF ? (E::R1 * r < L / 2 ? t + E::R1 * r : (cj ? L - t - E::R1 * r : L / 2))
                                : (cj ? L - k : k);
            ddc xa = zero, xv = zero;
            if (r0 < rows) xa = Da[kk];
            if (r1 < rows) xv = Db[kk];
            if (cj) {
                xa.h.y = -xa.h.y;
                xa.l.y = -xa.l.y;
                xv.h.y = -xv.h.y;
                xv.l.y = -xv.l.y;
            }
            v[r] = dd_add(xa, rot<true>(xv));  // Xa + i Xb
        }
    }
    E::template inv<true>(v, xb + p * E::S, t, swt);
    if (t < E::R2) {
        double* o = reinterpret_cast<double*>(E4);
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            if (!(HALF ? E::R2 * s < L / 2 : t + E::R2 * s < nx)) continue;
            const double2 e = dd_to(v[s]);
            const int64_t x = t + E::R2 * s;
            if (r0 < rows) o[4 * ((int64_t)r0 * nx + x) + 3] = e.x;
            if (r1 < rows) o[4 * ((int64_t)r1 * nx + x) + 3] = e.y;
        }
    }
}

bool launch2_dd_zpass_pot(int logL, const ddc* B, ddc* C, int Hx, int Ly, int nz, const void* pf, int pfmt,
                          const double2* pi, int image, int Hy, const ddc* tw, cudaStream_t s) {
#define SC_KDZP_GT(LL, HALF, TG)                                                                            \
    {                                                                                                       \
        if (set_smem(k2_dd_zpass_pot<LL, HALF, TG>, smem) != SC_OK) return false;                           \
        launch_pdl(k2_dd_zpass_pot<LL, HALF, TG>, grid, kColW * F2<LL>::NT, smem, s, B, C, Hx, Ly, nz,       \
                   (const TG*)pf, pi, image, Hy, tw);                                                       \
    }
#define SC_KDZP_GO(LL, HALF)                                                                                \
    {                                                                                                       \
        if (pfmt)                                                                                           \
            SC_KDZP_GT(LL, HALF, dreal)                                                                     \
        else                                                                                                \
            SC_KDZP_GT(LL, HALF, double)                                                                    \
    }
// (a dreal spectrum comes from the double-FP32 Green build, which takes
// power-of-two meshes only: nz = L/2)
#define SC_KDZP(LL)                                                                                         \
    {                                                                                                       \
        const size_t smem = sizeof(ddc) * kColW * F2<LL>::S * 2 +                                           \
                            (sizeof(double2) + sizeof(double)) * (LL / 2 + 1) * kColW;                      \
        const unsigned grid = (unsigned)(((int64_t)Hx * Ly + kColW - 1) / kColW);                           \
        if (2 * nz == LL)                                                                                   \
            SC_KDZP_GO(LL, true)                                                                            \
        else if (pfmt)                                                                                      \
            return false;                                                                                   \
        else                                                                                                \
            SC_KDZP_GT(LL, false, double)                                                                   \
    }
    SC_L_SWITCH(logL, SC_KDZP)
#undef SC_KDZP
#undef SC_KDZP_GO
#undef SC_KDZP_GT
    return true;
}

bool launch2_dd_inv_x1(int logL, const ddc* D, dnode4* E4, int nx, int rows, int Hx, const ddc* tw, cudaStream_t s) {
#define SC_KDX1(LL)                                                                                         \
    {                                                                                                       \
        constexpr int P = 256 / F2<LL>::NT;                                                                 \
        const size_t smem = sizeof(ddc) * P * F2<LL>::S;                                                    \
        const unsigned grid = (unsigned)(((rows + 1) / 2 + P - 1) / P);                                     \
        if (2 * nx == LL && 2 * (Hx - 1) == LL) {                                                           \
            if (set_smem(k2_dd_inv_x1<LL, true>, smem) != SC_OK) return false;                              \
            launch_pdl(k2_dd_inv_x1<LL, true>, grid, 256, smem, s, D, E4, nx, rows, Hx, tw);                \
        } else {                                                                                            \
            if (set_smem(k2_dd_inv_x1<LL, false>, smem) != SC_OK) return false;                             \
            launch_pdl(k2_dd_inv_x1<LL, false>, grid, 256, smem, s, D, E4, nx, rows, Hx, tw);               \
        }                                                                                                   \
    }
    SC_L_SWITCH(logL, SC_KDX1)
#undef SC_KDX1
    return true;
}

}  // namespace sc
