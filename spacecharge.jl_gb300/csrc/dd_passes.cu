// FP64 meshes: the free-space z pass in double-FP32 (dd.cuh), one of the
// double-FP32 passes of the FP64 pipeline:
//   k2_dd_zpass    forward z, Green products, three inverse z (free space)
//   k2_dd_col_inv  inverse y of the three components (dd_inverse.cu)
//   k2_dd_inv_x    inverse x, two rows per complex transform, packed nodes
//                  (dd_inverse.cu)
// Between the passes the spectra stay in double-FP32 (a ddc is 16 bytes, as
// a double2, so the FP64 pipeline's buffers hold them); FP64 values enter
// through an integer split and leave through one FP64 addition per part.
// Translation units of their own, so that they compile beside the others.
#include "fft2.cuh"
#include "pipeline.cuh"
#include "zstage.cuh"

namespace sc {

// z pass of an FP64 mesh in free space: the double-FP32 spectrum
// rho^(kx, ky, .) of the forward x and y passes is transformed forward,
// multiplied by i g for the three Green spectra (TG: double, split with
// integer operations, or dreal from the double-FP32 Green transform) and
// transformed back, the result kept in double-FP32 for the inverse passes.
// Same column tiles, thread layout and compile-time z patterns as the FP32
// zpass_body of pipeline2.cuh (free-space branch); the Green values are
// copied to shared memory asynchronously during the forward transform.
template <int L, bool HALF, typename TG>
__global__ void __launch_bounds__(kColW * F2<L>::NT, 1) k2_dd_zpass(const ddc* __restrict__ B, ddc* __restrict__ C,
                                                                   int Hx, int Ly, int nz, GreenView gv,
                                                                   const ddc* __restrict__ tw) {
    using E = F2<L>;
    constexpr int RL = E::R1;
    constexpr int HZ = L / 2 + 1;
    __shared__ ddc swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    ddc* xb = reinterpret_cast<ddc*>(smraw);
    ddc* spec = xb + kColW * E::S;
    TG* gsm = reinterpret_cast<TG*>(spec + kColW * E::S);  // [3][HZ][kColW]
    const int tile = blockIdx.x;
    const int c = threadIdx.x % kColW, t = threadIdx.x / kColW;
    const int64_t plane = (int64_t)Hx * Ly;
    prefetch_green<L, TG>(gsm, gv, Hx, Ly, tile);
    const int f = tile * kColW + c;
    const bool cok = f < plane;
    const int fl = cok ? f : (int)plane - 1;
    const int ky = fl / Hx;
    ddc* col = xb + c * E::S;
    ddc* sc = spec + c * E::S;
    ddc v[16];
    if (t < E::R2) {
        const ddc* Bc = B + fl;
        const ddc zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int z = t + E::R2 * s;
            const bool in = HALF ? E::R2 * s < L / 2 : z < nz;
            v[s] = in ? Bc[plane * z] : zero;
        }
    }
    E::template fwd<false>(v, col, t, swt);
    // this thread's spectrum values, kept for the three components (read
    // back by the same thread only)
    if (t < E::R1) {
#pragma unroll
        for (int r = 0; r < E::R2; ++r) sc[t + xoff(E::R1 * r)] = v[r];
    }
    cp_async_wait_all();
    __syncthreads();
    const float ysign = ky <= Ly / 2 ? 1.f : -1.f;
    for (int comp = 0; comp < 3; ++comp) {
        if (t < E::R1) {
            // signs as in zpass_body: component 1 odd along y, component 2
            // odd along z (kz > L/2)
            const float sy = comp == 1 ? ysign : 1.f;
            const float su = comp == 2 ? -sy : sy;
            const float sm = t > 0 ? su : sy;  // kz = L/2 + t
            const TG* gfc = gsm + comp * HZ * kColW + c;
            const TG* glo = gfc + t * kColW;
            const TG* ghi = gfc + (L - t) * kColW;
            const ddc* sct = sc + t;
#pragma unroll
            for (int r = 0; r < E::R2; ++r) {
                const TG gd = RL * r < L / 2 ? glo[RL * r * kColW] : ghi[-RL * r * kColW];
                const float sg = RL * r < L / 2 ? sy : RL * r == L / 2 ? sm : su;
                float gh, gl;
                if constexpr (std::is_same<TG, dreal>::value) {
                    gh = gd.h;
                    gl = gd.l;
                } else {
                    dd_split(gd, gh, gl);
                }
                v[r] = rot<true>(dd_scale(sct[xoff(RL * r)], gh * sg, gl * sg));  // X * (i g)
            }
        }
        E::template inv<true>(v, col, t, swt);
        if (t < E::R2 && cok) {
            ddc* Cc = C + comp * (plane * nz) + f;
#pragma unroll
            for (int s = 0; s < E::R1; ++s) {
                const int z = t + E::R2 * s;
                if (HALF ? E::R2 * s < L / 2 : z < nz) Cc[plane * z] = v[s];
            }
        }
    }
}

bool launch2_dd_zpass(int logL, const ddc* B, ddc* C, int Hx, int Ly, int nz, const GreenView& gv, int gfmt,
                      const ddc* tw, cudaStream_t s) {
    if (gv.image || logL > 8) return false;
#define SC_KDZ_GO(LL, HALF, TG)                                                                             \
    {                                                                                                       \
        const size_t smem = sizeof(ddc) * kColW * F2<LL>::S * 2 + sizeof(TG) * 3 * (LL / 2 + 1) * kColW;    \
        const int64_t ncol = (int64_t)Hx * Ly;                                                              \
        const unsigned grid = (unsigned)((ncol + kColW - 1) / kColW);                                       \
        if (set_smem(k2_dd_zpass<LL, HALF, TG>, smem) != SC_OK) return false;                               \
        launch_pdl(k2_dd_zpass<LL, HALF, TG>, grid, kColW * F2<LL>::NT, smem, s, B, C, Hx, Ly, nz, gv, tw); \
    }
#define SC_KDZ(LL)                                                                                          \
    {                                                                                                       \
        if (2 * nz == LL) {                                                                                 \
            if (gfmt)                                                                                       \
                SC_KDZ_GO(LL, true, dreal)                                                                  \
            else                                                                                            \
                SC_KDZ_GO(LL, true, double)                                                                 \
        } else {                                                                                            \
            if (gfmt)                                                                                       \
                SC_KDZ_GO(LL, false, dreal)                                                                 \
            else                                                                                            \
                SC_KDZ_GO(LL, false, double)                                                                \
        }                                                                                                   \
    }
    SC_L_SWITCH(logL, SC_KDZ)
#undef SC_KDZ
#undef SC_KDZ_GO
    return true;
}

}  // namespace sc
