// FP64 meshes: the x and y passes in double-FP32 (dd.cuh), before and
// after the double-FP32 z pass of dd_passes.cu (or the FP64 one, with the
// cathode image: the forward y pass then widens its output to FP64 and the
// inverse y pass splits its input).
#include "fft2.cuh"
#include "pipeline.cuh"
#include "zstage.cuh"

namespace sc {

// Transforms of the columns of nbatch batches and gridDim.y components,
// element (col, n, batch, comp) at base + col + n*as + batch*bs + comp*cs;
// one CTA per kColW columns of one component (blockIdx.y), the column
// layout of the FP32 col_body.  Forward: inputs n < n_valid (zero beyond),
// all L outputs.  Inverse (unnormalised): all L inputs, outputs
// n < n_store.  TI / TO: double2 (FP64) or ddc (double-FP32) buffers.
template <int L, bool INV, typename TI, typename TO>
__global__ void __launch_bounds__(kColW * F2<L>::NT, 2) k2_dd_col(const TI* __restrict__ in, TO* __restrict__ out,
                                                                 int ncols, int nbatch, int n_valid, int n_store,
                                                                 int64_t as_in, int64_t bs_in, int64_t cs_in,
                                                                 int64_t as_out, int64_t bs_out, int64_t cs_out,
                                                                 const ddc* __restrict__ tw) {
    using E = F2<L>;
    __shared__ ddc swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    ddc* xb = reinterpret_cast<ddc*>(smraw);
    const int c = threadIdx.x % kColW, t = threadIdx.x / kColW;
    const int64_t f = (int64_t)blockIdx.x * kColW + c;
    const int64_t total = (int64_t)ncols * nbatch;
    const bool cok = f < total;
    const int64_t fl = cok ? f : total - 1;  // past the end: read the last column, store nothing
    const int b = (int)(fl / ncols);
    const int col = (int)(fl - (int64_t)b * ncols);
    const int comp = blockIdx.y;
    ddc v[16];
    const TI* st = in + b * bs_in + comp * cs_in + col + t * as_in;
    TO* dt = out + b * bs_out + comp * cs_out + col + t * as_out;
    if constexpr (!INV) {
        const bool half = 2 * n_valid == L;  // sample s exists for R2*s < L/2
        if (t < E::R2) {
            const ddc zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
            for (int s = 0; s < E::R1; ++s) {
                const bool ok = half ? E::R2 * s < L / 2 : t + E::R2 * s < n_valid;
                v[s] = ok ? dd_load(st + E::R2 * s * as_in) : zero;
            }
        }
        E::template fwd<false>(v, xb + c * E::S, t, swt);
        if (t < E::R1 && cok) {
#pragma unroll
            for (int r = 0; r < E::R2; ++r) dd_store(dt + E::R1 * r * as_out, v[r]);
        }
    } else {
        if (t < E::R1) {
#pragma unroll
            for (int r = 0; r < E::R2; ++r) v[r] = dd_load(st + E::R1 * r * as_in);
        }
        E::template inv<true>(v, xb + c * E::S, t, swt);
        if (t < E::R2 && cok) {
            const bool half = 2 * n_store == L;
#pragma unroll
            for (int s = 0; s < E::R1; ++s)
                if (half ? E::R2 * s < L / 2 : t + E::R2 * s < n_store) dd_store(dt + E::R2 * s * as_out, v[s]);
        }
    }
}

// Two-for-one real split in double-FP32: Z = FFT(a + i b), Y = Z(L - k):
// A = (Z + conj Y)/2, B = (Z - conj Y)/(2i) (the halving is exact)
__device__ __forceinline__ void dd_split_pair(ddc Z, ddc Y, ddc& xa, ddc& xb) {
    const ddc cy{make_float2(Y.h.x, -Y.h.y), make_float2(Y.l.x, -Y.l.y)};
    const ddc sm = dd_add(Z, cy), df = dd_sub(Z, cy);
    const float2 hf = make_float2(0.5f, 0.5f);
    xa = ddc{__fmul2_rn(sm.h, hf), __fmul2_rn(sm.l, hf)};
    // (Z - conj Y)/(2i) = -i (Z - conj Y)/2
    xb = ddc{make_float2(0.5f * df.h.y, -0.5f * df.h.x), make_float2(0.5f * df.l.y, -0.5f * df.l.x)};
}

// Forward x: two real FP64 rows per complex transform (split with integer
// operations) -> their double-FP32 half spectra, Hx = L/2 + 1 per row.  The
// FP32 fwd_x_body's layout: P row pairs per CTA.
template <int L>
__global__ void __launch_bounds__(256, 1) k2_dd_fwd_x(const double* __restrict__ rho, ddc* __restrict__ A, int nx,
                                                     int rows, int Hx, const ddc* __restrict__ tw) {
    using E = F2<L>;
    __shared__ ddc swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    ddc* xb = reinterpret_cast<ddc*>(smraw);
    constexpr int P = 256 / E::NT;
    const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
    const int r0 = 2 * (blockIdx.x * P + p), r1 = r0 + 1;
    ddc* col = xb + p * E::S;
    ddc v[16];
    const bool half = 2 * nx == L && 2 * (Hx - 1) == L;
    if (t < E::R2) {
        const double* ra = rho + (int64_t)r0 * nx + t;
        const double* rb = ra + nx;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            ddc z{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            if (half ? E::R2 * s < L / 2 : t + E::R2 * s < nx) {
                if (r0 < rows) dd_split(ra[E::R2 * s], z.h.x, z.l.x);
                if (r1 < rows) dd_split(rb[E::R2 * s], z.h.y, z.l.y);
            }
            v[s] = z;
        }
    }
    E::template fwd<false>(v, col, t, swt);
    if (t < E::R1) {
#pragma unroll
        for (int r = 0; r < E::R2; ++r) col[t + xoff(E::R1 * r)] = v[r];
    }
    __syncthreads();
    if (r0 < rows) {
        constexpr int NT = E::NT;
        const int tm = t == 0 ? 0 : NT - t;  // the mirror L - k = tm + constant
        ddc* Aa = A + (int64_t)r0 * Hx + t;
        ddc* Ab = Aa + Hx;
#pragma unroll
        for (int i = 0; i <= L / (2 * NT); ++i) {
            if (i == L / (2 * NT) && t > 0) break;  // k = t + NT*i <= L/2
            const int km = t == 0 ? xoff((L - NT * i) & (L - 1)) : tm + xoff(L - NT * (i + 1));
            ddc xa, xbv;
            dd_split_pair(col[t + xoff(NT * i)], col[km], xa, xbv);
            Aa[NT * i] = xa;
            if (r1 < rows) Ab[NT * i] = xbv;
        }
    }
}

// Inverse x of the three components into packed FP64 nodes {Ex, Ey, Ez, 0}:
// rows r0 = 2p, r1 = 2p + 1 (p a row pair) go through one complex transform
// as Xa + i Xb, the Hermitian half-spectra (Hx = L/2 + 1 stored) extended by
// conjugation; the real part is row r0, the imaginary part row r1.  As the
// FP32 k2_inv_x: components 0 and 1 wait in shared memory for the node
// store.  HALF: Hx = L/2 + 1 and nx = L/2.
template <int L, bool HALF>
__global__ void __launch_bounds__(256, 1) k2_dd_inv_x(const ddc* __restrict__ D, dnode4* __restrict__ E4, int nx,
                                                     int rows, int Hx, int64_t cs, const ddc* __restrict__ tw) {
    using E = F2<L>;
    __shared__ ddc swt[L];
    stage_twiddles<L>(swt, tw);
    constexpr int P = 256 / E::NT;
    extern __shared__ __align__(16) unsigned char smraw[];
    ddc* xb = reinterpret_cast<ddc*>(smraw);
    ddc* keep = xb + P * E::S;  // [2][P][nx]
    const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
    const int r0 = 2 * (blockIdx.x * P + p), r1 = r0 + 1;
    ddc* col = xb + p * E::S;
    ddc v[16];
    const ddc zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    for (int comp = 0; comp < 3; ++comp) {
        const ddc* Dc = D + comp * cs;
        if (t < E::R1) {
            const ddc* Da = Dc + (int64_t)r0 * Hx;
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
        E::template inv<true>(v, col, t, swt);
        if (comp < 2 && t < E::R2) {
            ddc* kp = keep + (int64_t)(comp * P + p) * nx + t;
#pragma unroll
            for (int s = 0; s < E::R1; ++s)
                if (HALF ? E::R2 * s < L / 2 : t + E::R2 * s < nx) kp[E::R2 * s] = v[s];
        }
    }
    __syncthreads();
    if (t < E::R2) {
        const ddc* k0 = keep + (int64_t)p * nx + t;
        const ddc* k1 = keep + (int64_t)(P + p) * nx + t;
        dnode4* o0 = E4 + (int64_t)r0 * nx + t;
        dnode4* o1 = o0 + nx;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            if (!(HALF ? E::R2 * s < L / 2 : t + E::R2 * s < nx)) continue;
            const double2 ex = dd_to(k0[E::R2 * s]), ey = dd_to(k1[E::R2 * s]), ez = dd_to(v[s]);
            if (r0 < rows) st4<double>(o0 + E::R2 * s, dnode4{ex.x, ey.x, ez.x, 0.0});
            if (r1 < rows) st4<double>(o1 + E::R2 * s, dnode4{ex.y, ey.y, ez.y, 0.0});
        }
    }
}


template <bool INV, typename TI, typename TO>
bool launch2_dd_col(int logL, const TI* in, TO* out, int ncols, int nbatch, int ncomp, int n_valid, int n_store,
                    int64_t as_in, int64_t bs_in, int64_t cs_in, int64_t as_out, int64_t bs_out, int64_t cs_out,
                    const ddc* tw, cudaStream_t s) {
#define SC_KDC(LL)                                                                                          \
    {                                                                                                       \
        const size_t smem = sizeof(ddc) * kColW * F2<LL>::S;                                                \
        if (set_smem(k2_dd_col<LL, INV, TI, TO>, smem) != SC_OK) return false;                              \
        const dim3 grid((unsigned)(((int64_t)ncols * nbatch + kColW - 1) / kColW), ncomp);                  \
        launch_pdl(k2_dd_col<LL, INV, TI, TO>, grid, kColW * F2<LL>::NT, smem, s, in, out, ncols, nbatch,    \
                   n_valid, n_store, as_in, bs_in, cs_in, as_out, bs_out, cs_out, tw);                      \
    }
    SC_L_SWITCH(logL, SC_KDC)
#undef SC_KDC
    return true;
}
#define SC_DD_COL(INV, TI, TO)                                                                              \
    template bool launch2_dd_col<INV, TI, TO>(int, const TI*, TO*, int, int, int, int, int, int64_t, int64_t, \
                                              int64_t, int64_t, int64_t, int64_t, const ddc*, cudaStream_t);
SC_DD_COL(false, ddc, ddc)
SC_DD_COL(false, ddc, double2)
SC_DD_COL(true, ddc, ddc)
SC_DD_COL(true, double2, ddc)
#undef SC_DD_COL

bool launch2_dd_fwd_x(int logL, const double* rho, ddc* A, int nx, int rows, int Hx, const ddc* tw, cudaStream_t s) {
#define SC_KDF(LL)                                                                                          \
    {                                                                                                       \
        constexpr int P = 256 / F2<LL>::NT;                                                                 \
        const size_t smem = sizeof(ddc) * P * F2<LL>::S;                                                    \
        if (set_smem(k2_dd_fwd_x<LL>, smem) != SC_OK) return false;                                         \
        const int pairs = (rows + 1) / 2;                                                                   \
        launch_pdl(k2_dd_fwd_x<LL>, (pairs + P - 1) / P, 256, smem, s, rho, A, nx, rows, Hx, tw);           \
    }
    SC_L_SWITCH(logL, SC_KDF)
#undef SC_KDF
    return true;
}

bool launch2_dd_inv_x(int logL, const ddc* D, dnode4* E4, int nx, int rows, int Hx, int64_t cs, const ddc* tw,
                      cudaStream_t s) {
#define SC_KDX(LL)                                                                                          \
    {                                                                                                       \
        constexpr int P = 256 / F2<LL>::NT;                                                                 \
        const size_t smem = sizeof(ddc) * ((size_t)P * F2<LL>::S + (size_t)2 * P * nx);                     \
        const int pairs = (rows + 1) / 2;                                                                   \
        if (2 * nx == LL && 2 * (Hx - 1) == LL) {                                                           \
            if (set_smem(k2_dd_inv_x<LL, true>, smem) != SC_OK) return false;                               \
            launch_pdl(k2_dd_inv_x<LL, true>, (pairs + P - 1) / P, 256, smem, s, D, E4, nx, rows, Hx, cs, tw); \
        } else {                                                                                            \
            if (set_smem(k2_dd_inv_x<LL, false>, smem) != SC_OK) return false;                              \
            launch_pdl(k2_dd_inv_x<LL, false>, (pairs + P - 1) / P, 256, smem, s, D, E4, nx, rows, Hx, cs, tw); \
        }                                                                                                   \
    }
    SC_L_SWITCH(logL, SC_KDX)
#undef SC_KDX
    return true;
}

}  // namespace sc
