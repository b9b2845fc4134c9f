// FP32 pass kernels on the register-resident two-step FFT (fft2.cuh), for
// transform lengths 4..256; the Stockham kernels of pipeline.cuh remain for
// FP64 and for longer transforms.
//
// Column passes (y, z: columns are consecutive kx, contiguous in memory) map
// threads column-fastest, tid = c + W*t, W = 16 columns per CTA; row passes
// (x: rows contiguous) map tid = t + NT*p over P row pairs.
#pragma once

#include "fft2.cuh"
#include "pipeline.cuh"
#include "zstage.cuh"

namespace sc {

// CTAs per SM the register allocation of the z passes and the column passes
// is sized for (the z pass's two shared buffers, 70 KB at L = 256, allow 3)
#ifndef SC_ZPASS_MINB
#define SC_ZPASS_MINB 2
#endif
#ifndef SC_COL_MINB
#define SC_COL_MINB 1
#endif

// Batched strided column FFT.  Forward (INV = false): inputs n < n_valid
// (natural order, zero beyond; with `wrap` also n > L - n_valid), all L
// outputs.  Inverse: all L inputs, outputs n < n_store.  Element
// (col, n, batch, comp) at base + col + n*as + b*bs + comp*cs, where b is the
// batch index, or wrap_row(batch, bwrap_n, bwrap_L) when bwrap_n > 0.  In and
// out may alias (each CTA reads all of its columns before writing them).
__device__ __forceinline__ int wrap_row2(int c, int n, int L) { return c < n ? c : L - (2 * n - 1) + c; }

// Body of one CTA: column tile `tile` of component `comp`; xb holds kColW
// exchange columns.
template <int L, bool INV>
__device__ __forceinline__ void col_body(const float2* in, float2* out, int ncols, int nbatch, int n_valid,
                                         int n_store, int wrap, int bwrap_n, int bwrap_L, int64_t as_in,
                                         int64_t bs_in, int64_t cs_in, int64_t as_out, int64_t bs_out,
                                         int64_t cs_out, int64_t tile, int comp, const float2* swt, float2* xb) {
    using E = F2<L>;
    // columns of all batches flattened: f = col + ncols * batch (a tile may
    // straddle two batches: two contiguous segments)
    const int c = threadIdx.x % kColW, t = threadIdx.x / kColW;
    const int64_t f = tile * kColW + c;
    const int64_t total = (int64_t)ncols * nbatch;
    const bool cok = f < total;
    // columns past the end (the last tile only) read the last column and store nothing
    const int64_t fl = cok ? f : total - 1;
    const int bb = total < (int64_t)1 << 31 ? (int)((unsigned)fl / (unsigned)ncols) : (int)(fl / ncols);
    const int col = (int)(fl - (int64_t)bb * ncols);
    const int b = bwrap_n > 0 ? wrap_row2(bb, bwrap_n, bwrap_L) : bb;
    const float2* src = in + b * bs_in + comp * cs_in + col;
    float2* dst = out + b * bs_out + comp * cs_out + col;
    float2 v[16];
    if (!INV) {
        // n_valid = L/2 without wrap (power-of-two axes): sample s exists for R2*s < L/2
        const bool half = 2 * n_valid == L && !wrap;
        if (t < E::R2) {
            const float2* st = src + t * as_in;
#pragma unroll
            for (int s = 0; s < E::R1; ++s) {
                const int n = t + E::R2 * s;
                const bool ok = half ? E::R2 * s < L / 2 : (n < n_valid || (wrap && n > L - n_valid));
                v[s] = ok ? st[E::R2 * s * as_in] : make_float2(0.f, 0.f);
            }
        }
        E::template fwd<false>(v, xb + c * E::S, t, swt);
        if (t < E::R1 && cok) {
            float2* dt = dst + t * as_out;
#pragma unroll
            for (int r = 0; r < E::R2; ++r) dt[E::R1 * r * as_out] = v[r];
        }
    } else {
        if (t < E::R1) {
            const float2* st = src + t * as_in;
#pragma unroll
            for (int r = 0; r < E::R2; ++r) v[r] = st[E::R1 * r * as_in];
        }
        E::template inv<true>(v, xb + c * E::S, t, swt);
        if (t < E::R2 && cok) {
            const bool half = 2 * n_store == L;
            float2* dt = dst + t * as_out;
#pragma unroll
            for (int s = 0; s < E::R1; ++s)
                if (half ? E::R2 * s < L / 2 : t + E::R2 * s < n_store) dt[E::R2 * s * as_out] = v[s];
        }
    }
}

template <int L, bool INV>
__global__ void __launch_bounds__(kColW * F2<L>::NT, SC_COL_MINB) k2_col(const float2* in, float2* out, int ncols, int nbatch,
                                                            int n_valid, int n_store, int wrap, int bwrap_n, int bwrap_L,
                                                            int64_t as_in, int64_t bs_in, int64_t cs_in,
                                                            int64_t as_out, int64_t bs_out, int64_t cs_out,
                                                            const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    stage_twiddles<L>(swt, tw);
    __shared__ float2 xb[kColW * F2<L>::S];
    col_body<L, INV>(in, out, ncols, nbatch, n_valid, n_store, wrap, bwrap_n, bwrap_L, as_in, bs_in, cs_in, as_out,
                     bs_out, cs_out, blockIdx.x, blockIdx.y, swt, xb);
}

// Inverse y and x fused, one CTA per (z plane, component), Lx = Ly = L: the
// plane's Hx columns are inverse-transformed along y (the outputs y < ny stay
// in shared memory), then its rows, two per complex IFFT, along x into the
// component's lane of the packed float4 nodes.  Replaces inverse y + inverse
// x when the plane fits in shared memory; the intermediate D never goes to
// global memory.
// Body of one CTA: Cp is the (component, z plane) of C, `out` the plane's
// first node lane to write (stride 4 floats per node).
template <int L, bool HALF>
__device__ __forceinline__ void inv_yx_body(const float2* __restrict__ Cp, float* __restrict__ out, int nx, int ny,
                                            int Hx_, const float2* swt, unsigned char* smraw) {
    using E = F2<L>;
    constexpr int W = 256 / E::NT;  // columns (phase 1) or row pairs (phase 2) per round
    // HALF: nx = ny = L/2 and Hx = L/2 + 1 (power-of-two planes), so the
    // strides and which samples exist are compile-time constants
    const int Hx = HALF ? L / 2 + 1 : Hx_;
    float2* xb = reinterpret_cast<float2*>(smraw);  // W exchange columns
    float2* ds = xb + W * E::S;                     // [ny][Hx]: the plane after inverse y
    float2 v[16];
    // phase 1: inverse y of the Hx columns: rounds of W whole columns
    // (column-fastest thread map, coalesced loads), then the Hx mod W left
    // over (the Nyquist column of a power-of-two plane) with NT consecutive
    // threads per column, so that warps holding none of them skip the math
    const int full = Hx - Hx % W;
    {
        const int c = threadIdx.x % W, t = threadIdx.x / W;
        float2* col = xb + c * E::S;
        for (int k0 = 0; k0 < full; k0 += W) {
            const int kx = k0 + c;
            if (t < E::R1) {
                const float2* Ct = Cp + kx + (int64_t)Hx * t;
#pragma unroll
                for (int r = 0; r < E::R2; ++r) v[r] = Ct[(int64_t)Hx * E::R1 * r];
            }
            E::template inv<true>(v, col, t, swt);
            if (t < E::R2) {
                float2* dt = ds + t * Hx + kx;
#pragma unroll
                for (int s = 0; s < E::R1; ++s)
                    if (HALF ? E::R2 * s < L / 2 : t + E::R2 * s < ny) dt[E::R2 * s * Hx] = v[s];
            }
        }
    }
    if (full < Hx) {
        const int c = threadIdx.x / E::NT, t = threadIdx.x % E::NT;
        const int kx = full + c;
        const bool ok = kx < Hx;
        const bool busy = full + (int)((threadIdx.x & ~31u) / E::NT) < Hx;  // uniform per warp
        float2* col = xb + c * E::S;
        if (busy && t < E::R1) {
#pragma unroll
            for (int r = 0; r < E::R2; ++r) v[r] = ok ? Cp[kx + (int64_t)Hx * (t + E::R1 * r)] : make_float2(0.f, 0.f);
        }
        E::template inv<true>(v, col, t, swt, busy);
        if (t < E::R2 && ok) {
#pragma unroll
            for (int s = 0; s < E::R1; ++s) {
                const int y = t + E::R2 * s;
                if (HALF ? E::R2 * s < L / 2 : y < ny) ds[y * Hx + kx] = v[s];
            }
        }
    }
    __syncthreads();
    // phase 2: inverse x of the rows, two per complex IFFT (row-pair-fastest map)
    {
        const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
        float2* col = xb + p * E::S;
        for (int q0 = 0; q0 < (ny + 1) / 2; q0 += W) {
            const int y0 = 2 * (q0 + p), y1 = y0 + 1;
            if (t < E::R1) {
                const float2* da = ds + y0 * Hx;
                const float2* db = da + Hx;
#pragma unroll
                for (int r = 0; r < E::R2; ++r) {
                    const int k = t + E::R1 * r;
                    // HALF: k below L/2 for R1*r < L/2, above for R1*r >
                    // L/2, and L/2 + t at R1*r = L/2
                    const bool cj = HALF ? (E::R1 * r > L / 2 || (E::R1 * r == L / 2 && t > 0)) : k > L / 2;
                    const int kk = HALF ? (E::R1 * r < L / 2 ? t + E::R1 * r : (cj ? L - t - E::R1 * r : L / 2))
                                        : (cj ? L - k : k);
                    float2 xa = make_float2(0.f, 0.f), xbv = make_float2(0.f, 0.f);
                    if (y0 < ny) xa = da[kk];
                    if (y1 < ny) xbv = db[kk];
                    if (cj) {
                        xa.y = -xa.y;
                        xbv.y = -xbv.y;
                    }
                    v[r] = make_float2(xa.x - xbv.y, xa.y + xbv.x);  // Xa + i Xb
                }
            }
            E::template inv<true>(v, col, t, swt);
            if (t < E::R2) {
                float* o0 = out + 4 * ((int64_t)nx * y0 + t);
#pragma unroll
                for (int s = 0; s < E::R1; ++s) {
                    if (!(HALF ? E::R2 * s < L / 2 : t + E::R2 * s < nx)) continue;
                    if (y0 < ny) o0[4 * E::R2 * s] = v[s].x;
                    if (y1 < ny) o0[4 * (E::R2 * s + nx)] = v[s].y;
                }
            }
        }
    }
}

// blockIdx.x = z plane; blockIdx.y = c reads component c of C and writes
// lane lane0 + c of the nodes (the adjoint's rhobar: one component into
// lane 3).
template <int L>
__global__ void __launch_bounds__(256) k2_inv_yx(const float2* __restrict__ C, float* __restrict__ E4, int nx,
                                                 int ny, int nz, int Hx, int lane0, const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    const int z = blockIdx.x, comp = blockIdx.y;
    const int64_t plane = (int64_t)Hx * L;
    float* o = E4 + lane0 + comp + 4 * (int64_t)nx * ny * z;
    if (2 * nx == L && 2 * ny == L && 2 * (Hx - 1) == L)
        inv_yx_body<L, true>(C + (int64_t)comp * plane * nz + plane * z, o, nx, ny, Hx, swt, smraw);
    else
        inv_yx_body<L, false>(C + (int64_t)comp * plane * nz + plane * z, o, nx, ny, Hx, swt, smraw);
}

// x pass: two real rows per complex FFT -> their half spectra.
// Body of one CTA: row pairs blk * P + ...; xb holds P exchange columns.
template <int L>
__device__ __forceinline__ void fwd_x_body(const float* __restrict__ rho, float2* __restrict__ A, int nx, int rows,
                                           int Hx, int blk, const float2* swt, float2* xb) {
    using E = F2<L>;
    constexpr int P = 256 / E::NT;  // row pairs per CTA
    const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
    const int r0 = 2 * (blk * P + p), r1 = r0 + 1;
    float2* col = xb + p * E::S;
    float2 v[16];
    // power-of-two rows (nx = L/2, Hx = L/2 + 1): sample s exists for
    // R2*s < L/2, and the output indices are constants past a per-thread base
    const bool half = 2 * nx == L && 2 * (Hx - 1) == L;
    if (t < E::R2) {
        const float* ra = rho + (int64_t)r0 * nx + t;
        const float* rb = ra + nx;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int x = t + E::R2 * s;
            float re = 0.f, im = 0.f;
            if (half ? E::R2 * s < L / 2 : x < nx) {
                if (r0 < rows) re = ra[E::R2 * s];
                if (r1 < rows) im = rb[E::R2 * s];
            }
            v[s] = make_float2(re, im);
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
        float2* Aa = A + (int64_t)r0 * Hx + t;
        float2* Ab = Aa + Hx;
#pragma unroll
        for (int i = 0; i <= L / (2 * NT); ++i) {
            if (i == L / (2 * NT) && t > 0) break;  // k = t + NT*i <= L/2
            const int km = t == 0 ? xoff((L - NT * i) & (L - 1)) : tm + xoff(L - NT * (i + 1));
            float2 xa, xbv;
            split_pair(col[t + xoff(NT * i)], col[km], xa, xbv);
            Aa[NT * i] = xa;
            if (r1 < rows) Ab[NT * i] = xbv;
        }
    }
}

template <int L>
__global__ void __launch_bounds__(256) k2_fwd_x(const float* __restrict__ rho, float2* __restrict__ A, int nx,
                                                int rows, int Hx, const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    stage_twiddles<L>(swt, tw);
    __shared__ float2 xb[(256 / F2<L>::NT) * F2<L>::S];
    fwd_x_body<L>(rho, A, nx, rows, Hx, blockIdx.x, swt, xb);
}

// Forward x and y fused, one CTA per z plane, Lx = Ly = L: the plane's rows,
// two per complex FFT, into their half spectra in shared memory (as
// k2_fwd_x), then the Hx columns along y (as the forward k2_col: inputs
// y < ny, all L outputs) into B[kx + Hx*(ky + L*z)].  Replaces those two
// passes when the plane fits in shared memory; the x pass's output never
// goes to global memory.
// Body of one CTA: rz is the z plane of rho (ny rows of nx), Bz the plane
// of B (L rows of Hx).
template <int L>
__device__ __forceinline__ void fwd_xy_body(const float* __restrict__ rz, float2* __restrict__ Bz, int nx, int ny,
                                            int Hx, const float2* swt, unsigned char* smraw) {
    using E = F2<L>;
    constexpr int W = 256 / E::NT;  // row pairs (x pass) or columns (y pass) per round
    float2* xb = reinterpret_cast<float2*>(smraw);  // W exchange columns
    float2* ds = xb + W * E::S;                     // [ny][Hx]: the plane after the x pass
    float2 v[16];
    // x pass: rows y0, y1 = y0 + 1 (row-pair-fastest thread map)
    {
        const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
        float2* col = xb + p * E::S;
        // power-of-two rows (nx = L/2, Hx = L/2 + 1): constant sample and output offsets
        const bool half = 2 * nx == L && 2 * (Hx - 1) == L;
        for (int q0 = 0; q0 < (ny + 1) / 2; q0 += W) {
            const int y0 = 2 * (q0 + p), y1 = y0 + 1;
            if (t < E::R2) {
                const float* ra = rz + (int64_t)y0 * nx + t;
                const float* rb = ra + nx;
#pragma unroll
                for (int s = 0; s < E::R1; ++s) {
                    const int x = t + E::R2 * s;
                    float re = 0.f, im = 0.f;
                    if (half ? E::R2 * s < L / 2 : x < nx) {
                        if (y0 < ny) re = ra[E::R2 * s];
                        if (y1 < ny) im = rb[E::R2 * s];
                    }
                    v[s] = make_float2(re, im);
                }
            }
            E::template fwd<false>(v, col, t, swt);
            if (t < E::R1) {
#pragma unroll
                for (int r = 0; r < E::R2; ++r) col[t + xoff(E::R1 * r)] = v[r];
            }
            __syncthreads();
            if (y0 < ny) {
                constexpr int NT = E::NT;
                const int tm = t == 0 ? 0 : NT - t;  // the mirror L - k = tm + constant
                float2* da = ds + y0 * Hx + t;
                float2* db = da + Hx;
#pragma unroll
                for (int i = 0; i <= L / (2 * NT); ++i) {
                    if (i == L / (2 * NT) && t > 0) break;  // k = t + NT*i <= L/2
                    const int km = t == 0 ? xoff((L - NT * i) & (L - 1)) : tm + xoff(L - NT * (i + 1));
                    float2 xa, xbv;
                    split_pair(col[t + xoff(NT * i)], col[km], xa, xbv);
                    da[NT * i] = xa;
                    if (y1 < ny) db[NT * i] = xbv;
                }
            }
            __syncthreads();
        }
    }
    // y pass: the Hx columns, zero beyond y = ny: rounds of W whole columns
    // (column-fastest thread map), then the Hx mod W left over (the Nyquist
    // column of a power-of-two plane) with NT consecutive threads per column,
    // so that warps holding none of them skip the math
    const int full = Hx - Hx % W;
    {
        const int c = threadIdx.x % W, t = threadIdx.x / W;
        float2* col = xb + c * E::S;
        const bool yhalf = 2 * ny == L;
        for (int k0 = 0; k0 < full; k0 += W) {
            const int kx = k0 + c;
            if (t < E::R2) {
                const float2* dt = ds + t * Hx + kx;
#pragma unroll
                for (int s = 0; s < E::R1; ++s) {
                    const int n = t + E::R2 * s;
                    v[s] = (yhalf ? E::R2 * s < L / 2 : n < ny) ? dt[E::R2 * s * Hx] : make_float2(0.f, 0.f);
                }
            }
            E::template fwd<false>(v, col, t, swt);
            if (t < E::R1) {
                float2* bt = Bz + kx + (int64_t)Hx * t;
#pragma unroll
                for (int r = 0; r < E::R2; ++r) bt[(int64_t)Hx * E::R1 * r] = v[r];
            }
        }
    }
    if (full < Hx) {
        const int c = threadIdx.x / E::NT, t = threadIdx.x % E::NT;
        const int kx = full + c;
        const bool ok = kx < Hx;
        const bool busy = full + (int)((threadIdx.x & ~31u) / E::NT) < Hx;  // uniform per warp
        float2* col = xb + c * E::S;
        if (busy && t < E::R2) {
#pragma unroll
            for (int s = 0; s < E::R1; ++s) {
                const int n = t + E::R2 * s;
                v[s] = (ok && n < ny) ? ds[n * Hx + kx] : make_float2(0.f, 0.f);
            }
        }
        E::template fwd<false>(v, col, t, swt, busy);
        if (t < E::R1 && ok) {
#pragma unroll
            for (int r = 0; r < E::R2; ++r) Bz[kx + (int64_t)Hx * (t + E::R1 * r)] = v[r];
        }
    }
}

// blockIdx.x = z plane; blockIdx.y selects a component: input rho + y *
// in_cs, output B + y * out_cs.
template <int L>
__global__ void __launch_bounds__(256) k2_fwd_xy(const float* __restrict__ rho, float2* __restrict__ B, int nx,
                                                 int ny, int Hx, int64_t in_cs, int64_t out_cs,
                                                 const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    const int z = blockIdx.x;
    fwd_xy_body<L>(rho + blockIdx.y * in_cs + (int64_t)nx * ny * z, B + blockIdx.y * out_cs + (int64_t)Hx * L * z,
                   nx, ny, Hx, swt, smraw);
}

// Inverse x pass of the three components, two rows per complex IFFT, packed
// float4 output nodes.
template <int L, bool HALF>
__global__ void __launch_bounds__(256) k2_inv_x(const float2* __restrict__ D, float4* __restrict__ E4, int nx,
                                                int rows, int Hx, int64_t cs, const float2* __restrict__ tw) {
    using E = F2<L>;
    __shared__ float2 swt[L];
    stage_twiddles<L>(swt, tw);
    constexpr int P = 256 / E::NT;
    extern __shared__ __align__(16) unsigned char smraw[];
    float2* xb = reinterpret_cast<float2*>(smraw);
    float2* keep = xb + P * E::S;  // [2][P][nx]: components 0, 1 until the float4 store
    const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
    const int r0 = 2 * (blockIdx.x * P + p), r1 = r0 + 1;
    float2* col = xb + p * E::S;
    float2 v[16];
    for (int comp = 0; comp < 3; ++comp) {
        const float2* Dc = D + comp * cs;
        if (t < E::R1) {
            const float2* Da = Dc + (int64_t)r0 * Hx;
            const float2* Db = Da + Hx;
#pragma unroll
            for (int r = 0; r < E::R2; ++r) {
                const int k = t + E::R1 * r;
                // HALF (Hx = L/2 + 1): k below L/2 for R1*r < L/2, above
                // for R1*r > L/2, and L/2 + t at R1*r = L/2
                const bool cj = HALF ? (E::R1 * r > L / 2 || (E::R1 * r == L / 2 && t > 0)) : k > L / 2;
                const int kk = HALF ? (E::R1 * r < L / 2 ? t + E::R1 * r : (cj ? L - t - E::R1 * r : L / 2))
                                    : (cj ? L - k : k);
                float2 xa = make_float2(0.f, 0.f), xbv = make_float2(0.f, 0.f);
                if (r0 < rows) xa = Da[kk];
                if (r1 < rows) xbv = Db[kk];
                if (cj) {
                    xa.y = -xa.y;
                    xbv.y = -xbv.y;
                }
                v[r] = make_float2(xa.x - xbv.y, xa.y + xbv.x);  // Xa + i Xb
            }
        }
        E::template inv<true>(v, col, t, swt);
        if (comp < 2) {
            if (t < E::R2) {
                float2* kp = keep + (int64_t)(comp * P + p) * nx + t;
#pragma unroll
                for (int s = 0; s < E::R1; ++s)
                    if (HALF ? E::R2 * s < L / 2 : t + E::R2 * s < nx) kp[E::R2 * s] = v[s];
            }
        }
    }
    __syncthreads();
    if (t < E::R2) {
        const float2* k0 = keep + (int64_t)p * nx + t;
        const float2* k1 = keep + (int64_t)(P + p) * nx + t;
        float4* o0 = E4 + (int64_t)r0 * nx + t;
        float4* o1 = o0 + nx;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            if (!(HALF ? E::R2 * s < L / 2 : t + E::R2 * s < nx)) continue;
            const float2 ex = k0[E::R2 * s], ey = k1[E::R2 * s], ez = v[s];
            if (r0 < rows) o0[E::R2 * s] = make_float4(ex.x, ey.x, ez.x, 0.f);
            if (r1 < rows) o1[E::R2 * s] = make_float4(ex.y, ey.y, ez.y, 0.f);
        }
    }
}

// Copies one component's half-stored image spectrum for this CTA's kColW
// columns, gim[kz][column] for kz <= L/2, to shared memory asynchronously
// (img_half layout; img_smem_at rebuilds kz > L/2).
template <int L>
__device__ __forceinline__ void prefetch_img(float2* gim, const GreenView& gv, int comp, int Hx, int Ly, int tile) {
    constexpr int HZ = L / 2 + 1;
    const int64_t plane = (int64_t)Hx * Ly;
    const int64_t gstep = (int64_t)gv.Hx * gv.Hy;
    const int cc = threadIdx.x % kColW;
    const int ff = tile * kColW + cc;
    if (ff < plane) {
        const int kyy = ff / Hx, kxx = ff - kyy * Hx;
        const int kyf = kyy <= Ly / 2 ? kyy : Ly - kyy;
        const float2* src = reinterpret_cast<const float2*>(gv.gimg) + comp * gv.cs_img + kxx + (int64_t)gv.Hx * kyf;
        for (int kz = threadIdx.x / kColW; kz < HZ; kz += blockDim.x / kColW)
            cp_async8(gim + kz * kColW + cc, src + gstep * kz);
    }
    cp_async_commit();
}

// img_at on the shared-memory copy of prefetch_img
template <int L>
__device__ __forceinline__ float2 img_smem_at(const float2* gim, int kz, int c, int comp) {
    if (kz <= L / 2) return gim[kz * kColW + c];
    float2 v = gim[(L - kz) * kColW + c];
    if (comp < 2)
        v.x = -v.x;
    else
        v.y = -v.y;
    return v;
}

// z pass: forward z transform of rho^(kx, ky, .), products with the three
// Green spectra (image: rho^ at -kz times the image spectrum), three inverse
// transforms, z < nz stored.  The tile's free-space Green values (3 x
// (L/2+1) x kColW floats) are copied to shared memory asynchronously at the
// start, so their L2 latency overlaps the forward transform.
// Body of one CTA: `tile` is the CTA's column tile (kColW consecutive
// columns of the flattened (kx, ky) plane).  HALF: nz = L/2 (every
// power-of-two axis), so which z rows exist is known at compile time.
// Columns past the plane (the last tile only) load the plane's last column
// and store nothing, so no branch inside the unrolled loops tests them.
template <int L, bool HALF>
__device__ __forceinline__ void zpass_body(const float2* __restrict__ B, float2* __restrict__ C, int Hx, int Ly,
                                           int nz, const GreenView& gv, int tile, const float2* swt,
                                           unsigned char* smraw) {
    using E = F2<L>;
    constexpr int RL = E::R1;
    float2* xb = reinterpret_cast<float2*>(smraw);
    float2* spec = xb + kColW * E::S;  // natural-order spectrum of this tile's columns
    constexpr int HZ = L / 2 + 1;
    float* gsm = reinterpret_cast<float*>(spec + kColW * E::S);  // [3][HZ][kColW]
    // image, half-stored: one component's spectrum at a time, [HZ][kColW],
    // the next one copied in during the current one's inverse transform
    float2* gim = reinterpret_cast<float2*>(gsm + 3 * HZ * kColW);
    const bool img_smem = gv.image && gv.img_half;
    // columns are the (kx, ky) plane flattened: f = kx + Hx*ky is contiguous
    const int c = threadIdx.x % kColW, t = threadIdx.x / kColW;
    const int64_t plane = (int64_t)Hx * Ly;
    prefetch_green<L>(gsm, gv, Hx, Ly, tile);
    if (img_smem) prefetch_img<L>(gim, gv, 0, Hx, Ly, tile);
    const int64_t gstep = (int64_t)gv.Hx * gv.Hy;
    const int f = tile * kColW + c;
    const bool cok = f < plane;
    const int fl = cok ? f : (int)plane - 1;
    const int ky = fl / Hx;
    const int kx = fl - ky * Hx;
    float2* col = xb + c * E::S;
    float2* sc = spec + c * E::S;
    float2 v[16];
    if (t < E::R2) {
        const float2* Bc = B + fl;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int z = t + E::R2 * s;
            if constexpr (HALF)
                v[s] = E::R2 * s < L / 2 ? Bc[plane * z] : make_float2(0.f, 0.f);
            else
                v[s] = z < nz ? Bc[plane * z] : make_float2(0.f, 0.f);
        }
    }
    E::template fwd<false>(v, col, t, swt);
    if (t < E::R1) {
#pragma unroll
        for (int r = 0; r < E::R2; ++r) sc[t + xoff(E::R1 * r)] = v[r];
    }
    cp_async_wait_all();
    __syncthreads();
    const int kyf = ky <= Ly / 2 ? ky : Ly - ky;
    const float ysign = ky <= Ly / 2 ? 1.f : -1.f;
    for (int comp = 0; comp < 3; ++comp) {
        if (img_smem && comp > 0) {
            cp_async_wait_all();
            __syncthreads();
        }
        if (t < E::R1) {
            // kz = t + RL*r: below L/2 for RL*r < L/2 (folded index kz), at
            // or above it otherwise (folded index L - kz).  Signs: component
            // 1 is odd along y, component 2 odd along z (kz > L/2).
            const float sy = comp == 1 ? ysign : 1.f;
            const float su = comp == 2 ? -sy : sy;
            const float sm = t > 0 ? su : sy;  // kz = L/2 + t
            const float* gfc = gsm + comp * HZ * kColW + c;
            const float* glo = gfc + t * kColW;
            const float* ghi = gfc + (L - t) * kColW;
            const float2* sct = sc + t;
            if (!gv.image) {
#pragma unroll
                for (int r = 0; r < E::R2; ++r) {
                    const float g = RL * r < L / 2    ? glo[RL * r * kColW] * sy
                                    : RL * r == L / 2 ? ghi[-RL * r * kColW] * sm
                                                      : ghi[-RL * r * kColW] * su;
                    const float2 X = sct[xoff(RL * r)];
                    v[r] = make_float2(-X.y * g, X.x * g);  // X * (i g)
                }
            } else {
                const float2* gic =
                    reinterpret_cast<const float2*>(gv.gimg) + comp * gv.cs_img + kx + gv.Hx * kyf;
#pragma unroll
                for (int r = 0; r < E::R2; ++r) {
                    const int kz = t + RL * r;
                    const float g = RL * r < L / 2    ? glo[RL * r * kColW] * sy
                                    : RL * r == L / 2 ? ghi[-RL * r * kColW] * sm
                                                      : ghi[-RL * r * kColW] * su;
                    const float2 X = sct[xoff(RL * r)];
                    float2 out = make_float2(-X.y * g, X.x * g);  // X * (i g)
                    float2 gc = img_smem ? img_smem_at<L>(gim, kz, c, comp) : img_at(gic, gstep, kz, gv, comp);
                    if (comp == 1) {
                        gc.x *= ysign;
                        gc.y *= ysign;
                    }
                    v[r] = cadd(out, cmul(sc[xsw((L - kz) & (L - 1))], gc));
                }
            }
        }
        if (img_smem && comp < 2) {
            __syncthreads();  // every thread is done with this component's copy
            prefetch_img<L>(gim, gv, comp + 1, Hx, Ly, tile);
        }
        E::template inv<true>(v, col, t, swt);
        if (t < E::R2 && cok) {
            float2* Cc = C + comp * (plane * nz) + f;
#pragma unroll
            for (int s = 0; s < E::R1; ++s) {
                const int z = t + E::R2 * s;
                if (HALF ? E::R2 * s < L / 2 : z < nz) Cc[plane * z] = v[s];
            }
        }
    }
}

template <int L, bool HALF>
__global__ void __launch_bounds__(kColW * F2<L>::NT, SC_ZPASS_MINB) k2_zpass(const float2* __restrict__ B,
                                                                 float2* __restrict__ C, int Hx, int Ly, int nz,
                                                                 GreenView gv, const float2* __restrict__ tw) {
    __shared__ float2 swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    zpass_body<L, HALF>(B, C, Hx, Ly, nz, gv, blockIdx.x, swt, smraw);
}

// Adjoint z pass: three forward z transforms of Ebar_c, correlation with the
// conjugate Green spectra summed over components, one inverse transform.
template <int L, bool HALF>
__global__ void __launch_bounds__(kColW * F2<L>::NT, SC_ZPASS_MINB) k2_adj_zpass(const float2* __restrict__ C,
                                                                     float2* __restrict__ B, int Hx, int Ly, int nz,
                                                                     GreenView gv, const float2* __restrict__ tw) {
    // HALF: nz = L/2, so which z rows exist is known at compile time; the
    // free-space Green values and signs at constant offsets as in zpass_body
    using E = F2<L>;
    constexpr int RL = E::R1;
    __shared__ float2 swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    float2* xb = reinterpret_cast<float2*>(smraw);
    float2* spec = xb + kColW * E::S;
    const int c = threadIdx.x % kColW, t = threadIdx.x / kColW;
    const int64_t plane = (int64_t)Hx * Ly;
    const int f = blockIdx.x * kColW + c;
    const bool cok = f < plane;
    const int fl = cok ? f : (int)plane - 1;  // columns past the plane load the last one, store nothing
    const int ky = fl / Hx;
    const int kx = fl - ky * Hx;
    float2* col = xb + c * E::S;
    float2* sc = spec + c * E::S;
    constexpr int HZ = L / 2 + 1;
    float* gsm = reinterpret_cast<float*>(spec + kColW * E::S);  // [3][HZ][kColW]
    prefetch_green<L>(gsm, gv, Hx, Ly, blockIdx.x);
    const int kyf = ky <= Ly / 2 ? ky : Ly - ky;
    const float ysign = ky <= Ly / 2 ? 1.f : -1.f;
    const int64_t gstep = (int64_t)gv.Hx * gv.Hy;
    float2 acc[16], v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) acc[r] = make_float2(0.f, 0.f);
    for (int comp = 0; comp < 3; ++comp) {
        const float2* Cc = C + comp * (plane * nz) + fl;
        if (t < E::R2) {
#pragma unroll
            for (int s = 0; s < E::R1; ++s) {
                const int z = t + E::R2 * s;
                const bool ok = HALF ? E::R2 * s < L / 2 : z < nz;
                v[s] = ok ? Cc[plane * z] : make_float2(0.f, 0.f);
            }
        }
        E::template fwd<false>(v, col, t, swt);
        if (gv.image) {
            if (t < E::R1) {
#pragma unroll
                for (int r = 0; r < E::R2; ++r) sc[t + xoff(E::R1 * r)] = v[r];
            }
        }
        if (comp == 0) cp_async_wait_all();
        if (gv.image || comp == 0) __syncthreads();
        if (t < E::R1) {
            const float sy = comp == 1 ? ysign : 1.f;
            const float su = comp == 2 ? -sy : sy;
            const float sm = t > 0 ? su : sy;  // kz = L/2 + t
            const float* gfc = gsm + comp * HZ * kColW + c;
            const float* glo = gfc + t * kColW;
            const float* ghi = gfc + (L - t) * kColW;
            const float2* gic = reinterpret_cast<const float2*>(gv.gimg) + comp * gv.cs_img + kx + gv.Hx * kyf;
#pragma unroll
            for (int r = 0; r < E::R2; ++r) {
                const int kz = t + RL * r;
                const float g = RL * r < L / 2    ? glo[RL * r * kColW] * sy
                                : RL * r == L / 2 ? ghi[-RL * r * kColW] * sm
                                                  : ghi[-RL * r * kColW] * su;
                // Ebar^ * conj(i g) = Ebar^ * (-i g)
                acc[r].x += v[r].y * g;
                acc[r].y -= v[r].x * g;
                if (gv.image) {
                    const int kzm = (L - kz) & (L - 1);
                    float2 gc = img_at(gic, gstep, kzm, gv, comp);
                    if (comp == 1) {
                        gc.x *= ysign;
                        gc.y *= ysign;
                    }
                    acc[r] = cadd(acc[r], cmulc(sc[xsw(kzm)], gc));
                }
            }
        }
        if (gv.image) __syncthreads();  // spec is rewritten by the next component
    }
    E::template inv<true>(acc, col, t, swt);
    if (t < E::R2 && cok) {
        float2* Bc = B + f;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int z = t + E::R2 * s;
            if (HALF ? E::R2 * s < L / 2 : z < nz) Bc[plane * z] = acc[s];
        }
    }
}

// Adjoint inverse x pass of one component into the fourth lane of the
// packed nodes (rhobar).
template <int L>
__global__ void __launch_bounds__(256) k2_inv_x1(const float2* __restrict__ D, float* __restrict__ E4, int nx,
                                                 int rows, int Hx, const float2* __restrict__ tw) {
    using E = F2<L>;
    __shared__ float2 swt[L];
    stage_twiddles<L>(swt, tw);
    constexpr int P = 256 / E::NT;
    __shared__ float2 xb[P * E::S];
    const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
    const int r0 = 2 * (blockIdx.x * P + p), r1 = r0 + 1;
    float2 v[16];
    if (t < E::R1) {
#pragma unroll
        for (int r = 0; r < E::R2; ++r) {
            const int k = t + E::R1 * r;
            const bool cj = k > L / 2;
            const int kk = cj ? L - k : k;
            float2 xa = make_float2(0.f, 0.f), xbv = make_float2(0.f, 0.f);
            if (r0 < rows) xa = D[(int64_t)r0 * Hx + kk];
            if (r1 < rows) xbv = D[(int64_t)r1 * Hx + kk];
            if (cj) {
                xa.y = -xa.y;
                xbv.y = -xbv.y;
            }
            v[r] = make_float2(xa.x - xbv.y, xa.y + xbv.x);
        }
    }
    E::template inv<true>(v, xb + p * E::S, t, swt);
    if (t < E::R2) {
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int x = t + E::R2 * s;
            if (x >= nx) continue;
            if (r0 < rows) E4[4 * ((int64_t)r0 * nx + x) + 3] = v[s].x;
            if (r1 < rows) E4[4 * ((int64_t)r1 * nx + x) + 3] = v[s].y;
        }
    }
}

// Green transform on the parity-reduced lattice.  Kernel component c is odd
// along x for c = 0 and along y for c = 1, even along the other of the two,
// and in free space odd along z for c = 2 and even otherwise.  The transform
// of a full line (2n-1 samples, d = -(n-1)..n-1) is then the transform of its
// d >= 0 half extended with that parity: real for an even line, imaginary for
// an odd one.  Each pass stores that one real part for k <= L/2, so the three
// passes read and write real arrays over the d >= 0 octant only, two lines per
// complex FFT.  With exactly one odd axis per free-space component, the last
// pass leaves Im(K^), the compressed spectrum.  The image kernel has no parity
// in z: its z pass transforms the full line and forms the complex spectrum.
//
// The kernels run in FP32 (the mixed pipeline) or FP64 (the FP64 pipeline),
// Tr the real type.  Their exchange columns are in dynamic shared memory.
//
// x pass: rows r = ay + ny*iz of the stored octant G (iz = |dz| in free space,
// dz + nz - 1 for the image), out T[comp][r][kx], kx <= L/2.
// odd_x: the component that is odd along x (0 for the field; -1 for the
// potential kernel, which is even along every axis).
template <int L, typename Tr>
__global__ void __launch_bounds__(256) k3_green_x(const Tr* __restrict__ G, Tr* __restrict__ T, int nx,
                                                  int rows, int Hx, int64_t gcs, int64_t tcs, int odd_x,
                                                  const typename Cplx<Tr>::T2* __restrict__ tw) {
    using E = F2<L>;
    using T2 = typename Cplx<Tr>::T2;
    __shared__ T2 swt[L];
    stage_twiddles<L>(swt, tw);
    constexpr int P = 256 / E::NT;
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* xb = reinterpret_cast<T2*>(smraw);  // P exchange columns
    const int comp = blockIdx.y;
    const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
    const int r0 = 2 * (blockIdx.x * P + p), r1 = r0 + 1;
    const bool ok0 = r0 < rows, ok1 = r1 < rows;
    const Tr* g0 = G + comp * gcs + (int64_t)nx * r0;
    const Tr* g1 = g0 + nx;
    T2* col = xb + p * E::S;
    T2 v[16];
    if (t < E::R2) {
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int x = t + E::R2 * s;
            const int dx = x < nx ? x : (x > L - nx ? x - L : L);
            Tr a = 0, b = 0;
            if (dx != L) {
                const int ax = dx < 0 ? -dx : dx;
                if (ok0) a = __ldg(g0 + ax);
                if (ok1) b = __ldg(g1 + ax);
                if (comp == odd_x && dx < 0) a = -a, b = -b;
            }
            v[s] = Cplx<Tr>::make(a, b);
        }
    }
    E::template fwd<false>(v, col, t, swt);
    if (t < E::R1) {
#pragma unroll
        for (int r = 0; r < E::R2; ++r) col[t + xoff(E::R1 * r)] = v[r];
    }
    __syncthreads();
    if (ok0) {
        Tr* T0 = T + comp * tcs + (int64_t)Hx * r0;
        for (int k = t; k <= L / 2; k += E::NT) {
            T2 xa, xbv;
            split_pair(col[xsw(k)], col[xsw((L - k) & (L - 1))], xa, xbv);
            T0[k] = comp == odd_x ? xa.y : xa.x;
            if (ok1) T0[Hx + k] = comp == odd_x ? xbv.y : xbv.x;
        }
    }
}

// y or z pass of the parity-reduced Green transform: real lines along a
// strided axis, 2*kColW lines per CTA (line f and f + kColW share one complex
// FFT).  Line (col, b): input sample d >= 0 at in + b*bs_in + col + d*as_in,
// d < nh; with `odd_comp` == comp the extension is odd.  IMG (image z pass):
// the input holds the full line, d + nh - 1 for d = -(nh-1)..nh-1, and the
// output is the complex image spectrum -i^p X(kz) e^{-2 pi i kz (nh-1)/L}
// for kz <= L/2 (p = 1 for components 0 and 1; img_at gives the other kz
// from these); otherwise k <= L/2 of the kept
// real part is stored at out + b*bs_out + col + k*as_out.
// imask (image z pass): bit c set when component c was stored as the
// imaginary part along an odd axis, so its spectrum takes a factor i (3 for
// the field's x and y components; 0 for the potential).
template <int L, bool IMG, typename Tr>
__global__ void __launch_bounds__(kColW * F2<L>::NT, SC_COL_MINB) k3_green_col(const Tr* __restrict__ in, void* __restrict__ out,
                                                                  int ncols, int nbatch, int nh, int odd_comp,
                                                                  int64_t as_in, int64_t bs_in, int64_t cs_in,
                                                                  int64_t as_out, int64_t bs_out, int64_t cs_out,
                                                                  int imask,
                                                                  const typename Cplx<Tr>::T2* __restrict__ tw) {
    using E = F2<L>;
    using T2 = typename Cplx<Tr>::T2;
    __shared__ T2 swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* xb = reinterpret_cast<T2*>(smraw);  // kColW exchange columns
    const int c = threadIdx.x % kColW, t = threadIdx.x / kColW;
    const int comp = blockIdx.y;
    const int64_t total = (int64_t)ncols * nbatch;
    const int64_t fa = (int64_t)blockIdx.x * (2 * kColW) + c, fb = fa + kColW;
    const bool oka = fa < total, okb = fb < total;
    const int ba = oka ? (int)(fa / ncols) : 0, bb = okb ? (int)(fb / ncols) : 0;
    const int ca = (int)(fa - (int64_t)ba * ncols), cb = (int)(fb - (int64_t)bb * ncols);
    const Tr* sa = in + comp * cs_in + ba * bs_in + ca;
    const Tr* sb = in + comp * cs_in + bb * bs_in + cb;
    const bool odd = comp == odd_comp;
    T2* col = xb + c * E::S;
    T2 v[16];
    if (2 * nh == L && t < E::R2) {
        // nh = L/2: sample n = t + R2*s is d = n below L/2, d = n - L above,
        // nothing at L/2; its offset a per-thread base plus R2*s*as_in
        const int64_t blo = (IMG ? t + nh - 1 : t) * as_in;
        const int64_t bhi = (IMG ? t - nh - 1 : L - t) * as_in;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const bool lower = E::R2 * s < L / 2;
            const bool here = lower || E::R2 * s > L / 2 || t > 0;
            const int64_t step = (int64_t)(E::R2 * s) * as_in;
            const int64_t o = lower ? blo + step : (IMG ? bhi + step : bhi - step);
            Tr a = 0, b = 0;
            if (here) {
                if (oka) a = __ldg(sa + o);
                if (okb) b = __ldg(sb + o);
                if (!IMG && odd && !lower) a = -a, b = -b;
            }
            v[s] = Cplx<Tr>::make(a, b);
        }
    } else if (t < E::R2) {
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int n = t + E::R2 * s;
            const int d = n < nh ? n : (n > L - nh ? n - L : L);
            Tr a = 0, b = 0;
            if (d != L) {
                const int64_t o = (IMG ? d + nh - 1 : (d < 0 ? -d : d)) * as_in;
                if (oka) a = __ldg(sa + o);
                if (okb) b = __ldg(sb + o);
                if (!IMG && odd && d < 0) a = -a, b = -b;
            }
            v[s] = Cplx<Tr>::make(a, b);
        }
    }
    E::template fwd<false>(v, col, t, swt);
    if (t < E::R1) {
#pragma unroll
        for (int r = 0; r < E::R2; ++r) col[t + xoff(E::R1 * r)] = v[r];
    }
    __syncthreads();
    for (int k = t; k <= L / 2; k += E::NT) {
        T2 xa, xbv;
        split_pair(col[xsw(k)], col[xsw((L - k) & (L - 1))], xa, xbv);
        if (!IMG) {
            Tr* o = reinterpret_cast<Tr*>(out) + comp * cs_out + k * as_out;
            if (oka) o[ba * bs_out + ca] = odd ? xa.y : xa.x;
            if (okb) o[bb * bs_out + cb] = odd ? xbv.y : xbv.x;
        } else {
            // the line is real, so X(L - k) = conj X(k): only k <= L/2 is
            // stored, and img_at rebuilds the rest
            const T2 ph1 = swt[(k * (nh - 1)) & (L - 1)];  // w_L^(k (nh - 1)), staged in shared memory
            T2* o = reinterpret_cast<T2*>(out) + comp * cs_out;
            for (int w = 0; w < 2; ++w) {
                const bool okw = w == 0 ? oka : okb;
                if (!okw) continue;
                const T2 x = w == 0 ? xa : xbv;
                const T2 x1 = ((imask >> comp) & 1) ? Cplx<Tr>::make(-x.y, x.x) : x;  // times i
                const int64_t base = w == 0 ? (ba * bs_out + ca) : (bb * bs_out + cb);
                const T2 q1 = cmul(x1, ph1);
                o[base + k * as_out] = Cplx<Tr>::make(-q1.x, -q1.y);
            }
        }
    }
}

// x and y passes of the Green transform fused, one CTA per (stored z slice,
// component), Lx = Ly = L: the slice's ny rows are transformed along x (two
// per complex FFT) into shared memory, then its Hx columns along y (two per
// complex FFT) with the component's y parity, into T2[comp][iz][ky][kx].
// The x-pass output (k3_green_x's T1) never goes to global memory.
// FP32: three CTAs per SM at 80 registers; FP64: one, its slice takes up to
// 202 KB of shared memory
// odd_x, odd_y: the components odd along x and y (0 and 1 for the field;
// -1 for the potential kernel)
template <int L, typename Tr>
__global__ void __launch_bounds__(256, sizeof(Tr) == 4 ? 3 : 1) k3_green_xy(const Tr* __restrict__ G, Tr* __restrict__ T2out, int nx,
                                                   int ny, int Hx, int64_t gcs, int64_t t2cs, int odd_x, int odd_y,
                                                   const typename Cplx<Tr>::T2* __restrict__ tw) {
    using E = F2<L>;
    using T2 = typename Cplx<Tr>::T2;
    constexpr int W = 256 / E::NT;  // row pairs (x pass) or columns (y pass) per round
    __shared__ T2 swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* xb = reinterpret_cast<T2*>(smraw);        // W exchange columns
    Tr* ts = reinterpret_cast<Tr*>(xb + W * E::S);  // [ny][Hx]: the slice after the x pass
    const int iz = blockIdx.x, comp = blockIdx.y;
    T2 v[16];
    // x pass: rows y0, y1 = y0 + 1 of slice iz; component 0 is odd along x
    {
        const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
        T2* col = xb + p * E::S;
        const Tr* gs = G + comp * gcs + (int64_t)nx * ny * iz;
        for (int q0 = 0; q0 < (ny + 1) / 2; q0 += W) {
            const int y0 = 2 * (q0 + p), y1 = y0 + 1;
            const bool ok0 = y0 < ny, ok1 = y1 < ny;
            const Tr* g0 = gs + (int64_t)nx * y0;
            const Tr* g1 = g0 + nx;
            if (t < E::R2) {
#pragma unroll
                for (int s = 0; s < E::R1; ++s) {
                    const int x = t + E::R2 * s;
                    const int dx = x < nx ? x : (x > L - nx ? x - L : L);
                    Tr a = 0, b = 0;
                    if (dx != L) {
                        const int ax = dx < 0 ? -dx : dx;
                        if (ok0) a = __ldg(g0 + ax);
                        if (ok1) b = __ldg(g1 + ax);
                        if (comp == odd_x && dx < 0) a = -a, b = -b;
                    }
                    v[s] = Cplx<Tr>::make(a, b);
                }
            }
            E::template fwd<false>(v, col, t, swt);
            if (t < E::R1) {
#pragma unroll
                for (int r = 0; r < E::R2; ++r) col[t + xoff(E::R1 * r)] = v[r];
            }
            __syncthreads();
            if (ok0) {
                for (int k = t; k <= L / 2; k += E::NT) {
                    T2 xa, xbv;
                    split_pair(col[xsw(k)], col[xsw((L - k) & (L - 1))], xa, xbv);
                    ts[y0 * Hx + k] = comp == odd_x ? xa.y : xa.x;
                    if (ok1) ts[y1 * Hx + k] = comp == odd_x ? xbv.y : xbv.x;
                }
            }
            __syncthreads();
        }
    }
    // y pass: columns fa, fb = fa + W of the slice; component 1 is odd along y.
    // Columns kx < L/2 go through the FFT two per round; the last one
    // (kx = L/2, which would take a round of its own) by a direct sum.
    {
        const int c = threadIdx.x % W, t = threadIdx.x / W;
        T2* col = xb + c * E::S;
        const bool odd = comp == odd_y;
        Tr* out = T2out + comp * t2cs + (int64_t)Hx * (L / 2 + 1) * iz;
        for (int k = threadIdx.x; k <= L / 2; k += blockDim.x) {
            // X(k) = sum_d x(d) w^(k d), d = -(ny-1)..ny-1, x(-d) = -x(d) when odd
            Tr re = 0, im = 0;
            for (int d = 0; d < ny; ++d) {
                const Tr a = ts[d * Hx + L / 2];
                const T2 wp = swt[(k * d) & (L - 1)];
                if (d == 0) {
                    re += a;
                } else if (odd) {
                    im += Tr(2) * a * wp.y;  // x(d) (w^kd - w^-kd) = 2i x(d) Im w^kd
                } else {
                    re += Tr(2) * a * wp.x;
                }
            }
            out[(int64_t)k * Hx + L / 2] = odd ? im : re;
        }
        for (int k0 = 0; k0 < L / 2; k0 += 2 * W) {
            const int fa = k0 + c, fb = fa + W;
            const bool oka = fa < L / 2, okb = fb < L / 2;
            if (t < E::R2) {
#pragma unroll
                for (int s = 0; s < E::R1; ++s) {
                    const int n = t + E::R2 * s;
                    const int d = n < ny ? n : (n > L - ny ? n - L : L);
                    Tr a = 0, b = 0;
                    if (d != L) {
                        const int ad = d < 0 ? -d : d;
                        if (oka) a = ts[ad * Hx + fa];
                        if (okb) b = ts[ad * Hx + fb];
                        if (odd && d < 0) a = -a, b = -b;
                    }
                    v[s] = Cplx<Tr>::make(a, b);
                }
            }
            E::template fwd<false>(v, col, t, swt);
            if (t < E::R1) {
#pragma unroll
                for (int r = 0; r < E::R2; ++r) col[t + xoff(E::R1 * r)] = v[r];
            }
            __syncthreads();
            for (int k = t; k <= L / 2; k += E::NT) {
                T2 xa, xbv;
                split_pair(col[xsw(k)], col[xsw((L - k) & (L - 1))], xa, xbv);
                if (oka) out[(int64_t)k * Hx + fa] = odd ? xa.y : xa.x;
                if (okb) out[(int64_t)k * Hx + fb] = odd ? xbv.y : xbv.x;
            }
            __syncthreads();
        }
    }
}

// Paired Green transform of the field kernel: four real lines per complex
// FFT.  An even real line has a real spectrum E, an odd one an imaginary
// spectrum i P; for z = e1 + i e2 + o1 + i o2 (e even, o odd),
//   Z(k) = (E1 - P2) + i (E2 + P1),  Z(L - k) = (E1 + P2) + i (E2 - P1),
// so E1, E2, P1, P2 follow from Z(k) and Z(L - k).  The field kernel's
// components have that mix: along x component 0 is odd and 1 even, along y
// component 1 odd and 0 even, along z (free space) component 2 odd and 0, 1
// even.  Pairing components 0 and 1 in the x and y passes and 0 and 2 in the
// z pass does their transforms with half the FFTs of k3_green_xy and
// k3_green_col; the remaining component runs through those kernels alone.
template <typename T2, typename Tr>
__device__ __forceinline__ void unpack4(T2 Zk, T2 Zm, Tr& e1, Tr& e2, Tr& p1, Tr& p2) {
    e1 = Tr(0.5f) * (c_re(Zk) + c_re(Zm));
    p2 = Tr(0.5f) * (c_re(Zm) - c_re(Zk));
    e2 = Tr(0.5f) * (c_im(Zk) + c_im(Zm));
    p1 = Tr(0.5f) * (c_im(Zk) - c_im(Zm));
}

// The FP32 Green build's near cells, for k4_green_xy to fill in: the FP64
// antiderivative terms T[term][comp][corner] on the corners of the near box
// (ix < nbx, iy < nby, bz0 <= dz < bz1), and what the near test and the
// 8-point difference need.  T null: no near cells to fill (the FP64 build).
struct GreenNear {
    const double* T;
    int nx, ny, nz, image;
    int nbx, nby, bz0, bz1;
    float ux, uy, uz, uoff, ratio;  // the cell test: |centre| / hmax < ratio
    double fxy, fz;                 // gamma / (dx dy dz), 1 / (dx dy dz)
    double scale;                   // FPEI / (Lx Ly Lz)
};

// Whether the stored cell (ix, iy, dz) takes the FP64 corner difference: the
// test the far-cell quadrature skipped it by (native.cu oct_cell).
__device__ __forceinline__ bool green_near_cell(const GreenNear& g, int ix, int iy, int dz) {
    const float px = (float)ix * g.ux, py = (float)iy * g.uy, pz = fmaf((float)dz, g.uz, g.uoff);
    const float r = sqrtf(fmaf(px, px, fmaf(py, py, pz * pz)));
    return r < g.ratio && ix < g.nbx && iy < g.nby && dz >= g.bz0 && dz < g.bz1;
}

// The 8-point difference (green_functions.jl:108-111) of near cell (ix, iy,
// dz), component c, from the corner terms F = (T0 - T1 + T2) * factor_c.
__device__ __forceinline__ float green_near_value(const GreenNear& g, int c, int ix, int iy, int dz) {
    const int cx = g.nbx + 1, cy = g.nby + 1, cz = g.bz1 - g.bz0 + 1;
    const int64_t per = (int64_t)cx * cy * cz;
    const int64_t sy = cx, sz = (int64_t)cx * cy;
    const double fc = c == 2 ? g.fz : g.fxy;
    const double* t0 = g.T + c * per + ix + sy * iy + sz * (dz - g.bz0);
    const double* t1 = t0 + 3 * per;
    const double* t2 = t1 + 3 * per;
    double F[8];  // corner (a, b, e) at a + 2b + 4e
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int64_t q = (k & 1) + sy * ((k >> 1) & 1) + sz * (k >> 2);
        F[k] = (__ldg(t0 + q) - __ldg(t1 + q) + __ldg(t2 + q)) * fc;
    }
    const double G3 = F[7] - F[6] - F[5] - F[3] - F[0] + F[4] + F[2] + F[1];
    return (float)(G3 * g.scale);
}

// x and y passes of the field kernel's three components, Lx = Ly = L, NTH
// threads, one stored z slice per blockIdx.x and two CTA roles
// (blockIdx.y): role 0 transforms components 0 (odd along x, even along y)
// and 1 (even along x, odd along y) together, four lines per FFT; role 1
// transforms component 2 (even along both) with two lines per FFT through
// the same code, its odd partner zero.  The rows go along x into shared
// memory, then the columns along y into T2out[comp][iz][ky][kx].
// With near.T set (the FP32 build), a CTA whose slice meets the near box
// first writes that slice's near cells of its components into G (the far
// cells come from the preceding launch), so the near cells take no launch
// of their own; G is then read through L2 (__ldcg), which sees those writes.
// STG: the CTA first copies its slice of G (its components, nx*ny each) to
// shared memory with cp.async (16-byte chunks when g16), writes the near
// cells there, and the x pass reads shared memory instead of L2.
// HALF: nx = ny = L/2 and Hx = L/2 + 1 (power-of-two meshes), so every
// sample and output index is a per-thread base plus a constant.
template <int L, typename Tr, int NTH, bool STG, bool HALF>
__global__ void __launch_bounds__(NTH, 1) k4_green_xy(Tr* G, Tr* __restrict__ T2out, int nx,
                                                      int ny, int Hx, int64_t gcs, int64_t t2cs, GreenNear near,
                                                      int g16, int solo,
                                                      const typename Cplx<Tr>::T2* __restrict__ tw) {
    using E = F2<L>;
    using T2 = typename Cplx<Tr>::T2;
    constexpr int W = NTH / E::NT;  // row pairs (x pass) or column pairs (y pass) per round
    __shared__ T2 swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* xb = reinterpret_cast<T2*>(smraw);             // W exchange columns
    Tr* ts0 = reinterpret_cast<Tr*>(xb + W * E::S);  // [ny][Hx]: the lines even along y, after the x pass
    Tr* ts1 = ts0 + (int64_t)ny * Hx;                 // the lines odd along y (role 0)
    // staged slice, 16-byte aligned: [slot][ny][nx], slot 0 the component
    // odd along x (0; role 1: component 2), slot 1 component 1
    Tr* gs = reinterpret_cast<Tr*>(smraw + ((W * E::S * sizeof(T2) + 2 * sizeof(Tr) * ny * Hx + 15) & ~(size_t)15));
    const int iz = blockIdx.x;
    // solo: one component (0), even along x and y (the potential kernel):
    // every CTA takes role 1 with that component
    const bool pair = !solo && blockIdx.y == 0;
    const int c1 = solo ? 0 : 2;  // the component of role 1
    const int per = nx * ny;
    if constexpr (STG) {
        const Tr* src0 = G + (pair ? 0 : c1) * gcs + (int64_t)per * iz;
        for (int sl = 0; sl < (pair ? 2 : 1); ++sl) {
            const Tr* src = src0 + sl * gcs;
            Tr* dst = gs + sl * per;
            if (g16) {
                constexpr int K = 16 / sizeof(Tr);
                for (int i = threadIdx.x; i < per / K; i += NTH) cp_async16(dst + i * K, src + i * K);
            } else {
                for (int i = threadIdx.x; i < per; i += NTH) {
                    if constexpr (sizeof(Tr) == 4)
                        cp_async4(dst + i, src + i);
                    else
                        cp_async8(dst + i, src + i);
                }
            }
        }
        cp_async_commit();
        cp_async_wait_all();
        __syncthreads();
    }
    if (near.T) {
        const int dz = near.image ? iz - (near.nz - 1) : iz;
        if (dz >= near.bz0 && dz < near.bz1) {
            const int box = near.nbx * near.nby;
            for (int e = threadIdx.x; e < (pair ? 2 : 1) * box; e += NTH) {
                const int c = pair ? e / box : c1;
                const int r = e - (pair ? c : 0) * box;
                const int ix = r % near.nbx, iy = r / near.nbx;
                if (green_near_cell(near, ix, iy, dz)) {
                    const Tr val = (Tr)green_near_value(near, c, ix, iy, dz);
                    if constexpr (STG)
                        gs[(pair ? c : 0) * per + ix + nx * iy] = val;
                    else
                        G[c * gcs + ix + (int64_t)nx * (iy + (int64_t)ny * iz)] = val;
                }
            }
            __syncthreads();
        }
    }
    T2 v[16];
    {
        const int t = threadIdx.x % E::NT, p = threadIdx.x / E::NT;
        T2* col = xb + p * E::S;
        // even along x: component 1 (role 0) or 2 (role 1); odd: component 0
        const Tr* ge = STG ? gs + (pair ? per : 0) : G + (pair ? 1 : c1) * gcs + (int64_t)per * iz;
        const Tr* go = STG ? gs : G + (int64_t)per * iz;
        Tr* dst_e = pair ? ts1 : ts0;
        // RS (a slice too large to stage whole: 256-point FP32 planes, two x
        // rounds of 2W rows): each round's rows are copied with cp.async into
        // the upper halves of ts0 (the even-along-x component) and ts1 (the
        // odd one), which only the last round's output uses, one round ahead
        // of the transform
        constexpr bool RS = !STG && HALF && L / 4 == 2 * W && sizeof(Tr) == 4;
        const bool rs = RS && g16;
        Tr* re_ = ts0 + (ny / 2) * Hx;
        Tr* ro_ = ts1 + (ny / 2) * Hx;
        auto stage_rows = [&](int q) {  // rows 2q .. 2q + 2W - 1
            constexpr int K = 16 / sizeof(Tr);
            const int n16 = 2 * W * nx / K;
            const Tr* se = ge + (int64_t)nx * 2 * q;
            const Tr* so = go + (int64_t)nx * 2 * q;
            for (int i = threadIdx.x; i < n16; i += NTH) {
                cp_async16(re_ + i * K, se + i * K);
                if (pair) cp_async16(ro_ + i * K, so + i * K);
            }
            cp_async_commit();
        };
        if (rs) stage_rows(0);
        for (int q0 = 0; q0 < (ny + 1) / 2; q0 += W) {
            const int y0 = 2 * (q0 + p), y1 = y0 + 1;
            const bool ok0 = y0 < ny, ok1 = y1 < ny;
            if (rs) {
                cp_async_wait_all();
                __syncthreads();
            }
            if (HALF && t < E::R2) {
                // x = t + R2*s: d = x below L/2, d = x - L above, nothing at
                // x = L/2; |d| from a per-thread base and a constant offset
                const Tr* ep0 = rs ? re_ + nx * (y0 - 2 * q0) : ge + nx * y0;
                const Tr* op0 = rs ? ro_ + nx * (y0 - 2 * q0) : go + nx * y0;
#pragma unroll
                for (int s = 0; s < E::R1; ++s) {
                    const bool lower = E::R2 * s < L / 2;
                    const bool here = lower || E::R2 * s > L / 2 || t > 0;
                    const int ax = lower ? t + E::R2 * s : L - t - E::R2 * s;
                    Tr e1 = 0, e2 = 0, o1 = 0, o2 = 0;
                    if (here) {
                        if (ok0) e1 = (STG || rs) ? ep0[ax] : ldcg_r(ep0 + ax);
                        if (ok1) e2 = (STG || rs) ? ep0[nx + ax] : ldcg_r(ep0 + nx + ax);
                        if (pair && (s > 0 || t > 0)) {  // odd: nothing at d = 0
                            if (ok0) o1 = (STG || rs) ? op0[ax] : ldcg_r(op0 + ax);
                            if (ok1) o2 = (STG || rs) ? op0[nx + ax] : ldcg_r(op0 + nx + ax);
                            if (!lower) o1 = -o1, o2 = -o2;
                        }
                    }
                    v[s] = Cplx<Tr>::make(e1 + o1, e2 + o2);
                }
            } else if (t < E::R2) {
#pragma unroll
                for (int s = 0; s < E::R1; ++s) {
                    const int x = t + E::R2 * s;
                    const int dx = x < nx ? x : (x > L - nx ? x - L : L);
                    Tr e1 = 0, e2 = 0, o1 = 0, o2 = 0;
                    if (dx != L) {
                        const int ax = dx < 0 ? -dx : dx;
                        if constexpr (STG) {
                            if (ok0) e1 = ge[nx * y0 + ax];
                            if (ok1) e2 = ge[nx * y1 + ax];
                        } else {
                            if (ok0) e1 = ldcg_r(ge + (int64_t)nx * y0 + ax);
                            if (ok1) e2 = ldcg_r(ge + (int64_t)nx * y1 + ax);
                        }
                        // an odd line vanishes at d = 0 (the stored sample there is rounding)
                        if (pair && dx != 0) {
                            if constexpr (STG) {
                                if (ok0) o1 = go[nx * y0 + ax];
                                if (ok1) o2 = go[nx * y1 + ax];
                            } else {
                                if (ok0) o1 = ldcg_r(go + (int64_t)nx * y0 + ax);
                                if (ok1) o2 = ldcg_r(go + (int64_t)nx * y1 + ax);
                            }
                            if (dx < 0) o1 = -o1, o2 = -o2;
                        }
                    }
                    v[s] = Cplx<Tr>::make(e1 + o1, e2 + o2);
                }
            }
            if (rs) {
                __syncthreads();  // every thread has its samples: the staged rows are free
                if (q0 + W < (ny + 1) / 2) stage_rows(q0 + W);
            }
            E::template fwd<false>(v, col, t, swt);
            if (t < E::R1) {
#pragma unroll
                for (int r = 0; r < E::R2; ++r) col[t + xoff(E::R1 * r)] = v[r];
            }
            __syncthreads();
            if (HALF && ok0) {
                constexpr int HX = L / 2 + 1, NT = E::NT;
                const int tm = t == 0 ? 0 : NT - t;  // the mirror L - k = tm + constant
#pragma unroll
                for (int i = 0; i <= L / (2 * NT); ++i) {
                    if (i == L / (2 * NT) && t > 0) break;  // k = L/2 only at t = 0
                    const int k = t + NT * i;
                    const int km = t == 0 ? xoff((L - NT * i) & (L - 1)) : tm + xoff(L - NT * (i + 1));
                    Tr e1, e2, p1, p2;
                    unpack4(col[t + xoff(NT * i)], col[km], e1, e2, p1, p2);
                    dst_e[y0 * HX + k] = e1;
                    if (ok1) dst_e[y1 * HX + k] = e2;
                    if (pair) {
                        ts0[y0 * HX + k] = p1;
                        if (ok1) ts0[y1 * HX + k] = p2;
                    }
                }
            } else if (ok0) {
                for (int k = t; k <= L / 2; k += E::NT) {
                    Tr e1, e2, p1, p2;
                    unpack4(col[xsw(k)], col[xsw((L - k) & (L - 1))], e1, e2, p1, p2);
                    dst_e[y0 * Hx + k] = e1;
                    if (ok1) dst_e[y1 * Hx + k] = e2;
                    if (pair) {
                        ts0[y0 * Hx + k] = p1;
                        if (ok1) ts0[y1 * Hx + k] = p2;
                    }
                }
            }
            __syncthreads();
        }
    }
    {
        const int c = threadIdx.x % W, t = threadIdx.x / W;
        T2* col = xb + c * E::S;
        // even along y: component 0 (role 0) or 2 (role 1); odd: component 1
        Tr* out_e = T2out + (pair ? 0 : c1) * t2cs + (int64_t)Hx * (L / 2 + 1) * iz;
        Tr* out_o = T2out + t2cs + (int64_t)Hx * (L / 2 + 1) * iz;
        // the Nyquist column kx = L/2 by direct sums:
        // X(k) = sum_d x(d) w^(k d), d = -(ny-1)..ny-1
        // (four partial sums, so the loads of one step overlap the next)
        for (int k = threadIdx.x; k <= L / 2; k += NTH) {
            Tr re[4] = {0, 0, 0, 0}, im[4] = {0, 0, 0, 0};
            int d = 1;
            for (; d + 3 < ny; d += 4) {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const T2 wp = swt[(k * (d + u)) & (L - 1)];
                    re[u] += Tr(2) * ts0[(d + u) * Hx + L / 2] * c_re(wp);             // even: 2 x(d) Re w^kd
                    if (pair) im[u] += Tr(2) * ts1[(d + u) * Hx + L / 2] * c_im(wp);  // odd: 2i x(d) Im w^kd
                }
            }
            for (; d < ny; ++d) {
                const T2 wp = swt[(k * d) & (L - 1)];
                re[0] += Tr(2) * ts0[d * Hx + L / 2] * c_re(wp);
                if (pair) im[0] += Tr(2) * ts1[d * Hx + L / 2] * c_im(wp);
            }
            out_e[(int64_t)k * Hx + L / 2] = ts0[L / 2] + ((re[0] + re[1]) + (re[2] + re[3]));
            if (pair) out_o[(int64_t)k * Hx + L / 2] = (im[0] + im[1]) + (im[2] + im[3]);
        }
        for (int k0 = 0; k0 < L / 2; k0 += 2 * W) {
            const int fa = k0 + c, fb = fa + W;
            const bool oka = fa < L / 2, okb = fb < L / 2;
            if (HALF && t < E::R2) {
                // as the x pass, along y: rows of ts0 / ts1 (HX floats)
                constexpr int HX = L / 2 + 1;
                const Tr* lo0 = ts0 + t * HX;
                const Tr* hi0 = ts0 + (L - t) * HX;
                const Tr* lo1 = ts1 + t * HX;
                const Tr* hi1 = ts1 + (L - t) * HX;
#pragma unroll
                for (int s = 0; s < E::R1; ++s) {
                    const bool lower = E::R2 * s < L / 2;
                    const bool here = lower || E::R2 * s > L / 2 || t > 0;
                    const Tr* r0 = lower ? lo0 + E::R2 * s * HX : hi0 - E::R2 * s * HX;
                    const Tr* r1 = lower ? lo1 + E::R2 * s * HX : hi1 - E::R2 * s * HX;
                    Tr e1 = 0, e2 = 0, o1 = 0, o2 = 0;
                    if (here) {
                        if (oka) e1 = r0[fa];
                        if (okb) e2 = r0[fb];
                        if (pair && (s > 0 || t > 0)) {
                            if (oka) o1 = r1[fa];
                            if (okb) o2 = r1[fb];
                            if (!lower) o1 = -o1, o2 = -o2;
                        }
                    }
                    v[s] = Cplx<Tr>::make(e1 + o1, e2 + o2);
                }
            } else if (t < E::R2) {
#pragma unroll
                for (int s = 0; s < E::R1; ++s) {
                    const int n = t + E::R2 * s;
                    const int d = n < ny ? n : (n > L - ny ? n - L : L);
                    Tr e1 = 0, e2 = 0, o1 = 0, o2 = 0;
                    if (d != L) {
                        const int ad = d < 0 ? -d : d;
                        if (oka) e1 = ts0[ad * Hx + fa];
                        if (okb) e2 = ts0[ad * Hx + fb];
                        if (pair && d != 0) {
                            if (oka) o1 = ts1[ad * Hx + fa];
                            if (okb) o2 = ts1[ad * Hx + fb];
                            if (d < 0) o1 = -o1, o2 = -o2;
                        }
                    }
                    v[s] = Cplx<Tr>::make(e1 + o1, e2 + o2);
                }
            }
            E::template fwd<false>(v, col, t, swt);
            if (t < E::R1) {
#pragma unroll
                for (int r = 0; r < E::R2; ++r) col[t + xoff(E::R1 * r)] = v[r];
            }
            __syncthreads();
            if constexpr (HALF) {
                constexpr int HX = L / 2 + 1, NT = E::NT;
                const int tm = t == 0 ? 0 : NT - t;
                Tr* oe = out_e + (int64_t)t * HX;
                Tr* oo = out_o + (int64_t)t * HX;
#pragma unroll
                for (int i = 0; i <= L / (2 * NT); ++i) {
                    if (i == L / (2 * NT) && t > 0) break;  // k = L/2 only at t = 0
                    const int km = t == 0 ? xoff((L - NT * i) & (L - 1)) : tm + xoff(L - NT * (i + 1));
                    Tr e1, e2, p1, p2;
                    unpack4(col[t + xoff(NT * i)], col[km], e1, e2, p1, p2);
                    if (oka) oe[NT * i * HX + fa] = e1;
                    if (okb) oe[NT * i * HX + fb] = e2;
                    if (pair) {
                        if (oka) oo[NT * i * HX + fa] = p1;
                        if (okb) oo[NT * i * HX + fb] = p2;
                    }
                }
            } else {
                for (int k = t; k <= L / 2; k += E::NT) {
                    Tr e1, e2, p1, p2;
                    unpack4(col[xsw(k)], col[xsw((L - k) & (L - 1))], e1, e2, p1, p2);
                    if (oka) out_e[(int64_t)k * Hx + fa] = e1;
                    if (okb) out_e[(int64_t)k * Hx + fb] = e2;
                    if (pair) {
                        if (oka) out_o[(int64_t)k * Hx + fa] = p1;
                        if (okb) out_o[(int64_t)k * Hx + fb] = p2;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Free-space z pass of the field kernel's three components, two CTA roles
// (blockIdx.y): role 0 transforms components 0 (even along z) and 2 (odd)
// together, four lines per FFT; role 1 component 1 (even), two lines per
// FFT through the same code.  Column pairs fa, fb = fa + kColW of the ncols
// columns: input sample d >= 0 of component c at in + c*cs_in + col +
// d*as_in (d < nh), output k <= L/2 of the kept part (E for the even, P for
// the odd component) at out + c*cs_out + col + k*as_out.  Lines summed into
// one FFT keep the precision of the larger: component 2 lacks the factor
// gamma of components 0 and 1, so it enters multiplied by s2 (a power of two
// near gamma) and leaves divided by it, both exact.
template <int L, typename Tr, bool HALF>
__global__ void __launch_bounds__(kColW * F2<L>::NT, sizeof(Tr) == 4 ? 3 : 1) k4_green_col(const Tr* __restrict__ in,
                                                                           Tr* __restrict__ out, int ncols, int nh,
                                                                           int64_t as_in, int64_t cs_in,
                                                                           int64_t as_out, int64_t cs_out, Tr s2,
                                                                           int solo,
                                                                           const typename Cplx<Tr>::T2* __restrict__ tw) {
    using E = F2<L>;
    using T2 = typename Cplx<Tr>::T2;
    __shared__ T2 swt[L];
    stage_twiddles<L>(swt, tw);
    extern __shared__ __align__(16) unsigned char smraw[];
    T2* xb = reinterpret_cast<T2*>(smraw);
    // solo: one component (0), even along z (the potential kernel): every CTA
    // takes role 1 with that component
    const bool pair = !solo && blockIdx.y == 0;
    const int c1 = solo ? 0 : 1;  // the component of role 1
    const Tr* ie = in + (pair ? 0 : c1) * cs_in;
    const Tr* io = in + 2 * cs_in;
    Tr* oe = out + (pair ? 0 : c1) * cs_out;
    Tr* oo = out + 2 * cs_out;
    const int c = threadIdx.x % kColW, t = threadIdx.x / kColW;
    const int64_t fa = (int64_t)blockIdx.x * (2 * kColW) + c, fb = fa + kColW;
    const bool oka = fa < ncols, okb = fb < ncols;
    T2* col = xb + c * E::S;
    T2 v[16];
    if (HALF && t < E::R2) {
        // nh = L/2: sample n = t + R2*s is d = n below L/2, d = n - L above,
        // nothing at L/2; |d| * as_in from per-thread bases
        const Tr* elo = ie + t * as_in;
        const Tr* ehi = ie + (L - t) * as_in;
        const Tr* olo = io + t * as_in;
        const Tr* ohi = io + (L - t) * as_in;
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const bool lower = E::R2 * s < L / 2;
            const bool here = lower || E::R2 * s > L / 2 || t > 0;
            const int64_t o = (int64_t)(E::R2 * s) * as_in;
            const Tr* pe = lower ? elo + o : ehi - o;
            const Tr* po = lower ? olo + o : ohi - o;
            Tr e1 = 0, e2 = 0, o1 = 0, o2 = 0;
            if (here) {
                if (oka) e1 = ldg_r(pe + fa);
                if (okb) e2 = ldg_r(pe + fb);
                if (pair && (s > 0 || t > 0)) {
                    if (oka) o1 = s2 * ldg_r(po + fa);
                    if (okb) o2 = s2 * ldg_r(po + fb);
                    if (!lower) o1 = -o1, o2 = -o2;
                }
            }
            v[s] = Cplx<Tr>::make(e1 + o1, e2 + o2);
        }
    } else if (t < E::R2) {
#pragma unroll
        for (int s = 0; s < E::R1; ++s) {
            const int n = t + E::R2 * s;
            const int d = n < nh ? n : (n > L - nh ? n - L : L);
            Tr e1 = 0, e2 = 0, o1 = 0, o2 = 0;
            if (d != L) {
                const int64_t o = (int64_t)(d < 0 ? -d : d) * as_in;
                if (oka) e1 = ldg_r(ie + fa + o);
                if (okb) e2 = ldg_r(ie + fb + o);
                // an odd line vanishes at d = 0 (the stored sample there is rounding)
                if (pair && d != 0) {
                    if (oka) o1 = s2 * ldg_r(io + fa + o);
                    if (okb) o2 = s2 * ldg_r(io + fb + o);
                    if (d < 0) o1 = -o1, o2 = -o2;
                }
            }
            v[s] = Cplx<Tr>::make(e1 + o1, e2 + o2);
        }
    }
    E::template fwd<false>(v, col, t, swt);
    if (t < E::R1) {
#pragma unroll
        for (int r = 0; r < E::R2; ++r) col[t + xoff(E::R1 * r)] = v[r];
    }
    __syncthreads();
    const Tr inv2 = Tr(1) / s2;
    if constexpr (HALF) {
        constexpr int NT = E::NT;
        const int tm = t == 0 ? 0 : NT - t;
        Tr* pe = oe + t * as_out;
        Tr* po = oo + t * as_out;
#pragma unroll
        for (int i = 0; i <= L / (2 * NT); ++i) {
            if (i == L / (2 * NT) && t > 0) break;  // k = L/2 only at t = 0
            const int km = t == 0 ? xoff((L - NT * i) & (L - 1)) : tm + xoff(L - NT * (i + 1));
            const int64_t o = (int64_t)(NT * i) * as_out;
            Tr e1, e2, p1, p2;
            unpack4(col[t + xoff(NT * i)], col[km], e1, e2, p1, p2);
            if (oka) pe[o + fa] = e1;
            if (okb) pe[o + fb] = e2;
            if (pair) {
                if (oka) po[o + fa] = p1 * inv2;
                if (okb) po[o + fb] = p2 * inv2;
            }
        }
    } else {
        for (int k = t; k <= L / 2; k += E::NT) {
            Tr e1, e2, p1, p2;
            unpack4(col[xsw(k)], col[xsw((L - k) & (L - 1))], e1, e2, p1, p2);
            if (oka) oe[fa + k * as_out] = e1;
            if (okb) oe[fb + k * as_out] = e2;
            if (pair) {
                if (oka) oo[fa + k * as_out] = p1 * inv2;
                if (okb) oo[fb + k * as_out] = p2 * inv2;
            }
        }
    }
}

// Launch helpers: run the two-step kernel when L <= 256, report false
// otherwise (the caller falls back to the Stockham kernels).

static bool launch2_col(bool inv, int logL, const float2* in, float2* out, int ncols, int n_valid, int n_store,
                        int64_t as_in, int64_t bs_in, int64_t cs_in, int64_t as_out, int64_t bs_out, int64_t cs_out,
                        int nbatch, int ncomp, const float2* tw, cudaStream_t s, int wrap = 0, int bwrap_n = 0,
                        int bwrap_L = 0) {
    dim3 grid((unsigned)(((int64_t)ncols * nbatch + kColW - 1) / kColW), ncomp);
#define SC_K2COL(LL)                                                                                            \
    if (inv)                                                                                                    \
        launch_pdl(k2_col<LL, true>, grid, kColW * F2<LL>::NT, 0, s, in, out, ncols, nbatch, n_valid, n_store, wrap, bwrap_n, \
                                                              bwrap_L, as_in, bs_in, cs_in, as_out, bs_out,     \
                                                              cs_out, tw);                                      \
    else                                                                                                        \
        launch_pdl(k2_col<LL, false>, grid, kColW * F2<LL>::NT, 0, s, in, out, ncols, nbatch, n_valid, n_store, wrap, bwrap_n, \
                                                               bwrap_L, as_in, bs_in, cs_in, as_out, bs_out,    \
                                                               cs_out, tw);
    SC_L_SWITCH(logL, SC_K2COL)
#undef SC_K2COL
    return true;
}

static bool launch2_fwd_x(int logL, const float* rho, float2* A, int nx, int rows, int Hx, const float2* tw,
                          cudaStream_t s) {
#define SC_K2FX(LL)                                                          \
    {                                                                        \
        constexpr int P = 256 / F2<LL>::NT;                                  \
        const int pairs = (rows + 1) / 2;                                    \
        launch_pdl(k2_fwd_x<LL>, (pairs + P - 1) / P, 256, 0, s, rho, A, nx, rows, Hx, tw); \
    }
    SC_L_SWITCH(logL, SC_K2FX)
#undef SC_K2FX
    return true;
}

// The fused forward x+y pass: Lx = Ly and the plane in shared memory, at
// most `cap` bytes (as launch2_inv_yx).
static bool launch2_fwd_xy(int logLx, int logLy, const float* rho, float2* B, int nx, int ny, int nz, int Hx,
                           const float2* tw, cudaStream_t s, size_t cap, int ncomp = 1, int64_t in_cs = 0,
                           int64_t out_cs = 0) {
    if (logLx != logLy) return false;
#define SC_K2XY(LL)                                                                     \
    {                                                                                   \
        constexpr int W = 256 / F2<LL>::NT;                                             \
        const size_t smem = sizeof(float2) * ((size_t)W * F2<LL>::S + (size_t)ny * Hx); \
        if (smem > cap) return false;                                                   \
        if (set_smem(k2_fwd_xy<LL>, smem) != SC_OK) return false;                       \
        launch_pdl(k2_fwd_xy<LL>, dim3(nz, ncomp), 256, smem, s, rho, B, nx, ny, Hx, in_cs, out_cs, tw); \
    }
    SC_L_SWITCH(logLx, SC_K2XY)
#undef SC_K2XY
    return true;
}

// The fused inverse y+x pass needs Lx = Ly and the plane in shared memory.
// `cap`: the largest plane (bytes of shared memory) to fuse; above about
// 100 KB a CTA has an SM to itself, which pays only when other streams' work
// fills the rest (batch_issue).
static bool launch2_inv_yx(int logLx, int logLy, const float2* C, float4* E4, int nx, int ny, int nz, int Hx,
                           const float2* tw, cudaStream_t s, size_t cap, int ncomp = 3, int lane0 = 0) {
    if (logLx != logLy) return false;
#define SC_K2YX(LL)                                                                                   \
    {                                                                                                 \
        constexpr int W = 256 / F2<LL>::NT;                                                           \
        const size_t smem = sizeof(float2) * ((size_t)W * F2<LL>::S + (size_t)ny * Hx);               \
        if (smem > cap) return false;                                                                 \
        if (set_smem(k2_inv_yx<LL>, smem) != SC_OK) return false;                                     \
        launch_pdl(k2_inv_yx<LL>, dim3(nz, ncomp), 256, smem, s, C, reinterpret_cast<float*>(E4), nx, ny, nz, Hx, \
                   lane0, tw);                                                                                 \
    }
    SC_L_SWITCH(logLx, SC_K2YX)
#undef SC_K2YX
    return true;
}

static bool launch2_inv_x(int logL, const float2* D, float4* E4, int nx, int rows, int Hx, int64_t cs,
                          const float2* tw, cudaStream_t s) {
#define SC_K2IX_GO(LL, HALF)                                                                          \
    {                                                                                                 \
        if (set_smem(k2_inv_x<LL, HALF>, smem) != SC_OK) return false;                                \
        launch_pdl(k2_inv_x<LL, HALF>, (pairs + P - 1) / P, 256, smem, s, D, E4, nx, rows, Hx, cs, tw); \
    }
#define SC_K2IX(LL)                                                                                   \
    {                                                                                                 \
        constexpr int P = 256 / F2<LL>::NT;                                                           \
        const size_t smem = sizeof(float2) * (P * F2<LL>::S + 2 * (size_t)P * nx);                    \
        const int pairs = (rows + 1) / 2;                                                             \
        if (2 * nx == LL && 2 * (Hx - 1) == LL)                                                       \
            SC_K2IX_GO(LL, true)                                                                      \
        else                                                                                          \
            SC_K2IX_GO(LL, false)                                                                     \
    }
    SC_L_SWITCH(logL, SC_K2IX)
#undef SC_K2IX
#undef SC_K2IX_GO
    return true;
}

static bool launch2_zpass(int logL, const float2* B, float2* C, int Hx, int Ly, int nz, const GreenView& gv,
                          const float2* tw, cudaStream_t s) {
#define SC_K2Z(LL)                                                                          \
    {                                                                                       \
        const size_t smem = sizeof(float2) * kColW * F2<LL>::S * 2 +                        \
                            sizeof(float) * 3 * (LL / 2 + 1) * kColW +                          \
                            (gv.image && gv.img_half ? sizeof(float2) * (LL / 2 + 1) * kColW : 0); \
        const int64_t ncol = (int64_t)Hx * Ly;                                              \
        const unsigned grid = (unsigned)((ncol + kColW - 1) / kColW);                       \
        if (2 * nz == LL) {                                                                 \
            if (set_smem(k2_zpass<LL, true>, smem) != SC_OK) return false;                  \
            launch_pdl(k2_zpass<LL, true>, grid, kColW * F2<LL>::NT, smem, s, B, C, Hx, Ly, nz, gv, tw); \
        } else {                                                                            \
            if (set_smem(k2_zpass<LL, false>, smem) != SC_OK) return false;                 \
            launch_pdl(k2_zpass<LL, false>, grid, kColW * F2<LL>::NT, smem, s, B, C, Hx, Ly, nz, gv, tw); \
        }                                                                                   \
    }
    SC_L_SWITCH(logL, SC_K2Z)
#undef SC_K2Z
    return true;
}

// FP64 meshes, double-FP32 passes (dd_passes.cu, dd_xy.cu); false where
// they do not apply (the image for the z pass, transforms above 256
// points).  launch2_dd_col: column transforms (forward or inverse) of ncomp
// components; TI / TO: double2 (FP64) or ddc (double-FP32) buffers.
bool launch2_dd_fwd_x(int logL, const double* rho, ddc* A, int nx, int rows, int Hx, const ddc* tw, cudaStream_t s);
template <bool INV, typename TI, typename TO>
bool launch2_dd_col(int logL, const TI* in, TO* out, int ncols, int nbatch, int ncomp, int n_valid, int n_store,
                    int64_t as_in, int64_t bs_in, int64_t cs_in, int64_t as_out, int64_t bs_out, int64_t cs_out,
                    const ddc* tw, cudaStream_t s);
// The FP64 free-space Green transform in double-FP32 (dd_green.cu): the
// paired x+y and z passes of the field kernel (solo: the potential kernel,
// one component even along every axis) with dreal values, from the octant G
// to the spectrum `out` (the layout of the FP64 build).  Applies to
// power-of-two meshes (n = L/2 on every axis) with Lx = Ly in {64, 128} and
// Lz in {64, 128, 256}; dd_green_applies says whether.
bool dd_green_applies(int logLx, int logLy, int logLz, int nx, int ny, int nz);
bool launch_dd_green(int logLxy, int logLz, dreal* G, dreal* T2, dreal* out, int nx, int ny, int nz, int Hx,
                     int64_t gcs, int64_t t2cs, double gamma, const ddc* tw, cudaStream_t s, int solo = 0);
// gfmt: the free-space Green spectrum is double-FP32 (dreal) rather than FP64
bool launch2_dd_zpass(int logL, const ddc* B, ddc* C, int Hx, int Ly, int nz, const GreenView& gv, int gfmt,
                      const ddc* tw, cudaStream_t s);
bool launch2_dd_inv_x(int logL, const ddc* D, dnode4* E4, int nx, int rows, int Hx, int64_t cs, const ddc* tw,
                      cudaStream_t s);
// the scalar potential's z pass and inverse x pass (dd_pot.cu)
// pf: the free-space spectrum, FP64 (pfmt 0) or dreal (pfmt 1)
bool launch2_dd_zpass_pot(int logL, const ddc* B, ddc* C, int Hx, int Ly, int nz, const void* pf, int pfmt,
                          const double2* pi, int image, int Hy, const ddc* tw, cudaStream_t s);
bool launch2_dd_inv_x1(int logL, const ddc* D, dnode4* E4, int nx, int rows, int Hx, const ddc* tw, cudaStream_t s);

static bool launch2_adj_zpass(int logL, const float2* C, float2* B, int Hx, int Ly, int nz, const GreenView& gv,
                              const float2* tw, cudaStream_t s) {
#define SC_K2AZ(LL)                                                                         \
    {                                                                                       \
        const size_t smem = sizeof(float2) * kColW * F2<LL>::S * 2 +                        \
                            sizeof(float) * 3 * (LL / 2 + 1) * kColW;                           \
        const int64_t ncol = (int64_t)Hx * Ly;                                              \
        const unsigned grid = (unsigned)((ncol + kColW - 1) / kColW);                       \
        if (2 * nz == LL) {                                                                 \
            if (set_smem(k2_adj_zpass<LL, true>, smem) != SC_OK) return false;              \
            launch_pdl(k2_adj_zpass<LL, true>, grid, kColW * F2<LL>::NT, smem, s, C, B, Hx, Ly, nz, gv, tw); \
        } else {                                                                            \
            if (set_smem(k2_adj_zpass<LL, false>, smem) != SC_OK) return false;             \
            launch_pdl(k2_adj_zpass<LL, false>, grid, kColW * F2<LL>::NT, smem, s, C, B, Hx, Ly, nz, gv, tw); \
        }                                                                                   \
    }
    SC_L_SWITCH(logL, SC_K2AZ)
#undef SC_K2AZ
    return true;
}

static bool launch2_inv_x1(int logL, const float2* D, float* E4, int nx, int rows, int Hx, const float2* tw,
                           cudaStream_t s) {
#define SC_K2IX1(LL)                                                                  \
    {                                                                                 \
        constexpr int P = 256 / F2<LL>::NT;                                           \
        const int pairs = (rows + 1) / 2;                                             \
        launch_pdl(k2_inv_x1<LL>, (pairs + P - 1) / P, 256, 0, s, D, E4, nx, rows, Hx, tw);   \
    }
    SC_L_SWITCH(logL, SC_K2IX1)
#undef SC_K2IX1
    return true;
}

// ncomp kernel components (blockIdx.y); odd_x, odd_y, imask as in the
// kernels (the field's defaults: 3 components, 0, 1, 3).
template <typename Tr>
static bool launch3_green_x(int logL, const Tr* G, Tr* T, int nx, int rows, int Hx, int64_t gcs, int64_t tcs,
                            const typename Cplx<Tr>::T2* tw, cudaStream_t s, int ncomp = 3, int odd_x = 0) {
    using T2 = typename Cplx<Tr>::T2;
#define SC_K3GX(LL)                                                                 \
    {                                                                               \
        constexpr int P = 256 / F2<LL>::NT;                                         \
        const size_t smem = sizeof(T2) * P * F2<LL>::S;                             \
        if (set_smem(k3_green_x<LL, Tr>, smem) != SC_OK) return false;              \
        dim3 grid(((rows + 1) / 2 + P - 1) / P, ncomp);                             \
        launch_pdl(k3_green_x<LL, Tr>, grid, 256, smem, s, G, T, nx, rows, Hx, gcs, tcs, odd_x, tw); \
    }
    SC_L_SWITCH(logL, SC_K3GX)
#undef SC_K3GX
    return true;
}

// The fused x+y Green pass needs Lx = Ly and the slice in shared memory
// (100 KB in FP32, where three CTAs share an SM; the FP64 slice of a
// 128 x 128 plane takes 202 KB).
template <typename Tr>
static bool launch3_green_xy(int logLx, int logLy, const Tr* G, Tr* T2, int nx, int ny, int zc, int Hx,
                             int64_t gcs, int64_t t2cs, const typename Cplx<Tr>::T2* tw, cudaStream_t s,
                             int ncomp = 3, int odd_x = 0, int odd_y = 1) {
    using C2 = typename Cplx<Tr>::T2;
    if (logLx != logLy) return false;
    const size_t cap = sizeof(Tr) == 4 ? 100 * 1024 : 210 * 1024;
#define SC_K3XY(LL)                                                                                 \
    {                                                                                               \
        constexpr int W = 256 / F2<LL>::NT;                                                         \
        const size_t smem = sizeof(C2) * (size_t)W * F2<LL>::S + sizeof(Tr) * (size_t)ny * Hx;     \
        if (smem > cap) return false;                                                               \
        if (set_smem(k3_green_xy<LL, Tr>, smem) != SC_OK) return false;                             \
        launch_pdl(k3_green_xy<LL, Tr>, dim3(zc, ncomp), 256, smem, s, G, T2, nx, ny, Hx, gcs, t2cs, odd_x, odd_y, tw); \
    }
    SC_L_SWITCH(logLx, SC_K3XY)
#undef SC_K3XY
    return true;
}

template <typename Tr>
static bool launch3_green_col(bool img, int logL, const Tr* in, void* out, int ncols, int nbatch, int nh,
                              int odd_comp, int64_t as_in, int64_t bs_in, int64_t cs_in, int64_t as_out,
                              int64_t bs_out, int64_t cs_out, const typename Cplx<Tr>::T2* tw, cudaStream_t s,
                              int ncomp = 3, int imask = 3) {
    using T2 = typename Cplx<Tr>::T2;
    dim3 grid((unsigned)(((int64_t)ncols * nbatch + 2 * kColW - 1) / (2 * kColW)), ncomp);
#define SC_K3GC(LL)                                                                                           \
    {                                                                                                         \
        const size_t smem = sizeof(T2) * kColW * F2<LL>::S;                                                   \
        if (img) {                                                                                            \
            if (set_smem(k3_green_col<LL, true, Tr>, smem) != SC_OK) return false;                           \
            launch_pdl(k3_green_col<LL, true, Tr>, grid, kColW * F2<LL>::NT, smem, s, in, out, ncols, nbatch, nh, \
                       odd_comp, as_in, bs_in, cs_in, as_out, bs_out, cs_out, imask, tw);                    \
        } else {                                                                                              \
            if (set_smem(k3_green_col<LL, false, Tr>, smem) != SC_OK) return false;                          \
            launch_pdl(k3_green_col<LL, false, Tr>, grid, kColW * F2<LL>::NT, smem, s, in, out, ncols, nbatch, nh, \
                       odd_comp, as_in, bs_in, cs_in, as_out, bs_out, cs_out, imask, tw);                    \
        }                                                                                                     \
    }
    SC_L_SWITCH(logL, SC_K3GC)
#undef SC_K3GC
    return true;
}

// x and y passes of the field kernel's three components in one launch of
// k4_green_xy (256 threads, or 512 when the two slices need more than
// 100 KB of shared memory); solo: the one component of the potential kernel
// (even along x and y) at G and T2.  Returns false (nothing launched) where they do
// not fit; the caller then runs launch3_green_xy or the separate passes.
template <typename Tr>
static bool launch_green_xy_field(int logLx, int logLy, Tr* G, Tr* T2, int nx, int ny, int zc, int Hx,
                                  int64_t gcs, int64_t t2cs, const typename Cplx<Tr>::T2* tw, cudaStream_t s,
                                  const GreenNear& near = GreenNear{}, int solo = 0) {
    using C2 = typename Cplx<Tr>::T2;
    if (logLx != logLy) return false;
    const size_t planes = 2 * sizeof(Tr) * (size_t)ny * Hx;
    const size_t slice = 2 * sizeof(Tr) * (size_t)nx * ny + 16;  // the staged slice, with its alignment slack
    const int g16 = ((uintptr_t)G % 16 == 0 && (sizeof(Tr) * (size_t)nx * ny) % 16 == 0 &&
                     (sizeof(Tr) * (size_t)gcs) % 16 == 0) ? 1 : 0;
    bool ok = false;
#define SC_K4XY_GO(LL, NTH, STG, SM)                                                                        \
    {                                                                                                        \
        if (half) {                                                                                          \
            if (set_smem(k4_green_xy<LL, Tr, NTH, STG, true>, SM) != SC_OK) return false;                    \
            launch_pdl(k4_green_xy<LL, Tr, NTH, STG, true>, dim3(zc, solo ? 1 : 2), NTH, SM, s, G, T2, nx, ny, \
                       Hx, gcs, t2cs, near, g16, solo, tw);                                                   \
        } else {                                                                                             \
            if (set_smem(k4_green_xy<LL, Tr, NTH, STG, false>, SM) != SC_OK) return false;                   \
            launch_pdl(k4_green_xy<LL, Tr, NTH, STG, false>, dim3(zc, solo ? 1 : 2), NTH, SM, s, G, T2, nx,   \
                       ny, Hx, gcs, t2cs, near, g16, solo, tw);                                               \
        }                                                                                                    \
        ok = true;                                                                                           \
    }
#define SC_K4XY(LL)                                                                                          \
    {                                                                                                        \
        const size_t s256 = sizeof(C2) * (size_t)(256 / F2<LL>::NT) * F2<LL>::S + planes;                    \
        const size_t s512 = sizeof(C2) * (size_t)(512 / F2<LL>::NT) * F2<LL>::S + planes;                    \
        const bool half = 2 * nx == LL && 2 * ny == LL && 2 * (Hx - 1) == LL;                               \
        if (s256 + slice <= 100 * 1024)                                                                      \
            SC_K4XY_GO(LL, 256, true, s256 + slice)                                                          \
        else if (s256 <= 100 * 1024)                                                                         \
            SC_K4XY_GO(LL, 256, false, s256)                                                                 \
        else if (s512 <= 220 * 1024)                                                                         \
            SC_K4XY_GO(LL, 512, false, s512)                                                                 \
    }
    SC_L_SWITCH(logLx, SC_K4XY)
#undef SC_K4XY
#undef SC_K4XY_GO
    return ok;
}

// Free-space z pass of the field kernel's three components in one launch
// of k4_green_col; solo: the one component of the potential kernel (even
// along z).  Columns at in + c*cs_in + col + d*as_in, out + c*cs_out
// + col + k*as_out.
template <typename Tr>
static bool launch_green_z_field(int logL, const Tr* in, Tr* out, int ncols, int nh, int64_t as_in, int64_t cs_in,
                                 int64_t as_out, int64_t cs_out, double gamma, const typename Cplx<Tr>::T2* tw,
                                 cudaStream_t s, int solo = 0) {
    using T2 = typename Cplx<Tr>::T2;
    const Tr s2 = (Tr)exp2(rint(log2(gamma > 1.0 ? gamma : 1.0)));  // a power of two: exact scaling
    const dim3 grid((unsigned)(((int64_t)ncols + 2 * kColW - 1) / (2 * kColW)), solo ? 1 : 2);
#define SC_K4GC_GO(LL, HALF)                                                                                  \
    {                                                                                                         \
        if (set_smem(k4_green_col<LL, Tr, HALF>, smem) != SC_OK) return false;                                \
        launch_pdl(k4_green_col<LL, Tr, HALF>, grid, kColW * F2<LL>::NT, smem, s, in, out, ncols, nh, as_in,   \
                   cs_in, as_out, cs_out, s2, solo, tw);                                                       \
    }
#define SC_K4GC(LL)                                                                                           \
    {                                                                                                         \
        const size_t smem = sizeof(T2) * kColW * F2<LL>::S;                                                   \
        if (2 * nh == LL)                                                                                     \
            SC_K4GC_GO(LL, true)                                                                              \
        else                                                                                                  \
            SC_K4GC_GO(LL, false)                                                                             \
    }
    SC_L_SWITCH(logL, SC_K4GC)
#undef SC_K4GC
#undef SC_K4GC_GO
    return true;
}

}  // namespace sc
