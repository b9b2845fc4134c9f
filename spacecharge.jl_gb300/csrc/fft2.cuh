// Register-resident two-step FFT of compile-time length L = R1 * R2
// (R1, R2 <= 16) for batches of columns, one shared-memory exchange per
// transform.
//
// A column's elements are spread over NT = max(R1, R2) threads in one of two
// distributions:
//   data  ("A"): thread t < R2 holds n = t + R2*s,  s < R1   (v[s])
//   freq  ("B"): thread t < R1 holds k = t + R1*r,  r < R2   (v[r])
// fwd():  A -> B.  Step 1: DFT_R1 over s, written to the exchange buffer at
//         t*R1 + k1; step 2: thread t' reads t' + R1*r, twiddles by
//         w^(r t') (w = e^{-2 pi i/L}) and does DFT_R2 over r, which leaves
//         X[t' + R1*r] in its registers (the Stockham two-stage order).
// inv():  B -> A, the same two steps mirrored (unnormalised):
//         x[n1 + R2*n2] = sum_t' e^{2pi i t' n2/R1} e^{2pi i t' n1/L}
//                         sum_r P[t' + R1 r] e^{2pi i r n1/R2}.
// The exchange buffer holds a column at idx + idx/16 (a swizzle that keeps
// both thread-to-column mappings the kernels use free of bank conflicts),
// columns at an odd stride XS<L>.
#pragma once

#include "fft.cuh"

namespace sc {

template <int L>
struct XS {
    static constexpr int raw = L + L / 16;
    static constexpr int value = (raw & 1) ? raw : raw + 1;
};
__device__ __forceinline__ int xsw(int idx) { return idx + (idx >> 4); }
// The two access patterns of the exchange, with the swizzle split into a
// per-thread base and a compile-time offset (R divides 16, so a run of R
// consecutive indices starting at a multiple of R never crosses a multiple
// of 16, and t + R*r with t < R carries nothing into bit 4):
//   xsw(t * R + k) = xrow<R>(t) + k          for k < R
//   xsw(t + R * r) = t + xoff(R * r)         for t < R
__host__ __device__ constexpr int xoff(int i) { return i + (i >> 4); }
template <int R>
__device__ __forceinline__ int xrow(int t) {
    return t * R + ((t * R) >> 4);
}

template <int L>
struct Split;  // (R1, R2) for each length
template <> struct Split<4> { static constexpr int R1 = 2, R2 = 2; };
template <> struct Split<8> { static constexpr int R1 = 4, R2 = 2; };
template <> struct Split<16> { static constexpr int R1 = 4, R2 = 4; };
template <> struct Split<32> { static constexpr int R1 = 8, R2 = 4; };
template <> struct Split<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct Split<128> { static constexpr int R1 = 16, R2 = 8; };
template <> struct Split<256> { static constexpr int R1 = 16, R2 = 16; };

// Stage w_L^j = exp(-2 pi i j / L), j < L, from the device table of
// exp(-2 pi i k / kMaxL) into shared memory: the transforms below read their
// twiddles there (a shared-memory load instead of a global one).
template <int L, typename T2>
__device__ __forceinline__ void stage_twiddles(T2* sw, const T2* __restrict__ tw) {
    // The table is written once per device, before any transform: it is read
    // ahead of the wait for the preceding grid (programmatic launch).  Every
    // two-step kernel starts here, so the wait below orders all of its other
    // global-memory accesses after the grids it follows.
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        if constexpr (std::is_same<T2, ddc>::value)
            sw[j] = tw[j * (kMaxL / L)];
        else
            sw[j] = __ldg(tw + j * (kMaxL / L));
    }
    pdl_wait();
    __syncthreads();
}

template <int L>
struct F2 {
    static constexpr int R1 = Split<L>::R1, R2 = Split<L>::R2;
    static constexpr int NT = R1 > R2 ? R1 : R2;
    static constexpr int S = XS<L>::value;

    // A -> B.  v holds R1 (data) values on entry when t < R2; on exit R2
    // (spectrum) values when t < R1.  `col` is this column's exchange buffer,
    // `sw` the staged twiddles w_L^j.
    // `active` as in inv().
    template <bool INV, typename T2>
    __device__ __forceinline__ static void fwd(T2 (&v)[16], T2* col, int t, const T2* sw, bool active = true) {
        if (active && t < R2) {
            dft<R1, INV>(v);
            T2* cw = col + xrow<R1>(t);
#pragma unroll
            for (int k = 0; k < R1; ++k) cw[k] = v[k];
        }
        __syncthreads();
        if (active && t < R1) {
            const T2* cr = col + t;
#pragma unroll
            for (int r = 0; r < R2; ++r) {
                T2 a = cr[xoff(R1 * r)];
                if (r > 0) {
                    const T2 w = sw[r * t];
                    a = INV ? cmulc(a, w) : cmul(a, w);
                }
                v[r] = a;
            }
            dft<R2, INV>(v);
        }
        __syncthreads();
    }

    // B -> A (unnormalised inverse when INV).  v holds R2 spectrum values on
    // entry when t < R1; on exit R1 data values when t < R2.  `active` false
    // (uniform over each warp) skips the arithmetic but keeps the two
    // barriers, so warps without a column cost almost no issue slots.
    template <bool INV, typename T2>
    __device__ __forceinline__ static void inv(T2 (&v)[16], T2* col, int t, const T2* sw, bool active = true) {
        if (active && t < R1) {
            dft<R2, INV>(v);
            T2* cw = col + xrow<R2>(t);
#pragma unroll
            for (int n1 = 0; n1 < R2; ++n1) {
                T2 a = v[n1];
                if (n1 > 0 && t > 0) {
                    const T2 w = sw[n1 * t];
                    a = INV ? cmulc(a, w) : cmul(a, w);
                }
                cw[n1] = a;
            }
        }
        __syncthreads();
        if (active && t < R2) {
            const T2* cr = col + t;
#pragma unroll
            for (int j = 0; j < R1; ++j) v[j] = cr[xoff(j * R2)];
            dft<R1, INV>(v);
        }
        __syncthreads();
    }
};

}  // namespace sc
