// Column tiles of the z passes and their asynchronous shared-memory
// staging, shared by the FP32 kernels of pipeline2.cuh and the FP64
// double-FP32 z pass (dd_passes.cu).
#pragma once

#include "pipeline.cuh"

namespace sc {

constexpr int kColW = 16;  // columns per CTA of the column passes

// MACRO(L) for the transform length 2^logL, 4..256 (the register two-step
// lengths); any other length makes the enclosing function return false
#define SC_L_SWITCH(logL, MACRO) \
    switch (logL) {              \
        case 2: MACRO(4); break; \
        case 3: MACRO(8); break; \
        case 4: MACRO(16); break; \
        case 5: MACRO(32); break; \
        case 6: MACRO(64); break; \
        case 7: MACRO(128); break; \
        case 8: MACRO(256); break; \
        default: return false;   \
    }

// Asynchronous 4-byte global -> shared copies (cp.async, sm_80+), waited
// for with cp_async_wait_all before a barrier.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Copies this CTA's free-space Green values, gsm[comp][kzf][column] for
// kzf <= L/2 and the tile's kColW columns (kx, ky folded to ky <= Ly/2), to
// shared memory asynchronously; cp_async_wait_all + a barrier before use.
// blockDim.x is a multiple of kColW, so each thread keeps one column.
// G: the Green function's real type (float, or double on FP64 meshes).
template <int L, typename G = float>
__device__ __forceinline__ void prefetch_green(G* gsm, const GreenView& gv, int Hx, int Ly, int tile) {
    constexpr int HZ = L / 2 + 1;
    const int64_t plane = (int64_t)Hx * Ly;
    const int64_t gstep = (int64_t)gv.Hx * gv.Hy;
    const int cc = threadIdx.x % kColW;
    const int ff = tile * kColW + cc;
    if (ff < plane) {
        const int kyy = ff / Hx, kxx = ff - kyy * Hx;
        const int kyf = kyy <= Ly / 2 ? kyy : Ly - kyy;
        const G* src = reinterpret_cast<const G*>(gv.gfree) + kxx + (int64_t)gv.Hx * kyf;
        const int k0 = threadIdx.x / kColW, kstep = blockDim.x / kColW;
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            const G* sc = src + comp * gv.cs_free + gstep * k0;
            G* dc = gsm + (comp * HZ + k0) * kColW + cc;
            for (int kzf = k0; kzf < HZ; kzf += kstep, sc += gstep * kstep, dc += kColW * kstep) {
                if constexpr (sizeof(G) == 4)
                    cp_async4(dc, sc);
                else
                    cp_async8(dc, sc);
            }
        }
    }
    cp_async_commit();
}

}  // namespace sc
