// Staged batch kick: the per-bunch table that the multi-bunch stage kernels
// read.  sc_batch_kick runs each stage of the kick (clear, deposit, node sum,
// forward transforms, z pass, inverse y+x, gather) as one launch over a group
// of bunches instead of one launch per bunch and stage.  A launch's CTAs are
// mapped to bunches through a table of CtaRef, one per CTA, built on the host
// when the batch's arguments change.
#pragma once

#include "cells.cuh"
#include "pipeline.cuh"

namespace sc {

// One bunch of a staged batch, as its stage kernels see it.
struct BunchDesc {
    const void* x;
    const void* y;
    const void* z;
    const void* q;
    void* ex;
    void* ey;
    void* ez;
    int64_t n;  // particles
    Axes ax;    // mesh geometry (cell-index arithmetic of the deposit and gather)
    float* rho;
    float4* corner;  // per-cell corner slots of the vector deposit; null: scalar atomics into rho
    float4* efield;  // packed (Ex, Ey, Ez, 0) nodes
    unsigned long long* oob;
    int nx, ny, nz, Hx, Ly;
    float2* A;  // forward x output (two-pass forward transform), Hx x ny x nz
    float2* B;  // forward x+y output, Hx x Ly x nz
    float2* C;  // z pass output, 3 x Hx x Ly x nz
    GreenView gv;
};

// A contiguous range of floats to zero (kb_clear).
struct ClearSeg {
    float* p;
    int64_t n;
};

// CTA -> (table entry, CTA index within that entry) of a staged launch.
struct CtaRef {
    int item;
    int local;
};

// The mesh's geometry as the deposit and gather kernels take it (deposit.cu).
Axes make_axes(const sc_mesh* m);

// columns per CTA of the z pass and the column passes (pipeline2.cuh kColW)
constexpr int kBatchZCols = 16;

// Floats one kb_clear CTA zeroes.
constexpr int kClearChunk = 256 * 4 * 16;

// ---- launchers (deposit.cu, gather.cu, batch_fft.cu); `map` holds `ctas`
// CtaRef for this launch.  Each returns SC_OK or an error after a failed
// launch.
int batch_clear_launch(const ClearSeg* segs, const CtaRef* map, int64_t ctas, cudaStream_t s);
// particles per CTA of kb_deposit and of kb_gather
int batch_deposit_particles_per_cta();
int batch_gather_particles_per_cta();
// allocates the mesh's corner slots of the vector deposit if it has none
int corner_alloc(sc_mesh* m);
int batch_deposit_launch(const BunchDesc* tab, const CtaRef* map, int64_t ctas, int dtype, cudaStream_t s);
int batch_corner_sum_launch(const BunchDesc* tab, const CtaRef* map, int64_t ctas, cudaStream_t s);
int batch_gather_launch(const BunchDesc* tab, const CtaRef* map, int64_t ctas, int dtype, cudaStream_t s);
// transform passes of one grid class (transform length 2^logL along x and y,
// 2^logLz along z); smem_plane: the largest ny * Hx of the group
int batch_fwd_xy_launch(int logL, const BunchDesc* tab, const CtaRef* map, int64_t ctas, size_t smem_plane,
                        cudaStream_t s);
// the forward x and y passes as two launches (the fused pass's alternative)
int batch_fwd_x_launch(int logL, const BunchDesc* tab, const CtaRef* map, int64_t ctas, cudaStream_t s);
int batch_fwd_y_launch(int logL, const BunchDesc* tab, const CtaRef* map, int64_t ctas, cudaStream_t s);
// CTAs of those two passes for one bunch
int64_t batch_fwd_x_ctas(int logL, int64_t rows);
int64_t batch_fwd_y_ctas(int64_t columns);
int batch_zpass_launch(int logLz, const BunchDesc* tab, const CtaRef* map, int64_t ctas, bool image,
                       cudaStream_t s);
int batch_inv_yx_launch(int logL, const BunchDesc* tab, const CtaRef* map, int64_t ctas, size_t smem_plane,
                        cudaStream_t s);
// shared memory (bytes) of the fused plane passes for a plane of ny x Hx
size_t batch_plane_smem(int logL, int64_t plane);

}  // namespace sc
