// Tile-sorted CIC deposit (SC_DEPOSIT_TILED) and the matching tile-staged
// gather used by sc_kick.
//
// Cells are grouped in tiles of 8x8x8; a tile's charge lands on its 9x9x9
// nodes.
//   k_tbin     : exact cell index (deposition.jl:39-46), tile id, slot in
//                the tile: a CTA histograms its particles' tiles in shared
//                memory and takes one global atomic per (CTA, tile);
//   scan       : tile offsets and work items (tile chunks of kChunk particles);
//   k_tscatter : records (fx, fy, fz, q, in-tile cell, source index) to tile order;
//   k_tdep     : one CTA per tile chunk accumulates its particles' 8 corner
//                charges into the 729 nodes in shared memory, then adds the
//                non-zero nodes to rho with coalesced atomics;
//   k_tgather  : one CTA per tile chunk stages the tile's 729 packed field
//                nodes in shared memory and interpolates its particles from
//                there, writing each result to the particle's original slot.
// The global atomics drop from 8 per particle to at most 729 per chunk, and
// the gather's 8 scattered node loads per particle become shared-memory
// reads.
#include "cells.cuh"
#include "sc_internal.cuh"

namespace sc {

Axes make_axes(const sc_mesh* m);

constexpr int kTile = 8;                   // cells per tile edge
constexpr int kTN = kTile + 1;             // nodes per tile edge
constexpr int kTNodes = kTN * kTN * kTN;   // 729
constexpr int kChunk = 2048;               // particles per work item
constexpr int kSmemTiles = 8192;           // tiles histogrammed in shared memory
constexpr int kBinPer = 4;                 // particles per thread in k_tbin

template <typename A>
struct TCell;
template <>
struct TCell<float> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, float& f) {
        return cell_df32(x, a, i, f);
    }
    template <typename P>
    __device__ __forceinline__ static float cvt(P v) { return f64_to_f32(v); }
};
template <>
struct TCell<double> {
    template <typename P>
    __device__ __forceinline__ static bool run(P x, const AxisP& a, int& i, double& f) {
        return cell_dp(x, a, i, f);
    }
    template <typename P>
    __device__ __forceinline__ static double cvt(P v) { return (double)v; }
};

template <typename A>
struct TRec {
    A fx, fy, fz, q;
};

struct TileGeom {
    int ntx, nty, ntz, ntiles;
};

template <typename P, typename A>
__global__ void __launch_bounds__(256) k_tbin(const P* __restrict__ px, const P* __restrict__ py,
                                              const P* __restrict__ pz, const P* __restrict__ pq, int64_t n,
                                              Axes ax, TileGeom tg, int* __restrict__ key, int* __restrict__ ticket,
                                              TRec<A>* __restrict__ rec, int* __restrict__ count,
                                              unsigned long long* __restrict__ oob) {
    extern __shared__ int hist[];  // tg.ntiles entries when they fit
    const bool sm = tg.ntiles <= kSmemTiles;
    if (sm) {
        for (int i = threadIdx.x; i < tg.ntiles; i += blockDim.x) hist[i] = 0;
        __syncthreads();
    }
    const int64_t base = (int64_t)blockIdx.x * (blockDim.x * kBinPer) + threadIdx.x;
    int tile[kBinPer], rank[kBinPer];
    unsigned skipped = 0;
#pragma unroll
    for (int k = 0; k < kBinPer; ++k) {
        const int64_t p = base + (int64_t)k * blockDim.x;
        tile[k] = -1;
        if (p >= n) continue;
        int ix, iy, iz;
        TRec<A> r;
        const bool ok = TCell<A>::run(px[p], ax.a[0], ix, r.fx) & TCell<A>::run(py[p], ax.a[1], iy, r.fy) &
                        TCell<A>::run(pz[p], ax.a[2], iz, r.fz);
        if (!ok) {
            key[p] = -1;
            ++skipped;
            continue;
        }
        r.q = TCell<A>::cvt(pq[p]);
        const int t = (ix >> 3) + tg.ntx * ((iy >> 3) + tg.nty * (iz >> 3));
        const int local = (ix & 7) | ((iy & 7) << 3) | ((iz & 7) << 6);
        tile[k] = t;
        key[p] = (t << 9) | local;
        rec[p] = r;
        rank[k] = sm ? atomicAdd(hist + t, 1) : atomicAdd(count + t, 1);
    }
    if (skipped) atomicAdd(oob, (unsigned long long)skipped);
    if (sm) {
        __syncthreads();
        for (int i = threadIdx.x; i < tg.ntiles; i += blockDim.x) {
            const int c = hist[i];
            if (c) hist[i] = atomicAdd(count + i, c);  // this CTA's base slot in tile i
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < kBinPer; ++k) {
        if (tile[k] < 0) continue;
        const int64_t p = base + (int64_t)k * blockDim.x;
        ticket[p] = sm ? hist[tile[k]] + rank[k] : rank[k];
    }
}

// One block: offsets of the tiles and of their work items (chunks).
__global__ void __launch_bounds__(1024) k_tscan(const int* __restrict__ count, int* __restrict__ offset,
                                                int* __restrict__ woff, int ntiles) {
    __shared__ int sm[32];
    __shared__ int carry[2];
    if (threadIdx.x == 0) carry[0] = carry[1] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < ntiles; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int c = i < ntiles ? count[i] : 0;
        int v[2] = {c, (c + kChunk - 1) / kChunk};
        for (int q = 0; q < 2; ++q) {
            int x = v[q];
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) sm[warp] = x;
            __syncthreads();
            if (warp == 0) {
                int s = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0;
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, s, o);
                    if (lane >= o) s += y;
                }
                sm[lane] = s;
            }
            __syncthreads();
            const int excl = (warp ? sm[warp - 1] : 0) + x - v[q] + carry[q];
            const int total = sm[(blockDim.x >> 5) - 1];
            if (i < ntiles) (q == 0 ? offset : woff)[i] = excl;
            __syncthreads();
            if (threadIdx.x == 0) carry[q] += total;
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        offset[ntiles] = carry[0];
        woff[ntiles] = carry[1];
    }
}

template <typename A>
__global__ void __launch_bounds__(256) k_tscatter(const int* __restrict__ key, const int* __restrict__ ticket,
                                                  const TRec<A>* __restrict__ rec, const int* __restrict__ offset,
                                                  TRec<A>* __restrict__ srec, int* __restrict__ skey,
                                                  int* __restrict__ sidx, int64_t n) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int k = key[p];
    if (k < 0) return;
    const int pos = offset[k >> 9] + ticket[p];
    srec[pos] = rec[p];
    skey[pos] = k;
    sidx[pos] = (int)p;
}

// Work item -> (tile, first particle, count) by binary search of woff.
__device__ __forceinline__ bool work_item(int b, const int* __restrict__ woff, const int* __restrict__ offset,
                                          int ntiles, int& tile, int& first, int& cnt) {
    if (b >= woff[ntiles]) return false;
    int lo = 0, hi = ntiles;  // largest t with woff[t] <= b
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (woff[mid] <= b) lo = mid;
        else hi = mid;
    }
    while (lo + 1 <= ntiles && woff[lo + 1] <= b) ++lo;  // skip empty tiles sharing the offset
    tile = lo;
    const int c = b - woff[lo];
    first = offset[lo] + c * kChunk;
    const int end = offset[lo + 1];
    cnt = min(kChunk, end - first);
    return cnt > 0;
}

template <typename A>
__global__ void __launch_bounds__(256) k_tdep(const TRec<A>* __restrict__ srec, const int* __restrict__ skey,
                                              const int* __restrict__ offset, const int* __restrict__ woff,
                                              TileGeom tg, int nx, int ny, int nz, A* __restrict__ rho) {
    __shared__ A acc[kTNodes];
    int tile, first, cnt;
    if (!work_item(blockIdx.x, woff, offset, tg.ntiles, tile, first, cnt)) return;
    for (int i = threadIdx.x; i < kTNodes; i += blockDim.x) acc[i] = A(0);
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const TRec<A> r = srec[first + i];
        const int local = skey[first + i] & 511;
        const int lx = local & 7, ly = (local >> 3) & 7, lz = local >> 6;
        const A wx0 = A(1) - r.fx, wy0 = A(1) - r.fy, wz0 = A(1) - r.fz;
        A* a = acc + lx + kTN * (ly + kTN * lz);
        // deposition.jl:67-74 corner order and products
        atomicAdd(a, r.q * wx0 * wy0 * wz0);
        atomicAdd(a + 1, r.q * r.fx * wy0 * wz0);
        atomicAdd(a + kTN, r.q * wx0 * r.fy * wz0);
        atomicAdd(a + 1 + kTN, r.q * r.fx * r.fy * wz0);
        atomicAdd(a + kTN * kTN, r.q * wx0 * wy0 * r.fz);
        atomicAdd(a + 1 + kTN * kTN, r.q * r.fx * wy0 * r.fz);
        atomicAdd(a + kTN + kTN * kTN, r.q * wx0 * r.fy * r.fz);
        atomicAdd(a + 1 + kTN + kTN * kTN, r.q * r.fx * r.fy * r.fz);
    }
    __syncthreads();
    const int tx = tile % tg.ntx, ty = (tile / tg.ntx) % tg.nty, tz = tile / (tg.ntx * tg.nty);
    for (int i = threadIdx.x; i < kTNodes; i += blockDim.x) {
        const A v = acc[i];
        if (v == A(0)) continue;
        const int gx = tx * kTile + i % kTN, gy = ty * kTile + (i / kTN) % kTN, gz = tz * kTile + i / (kTN * kTN);
        if (gx < nx && gy < ny && gz < nz) atomicAdd(rho + gx + (int64_t)nx * (gy + (int64_t)ny * gz), v);
    }
}

template <typename A>
struct PackedV;
template <>
struct PackedV<float> {
    using V = float4;
};
template <>
struct PackedV<double> {
    using V = dnode4;
};

template <typename P, typename A>
__device__ __forceinline__ P tout(A v);
template <>
__device__ __forceinline__ float tout<float, float>(float v) { return v; }
template <>
__device__ __forceinline__ double tout<double, float>(float v) { return f32_to_f64(v); }
template <>
__device__ __forceinline__ float tout<float, double>(double v) { return (float)v; }
template <>
__device__ __forceinline__ double tout<double, double>(double v) { return v; }

template <typename P, typename A>
__global__ void __launch_bounds__(256) k_tgather(const TRec<A>* __restrict__ srec, const int* __restrict__ skey,
                                                 const int* __restrict__ sidx, const int* __restrict__ offset,
                                                 const int* __restrict__ woff, TileGeom tg, int nx, int ny, int nz,
                                                 const typename PackedV<A>::V* __restrict__ ef, P* __restrict__ ex,
                                                 P* __restrict__ ey, P* __restrict__ ez) {
    using V = typename PackedV<A>::V;
    __shared__ V node[kTNodes];
    int tile, first, cnt;
    if (!work_item(blockIdx.x, woff, offset, tg.ntiles, tile, first, cnt)) return;
    const int tx = tile % tg.ntx, ty = (tile / tg.ntx) % tg.nty, tz = tile / (tg.ntx * tg.nty);
    for (int i = threadIdx.x; i < kTNodes; i += blockDim.x) {
        const int gx = tx * kTile + i % kTN, gy = ty * kTile + (i / kTN) % kTN, gz = tz * kTile + i / (kTN * kTN);
        V v{};
        if (gx < nx && gy < ny && gz < nz) v = ef[gx + (int64_t)nx * (gy + (int64_t)ny * gz)];
        node[i] = v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const TRec<A> r = srec[first + i];
        const int local = skey[first + i] & 511;
        const int lx = local & 7, ly = (local >> 3) & 7, lz = local >> 6;
        const A ux = A(1) - r.fx, uy = A(1) - r.fy, uz = A(1) - r.fz;
        // interpolation.jl:46-53 weights, corners in the order of :56-85
        const A w[8] = {ux * uy * uz, r.fx * uy * uz, ux * r.fy * uz, r.fx * r.fy * uz,
                        ux * uy * r.fz, r.fx * uy * r.fz, ux * r.fy * r.fz, r.fx * r.fy * r.fz};
        const V* b = node + lx + kTN * (ly + kTN * lz);
        const int off[8] = {0, 1, kTN, 1 + kTN, kTN * kTN, 1 + kTN * kTN, kTN + kTN * kTN, 1 + kTN + kTN * kTN};
        A sx = 0, sy = 0, sz = 0;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const V v = b[off[c]];
            sx += v.x * w[c];
            sy += v.y * w[c];
            sz += v.z * w[c];
        }
        const int p = sidx[first + i];
        ex[p] = tout<P, A>(sx);
        ey[p] = tout<P, A>(sy);
        ez[p] = tout<P, A>(sz);
    }
}

struct TileWork {
    int64_t cap_n = 0;
    int cap_tiles = 0;
    int *key = nullptr, *ticket = nullptr, *skey = nullptr, *sidx = nullptr;
    int *count = nullptr, *offset = nullptr, *woff = nullptr;
    void *rec = nullptr, *srec = nullptr;
    TileGeom tg;
    int64_t n = 0;           // particles binned by the last tiled deposit
    const void* src = nullptr;  // their x pointer (identifies the binning for the gather)
};

static TileGeom tile_geom(const sc_mesh* m) {
    TileGeom g;
    g.ntx = (m->n[0] - 1 + kTile - 1) / kTile;
    g.nty = (m->n[1] - 1 + kTile - 1) / kTile;
    g.ntz = (m->n[2] - 1 + kTile - 1) / kTile;
    g.ntiles = g.ntx * g.nty * g.ntz;
    return g;
}

template <typename P, typename A>
static int tiled_t(sc_mesh* m, const P* x, const P* y, const P* z, const P* q, int64_t n, cudaStream_t s) {
    TileWork* w = reinterpret_cast<TileWork*>(m->tilework);
    if (!w) {
        w = new TileWork();
        m->tilework = w;
    }
    const TileGeom tg = tile_geom(m);
    if (tg.ntiles >= (1 << 22)) return fail(SC_ERR_UNSUPPORTED, "mesh too large for the tiled deposit");
    w->src = nullptr;  // no binning for the gather until this one is issued
    // capacity 0 until every buffer of the set is in place: a failed
    // allocation leaves the set to be reallocated by the next call
    if (w->cap_n < n) {
        w->cap_n = 0;
        SC_CUDA(dev_realloc(&w->key, sizeof(int) * n));
        SC_CUDA(dev_realloc(&w->ticket, sizeof(int) * n));
        SC_CUDA(dev_realloc(&w->skey, sizeof(int) * n));
        SC_CUDA(dev_realloc(&w->sidx, sizeof(int) * n));
        SC_CUDA(dev_realloc(&w->rec, sizeof(TRec<double>) * n));
        SC_CUDA(dev_realloc(&w->srec, sizeof(TRec<double>) * n));
        w->cap_n = n;
    }
    if (w->cap_tiles < tg.ntiles) {
        w->cap_tiles = 0;
        SC_CUDA(dev_realloc(&w->count, sizeof(int) * (tg.ntiles + 1)));
        SC_CUDA(dev_realloc(&w->offset, sizeof(int) * (tg.ntiles + 1)));
        SC_CUDA(dev_realloc(&w->woff, sizeof(int) * (tg.ntiles + 1)));
        w->cap_tiles = tg.ntiles;
    }
    w->tg = tg;
    w->n = n;
    w->src = x;
    const Axes ax = make_axes(m);
    SC_CUDA(cudaMemsetAsync(w->count, 0, sizeof(int) * (tg.ntiles + 1), s));
    const size_t hsm = tg.ntiles <= kSmemTiles ? sizeof(int) * tg.ntiles : 0;
    const int64_t bblocks = (n + 256 * kBinPer - 1) / (256 * kBinPer);
    k_tbin<P, A><<<bblocks, 256, hsm, s>>>(x, y, z, q, n, ax, tg, w->key, w->ticket, (TRec<A>*)w->rec, w->count,
                                           m->oob);
    SC_LAUNCH_CHECK("k_tbin");
    k_tscan<<<1, 1024, 0, s>>>(w->count, w->offset, w->woff, tg.ntiles);
    SC_LAUNCH_CHECK("k_tscan");
    k_tscatter<A><<<(n + 255) / 256, 256, 0, s>>>(w->key, w->ticket, (const TRec<A>*)w->rec, w->offset,
                                                  (TRec<A>*)w->srec, w->skey, w->sidx, n);
    SC_LAUNCH_CHECK("k_tscatter");
    const int64_t items = n / kChunk + tg.ntiles + 1;  // upper bound on work items
    k_tdep<A><<<items, 256, 0, s>>>((const TRec<A>*)w->srec, w->skey, w->offset, w->woff, tg, m->n[0], m->n[1],
                                    m->n[2], (A*)m->rho);
    SC_LAUNCH_CHECK("k_tdep");
    m->launches += 4;
    return SC_OK;
}

int deposit_tiled_launch(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n,
                         int dtype, cudaStream_t s) {
    if (m->precision == SC_PREC_PLAIN64)
        return fail(SC_ERR_UNSUPPORTED, "the tiled deposit needs a hand-written pipeline mesh (fp64 or mixed)");
    if (n > (int64_t)0x7fffffff) return fail(SC_ERR_UNSUPPORTED, "the tiled deposit supports at most 2^31-1 particles");
    if (m->precision == SC_PREC_MIXED) {
        if (dtype == SC_F64)
            return tiled_t<double, float>(m, (const double*)x, (const double*)y, (const double*)z, (const double*)q,
                                          n, s);
        return tiled_t<float, float>(m, (const float*)x, (const float*)y, (const float*)z, (const float*)q, n, s);
    }
    if (dtype == SC_F64)
        return tiled_t<double, double>(m, (const double*)x, (const double*)y, (const double*)z, (const double*)q, n,
                                       s);
    return tiled_t<float, double>(m, (const float*)x, (const float*)y, (const float*)z, (const float*)q, n, s);
}

// Gather from the binning of the last tiled deposit of these particles (the
// caller guarantees they have not moved since, as inside sc_kick).
int gather_tiled_launch(sc_mesh* m, const void* x, int64_t n, int dtype, void* ex, void* ey, void* ez,
                        cudaStream_t s) {
    TileWork* w = reinterpret_cast<TileWork*>(m->tilework);
    if (!w || w->n != n || w->src != x) return fail(SC_ERR_INVALID, "no tiled binning of these particles");
    const int64_t items = n / kChunk + w->tg.ntiles + 1;
    const int nx = m->n[0], ny = m->n[1], nz = m->n[2];
    // particles outside the mesh are in no tile; their field is zero, as in
    // the packed gather
    const size_t bytes = (size_t)n * (dtype == SC_F64 ? 8 : 4);
    SC_CUDA(cudaMemsetAsync(ex, 0, bytes, s));
    SC_CUDA(cudaMemsetAsync(ey, 0, bytes, s));
    SC_CUDA(cudaMemsetAsync(ez, 0, bytes, s));
    if (m->precision == SC_PREC_MIXED) {
        if (dtype == SC_F64)
            k_tgather<double, float><<<items, 256, 0, s>>>((const TRec<float>*)w->srec, w->skey, w->sidx, w->offset,
                                                           w->woff, w->tg, nx, ny, nz, (const float4*)m->efield,
                                                           (double*)ex, (double*)ey, (double*)ez);
        else
            k_tgather<float, float><<<items, 256, 0, s>>>((const TRec<float>*)w->srec, w->skey, w->sidx, w->offset,
                                                          w->woff, w->tg, nx, ny, nz, (const float4*)m->efield,
                                                          (float*)ex, (float*)ey, (float*)ez);
    } else {
        if (dtype == SC_F64)
            k_tgather<double, double><<<items, 256, 0, s>>>((const TRec<double>*)w->srec, w->skey, w->sidx,
                                                            w->offset, w->woff, w->tg, nx, ny, nz,
                                                            (const dnode4*)m->efield, (double*)ex, (double*)ey,
                                                            (double*)ez);
        else
            k_tgather<float, double><<<items, 256, 0, s>>>((const TRec<double>*)w->srec, w->skey, w->sidx,
                                                           w->offset, w->woff, w->tg, nx, ny, nz,
                                                           (const dnode4*)m->efield, (float*)ex, (float*)ey,
                                                           (float*)ez);
    }
    SC_LAUNCH_CHECK("k_tgather");
    m->launches += 1;
    return SC_OK;
}

void tiled_release(sc_mesh* m) {
    TileWork* w = reinterpret_cast<TileWork*>(m->tilework);
    if (!w) return;
    void* ptrs[] = {w->key, w->ticket, w->skey, w->sidx, w->count, w->offset, w->woff, w->rec, w->srec};
    for (void* p : ptrs) cudaFree(p);
    delete w;
    m->tilework = nullptr;
}

}  // namespace sc
