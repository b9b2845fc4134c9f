// Internal declarations shared by the CUDA translation units of
// libspacecharge_gb300.so.  Nothing here is part of the public C ABI.
#pragma once

#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/spacecharge_gb300.h"

namespace sc {

// src/utils.jl:7-8
constexpr double kClight = 299792458.0;
constexpr double kFpei = kClight * kClight * 1.0e-7;

// Antiderivative of 1/r, potential_green_function of
// src/green_functions.jl:13-22 (defined in the reference, not called there):
// zero at r = 0, the same expression and order.
__device__ __forceinline__ double potential_green_n(double x, double y, double z) {
    const double r = sqrt(x * x + y * y + z * z);
    if (r == 0.0) return 0.0;
    const double half = 0.5;
    return -half * z * z * atan(x * y / (z * r)) - half * y * y * atan(x * z / (y * r)) -
           half * x * x * atan(y * z / (x * r)) + y * z * log(x + r) + x * z * log(y + r) + x * y * log(z + r);
}

// Packed FP64 field node (Ex, Ey, Ez, 0); 32-byte aligned.
struct __align__(32) dnode4 {
    double x, y, z, w;
};

// Longest transform per axis of the hand-written FFT (power of two).
constexpr int kMaxL = 1024;
constexpr int kMaxLog = 10;

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

#define SC_CUDA(call)                                            \
    do {                                                         \
        cudaError_t _e = (call);                                 \
        if (_e != cudaSuccess) return ::sc::cuda_fail(_e, #call); \
    } while (0)

// Every device buffer of the library comes from dev_alloc.  On failure *p is
// null and the runtime's last-error slot is cleared, so the next launch check
// does not report the failed allocation again.  sc_test_fail_allocations
// makes it fail on demand, without calling the runtime.
cudaError_t dev_alloc(void** p, size_t bytes);
// Frees *p, then allocates `bytes` in its place (*p null on failure).
cudaError_t dev_realloc(void** p, size_t bytes);
template <typename T>
inline cudaError_t dev_alloc(T** p, size_t bytes) {
    return dev_alloc(reinterpret_cast<void**>(p), bytes);
}
template <typename T>
inline cudaError_t dev_realloc(T** p, size_t bytes) {
    return dev_realloc(reinterpret_cast<void**>(p), bytes);
}

#define SC_LAUNCH_CHECK(what)                                    \
    do {                                                         \
        cudaError_t _e = cudaGetLastError();                     \
        if (_e != cudaSuccess) return ::sc::cuda_fail(_e, what); \
    } while (0)

#define SC_TRY(...)                       \
    do {                                  \
        int _s = (__VA_ARGS__);           \
        if (_s != SC_OK) return _s;       \
    } while (0)

// ------------------------------------------- programmatic dependent launch
// The kernels of the kick's stream chains are launched with programmatic
// stream serialization: a kernel is scheduled as the blocks of the one before
// it retire, and runs its independent prologue (twiddle staging, index
// arithmetic) before pdl_wait().  pdl_wait() returns once every preceding
// grid has completed and its writes are visible, so every kernel launched
// through launch_pdl calls it before its first global memory access that
// reads earlier results or writes what earlier kernels read.  In a kernel
// launched normally it is a no-op.  No kernel triggers its dependents early
// (griddepcontrol.launch_dependents): dependents resident ahead of time made
// the captured kick 10 % slower, while launch at block retirement makes it
// 2 % faster and the adjoint 8 % faster.  SC_PDL=0 in the environment
// launches everything normally.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

bool pdl_enabled();

template <typename... P, typename... A>
inline void launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    // a failure is left in the runtime's last-error slot for SC_LAUNCH_CHECK
    (void)cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

// ------------------------------------------------------- per-device state
struct DeviceCtx {
    int device = -1;
    float2* tw32 = nullptr;   // exp(-2 pi i k / kMaxL), k < kMaxL, FP32
    double2* tw64 = nullptr;  // the same in FP64
    void* twdd = nullptr;     // the same as double-FP32 pairs (ddc, dd.cuh): {hi re, hi im}, {lo re, lo im}
    double* partials = nullptr;  // bounds reduction partials
    int partial_blocks = 0;
    double* ext_host = nullptr;  // the reduction's 6 extrema: page-locked, mapped,
    double* ext_dev = nullptr;   // written by the final kernel through ext_dev
    unsigned long long ext_seq = 0;  // sequence number the final kernel writes after them
    int sm_count = 0;
};
int device_ctx(DeviceCtx** out);  // for the current device
int fft_engine();                 // 0 = register two-step where possible, 1 = Stockham only
// autotuned (engine, lgW) for a transform shape, if any (returns false if none)
bool tuned_choice(int device, int precision, const int L[3], int* engine, int* lgW);

// ----------------------------------------------------------- Green cache
struct GreenKey {
    double delta[3];
    double gamma;
    double offset_z;
    int fmt = 0;  // 0: the mesh's real type; 1: double-FP32 (dreal), for the double-FP32 z pass
    bool valid = false;
};

// ------------------------------------------------------------------ mesh
struct NativeWork {
    // transform lengths and half-spectrum width
    int L[3] = {0, 0, 0};
    int log2L[3] = {0, 0, 0};
    int Hx = 0;
    size_t elem = 0;        // sizeof(T2) of the pipeline
    void* A = nullptr;      // Hx x ny x nz            (after x pass)
    void* B = nullptr;      // Hx x Ly x nz            (after y pass)
    void* C = nullptr;      // 3 x Hx x Ly x nz        (after z pass)
    void* D = nullptr;      // 3 x Hx x ny x nz        (after inverse y)
    void* adjE = nullptr;   // adjoint: 3 x N accumulated dL/dE (T)
    void* adjcorner = nullptr;  // adjoint, mixed: 3 x 8N per-cell corner slots (float)
    // Green function construction
    double* fcorner = nullptr;  // FP64 antiderivative on corner lattice
    double* fnear = nullptr;    // FP32 path: FP64 antiderivative on the near-box corners
    int64_t fnear_cap = 0;
    void* kgrid = nullptr;      // real kernel on the L grid (T)
    void* kspec = nullptr;      // its half spectrum (T2), Hx x Ly x Lz
    void* goct = nullptr;       // FP32 path: kernel values on the octant/quadrant, 3 comps
    void* goct_img = nullptr;   //   the image build's own scratch (the two builds can run concurrently)
    void* gtmp_img = nullptr;
    double* fnear_img = nullptr;
    int64_t fnear_img_cap = 0;
    void* gspec = nullptr;      // FP32 Stockham path: 3 half spectra Hx x Ly x Lz being transformed
    void* gtmp = nullptr;       // FP32 two-step path: parity-reduced x and y pass outputs (float)
    void* gfree = nullptr;      // compressed free-space spectra, 3 comps (T)
    void* gimg = nullptr;       // compressed image spectra, 3 comps (T2)
    GreenKey key_free, key_img;
    bool img_half = false;  // gimg holds kz <= Lz/2 only (the FP32 two-step build)
    int engine = -1;  // -1: process-wide setting; 0: two-step; 1: Stockham
    int lgW = -1;     // Stockham column tile (log2), -1: default
    // scalar potential (potential.cu): compressed spectra of the potential
    // kernel (free space: real, T, Hx x Hy x Hz; image: complex, T2, kz <= Lz/2)
    // and the scratch of their build
    void* pfree = nullptr;
    void* pimg = nullptr;
    void* pscratch = nullptr;
    int64_t pscratch_cap = 0;
    GreenKey key_pfree, key_pimg;
};

struct PlainWork {
    cufftHandle plan = 0;
    bool plan_ok = false;
    double2* crho = nullptr;
    double2* cgrn = nullptr;
    double2* tmp = nullptr;
};

}  // namespace sc

namespace sc {
// CUDA-event stage timer (used only while profiling is enabled).
struct StageTimer {
    bool enabled = false;
    struct Pair {
        cudaEvent_t a, b;
    };
    std::vector<Pair> ev[SC_NUM_STAGES];
    size_t used[SC_NUM_STAGES] = {};
    int open_stage = -1;
    void begin(int stage, cudaStream_t s);
    void end(cudaStream_t s);
    void release();
};
// NVTX range names of the stages (visible to nsys/ncu NVTX filters)
const char* stage_name(int stage);

// RAII bracket: `StageScope t(m, SC_STAGE_X, s);` -- an NVTX range on the
// host always, CUDA events on the stream when the mesh's profiling is on.
struct StageScope {
    StageTimer* t;
    cudaStream_t s;
    StageScope(StageTimer& tm, int stage, cudaStream_t st) : t(&tm), s(st) {
        nvtxRangePushA(stage_name(stage));
        if (t->enabled) t->begin(stage, s);
    }
    ~StageScope() {
        if (t->enabled) t->end(s);
        nvtxRangePop();
    }
};
}  // namespace sc

struct sc_mesh {
    int n[3];
    int64_t N;
    double lo[3], hi[3], delta[3];
    double gamma, total_charge;
    int precision;
    int device;
    bool green_cache = true;
    bool df32 = false;  // FP64 meshes: transforms and gather in double-FP32 (sc_mesh_set_fp64_arithmetic)
    void* rho = nullptr;     // T[N]
    void* efield = nullptr;  // planar T[3N] or packed T[4N]
    unsigned long long* oob = nullptr;  // device counter of skipped particles
    sc::NativeWork nw;
    sc::PlainWork pw;
    sc::StageTimer timer;
    int64_t launches = 0;     // kernels launched by this mesh
    void* sortwork = nullptr; // sorted-deposit buffers (deposit_sorted.cu)
    void* tilework = nullptr; // tiled-deposit buffers (deposit_tiled.cu)
    void* corner = nullptr;   // vector-deposit per-cell corners, float[8N]
    cudaStream_t side = nullptr;  // Green build concurrent with the deposit (native_green_async)
    cudaStream_t side2 = nullptr; // the image build, beside the free-space one
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr;
    bool kick_graph = true;       // sc_kick replays a captured graph on repeated calls
    void* kickgraph = nullptr;    // its state (api.cu)
    void* hostpipe = nullptr;     // sc_kick_host staging buffers and copy streams (api.cu)
    void* trackE = nullptr;       // sc_track: E at the particles, 3 x track_cap
    int64_t track_cap = 0;
    size_t track_elem = 0;
    int kick_mode = SC_DEPOSIT_ATOMIC;  // deposit mode of sc_kick
    int64_t green_epoch = 0;            // bumped by every Green spectrum build
    // largest shared-memory plane of the fused inverse y+x pass: 100 KB keeps
    // two CTAs per SM; batch_issue raises it while other bunches run beside
    size_t fused_smem_cap = 100 * 1024;
    // set by batch_issue while other bunches' kernels run beside this mesh's
    bool beside_others = false;
    // set by the host-buffer kick: its Green build, started beside the H2D
    // copies, has finished before the solve's forward passes run
    bool green_ahead = false;
};

namespace sc {

// Makes a mesh's device current for the scope of an entry point.
struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

inline size_t field_elem_bytes(int precision) {
    return precision == SC_PREC_MIXED ? 4 : 8;
}

// Kernel-side mesh geometry, passed by value.
struct Geom {
    int n[3];
    double lo[3];
    double delta[3];
    double inv[3];  // 1/delta rounded to FP64
};
Geom make_geom(const sc_mesh* m);

// entry points implemented per translation unit -------------------------
int bounds_reduce(const void* x, const void* y, const void* z, int64_t n, int dtype,
                  double mins[3], double maxs[3], cudaStream_t s);

// assign: the deposit writes rho instead of adding to it, where
// deposit_assigns(m, mode) (the vector deposit's node sum); rho is then not
// cleared beforehand
int deposit_launch(sc_mesh* m, const void* x, const void* y, const void* z, const void* q,
                   int64_t n, int dtype, int mode, cudaStream_t s, bool assign = false);
bool deposit_assigns(const sc_mesh* m, int mode);
// out[node] += sum of the node's entries in the 8 cells around it (float[8N]
// per-cell corner slots, the vector deposit's layout)
int corner_sum_launch(sc_mesh* m, const float* corner, float* out, cudaStream_t s, bool assign = false);
// chunked deposit of sc_kick_host (deposit.cu)
bool deposit_chunkable(const sc_mesh* m, int mode);
int deposit_chunk_begin(sc_mesh* m, int mode, cudaStream_t s);
int deposit_chunk_add(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
                      int mode, cudaStream_t s);
int deposit_chunk_finish(sc_mesh* m, int mode, cudaStream_t s);
// the kick as stream work, without graph replay (api.cu)
int kick_issue(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
               int at_cathode, void* ex, void* ey, void* ez, cudaStream_t s);
void kick_graph_release(sc_mesh* m);
// Appends what a captured kick of this mesh depends on besides its arguments:
// flags, tuning choices, geometry (kernel arguments captured by value), the
// Green epoch (cached spectra) and the allocation generation (workspace
// addresses).  A graph replays only while this is unchanged.  Without the
// epoch (with_epoch = false) it keys what a batch's stage plan depends on.
void mesh_state_key(const sc_mesh* m, std::vector<int64_t>& k, bool with_epoch = true);
// Counts device allocations and frees made through dev_alloc / dev_realloc.
int64_t alloc_generation();
void host_pipe_release(sc_mesh* m);
// new bounds for a mesh (sc_track's refit); cached spectra and graphs see the
// change through their keys
int mesh_set_geometry(sc_mesh* m, const double lo[3], const double hi[3], const double delta[3]);
// true when the next solve would (re)build a Green spectrum
// dd_ok: the caller's z pass takes a double-FP32 free-space spectrum (every
// forward solve; not the FP64 adjoint's z pass)
bool native_green_stale(const sc_mesh* m, int at_cathode, bool dd_ok = true);
// early: load the positions before waiting for the preceding grid (only
// where no preceding grid writes them: the kick, after its own passes)
int gather_launch(sc_mesh* m, const void* x, const void* y, const void* z, int64_t n,
                  int dtype, void* ex, void* ey, void* ez, cudaStream_t s, bool early = false);

int cell_index_launch(sc_mesh* m, const void* x, const void* y, const void* z, int64_t n, int dtype,
                      int32_t* idx, double* frac, cudaStream_t s);

void sorted_release(sc_mesh* m);
void tiled_release(sc_mesh* m);
int deposit_tiled_launch(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n,
                         int dtype, cudaStream_t s);
int gather_tiled_launch(sc_mesh* m, const void* x, int64_t n, int dtype, void* ex, void* ey, void* ez,
                        cudaStream_t s);

int plain_solve(sc_mesh* m, int at_cathode, cudaStream_t s);
int plain_potential(sc_mesh* m, int at_cathode, void* phi, cudaStream_t s);
int plain_release(sc_mesh* m);

int native_prepare(sc_mesh* m);  // sizes only (no allocation)
// green_ready: the Green spectra of this solve are being built on another
// stream and are complete when this event fires (native_green_async)
int native_solve(sc_mesh* m, int at_cathode, cudaStream_t s, cudaEvent_t green_ready = nullptr);
// When the next solve would build Green spectra, starts that build on the
// mesh's side stream (forked from s) and returns in *ready the event that
// marks its end; otherwise *ready = nullptr.  The spectra do not depend on
// rho, so the caller's deposit overlaps the build.
int native_green_async(sc_mesh* m, int at_cathode, cudaStream_t s, cudaEvent_t* ready, bool dd_ok = true);
int native_ensure_green(sc_mesh* m, int at_cathode, cudaStream_t s, bool dd_ok = true);
int native_autotune(sc_mesh* m, cudaStream_t s, int* choice);
int native_solve_noalloc(const int32_t* grid, const double* delta, double gamma, const float* rho, float* efield,
                         cudaStream_t s);
int adjoint_launch(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
                   int at_cathode, const void* gex, const void* gey, const void* gez, const void* ggrid, void* dx,
                   void* dy, void* dz, void* dq, cudaStream_t s);
int native_release(sc_mesh* m);
// the forward x and y transforms of the mesh's rho into the workspace's B
// (the field solve's, alone on the GPU: fused where the plane fits)
// dd: FP64 meshes, the forward passes in double-FP32 (native_dd_applies)
int native_forward(sc_mesh* m, cudaStream_t s, bool dd = false);
// FP64 mesh in double-FP32 mode whose lengths fit the double-FP32 passes
bool native_dd_applies(const sc_mesh* m);
// scalar potential of the mesh's rho on the hand-written pipeline (T phi[N],
// x fastest); SC_ERR_UNSUPPORTED where a transform is longer than 256
int native_potential(sc_mesh* m, int at_cathode, void* phi, cudaStream_t s);

}  // namespace sc
