// C-ABI entry points: argument validation with the reference's error
// messages, mesh lifecycle and dispatch to the kernels of each precision.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "sc_internal.cuh"

namespace sc {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    return e == cudaErrorMemoryAllocation ? SC_ERR_OOM : SC_ERR_CUDA;
}

// ----------------------------------------------------- device allocation
// Successful allocations still allowed before injected failures (< 0: none).
static std::atomic<int64_t> g_alloc_allow{-1};
static std::atomic<int64_t> g_alloc_gen{0};

int64_t alloc_generation() { return g_alloc_gen.load(); }

cudaError_t dev_alloc(void** p, size_t bytes) {
    *p = nullptr;
    int64_t left = g_alloc_allow.load();
    while (left >= 0) {
        if (left == 0) return cudaErrorMemoryAllocation;
        if (g_alloc_allow.compare_exchange_weak(left, left - 1)) break;
    }
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        (void)cudaGetLastError();
        return e;
    }
    g_alloc_gen.fetch_add(1);
    return e;
}

cudaError_t dev_realloc(void** p, size_t bytes) {
    if (*p) {
        cudaFree(*p);
        *p = nullptr;
        g_alloc_gen.fetch_add(1);
    }
    return dev_alloc(p, bytes);
}

// ------------------------------------------------------- per-device state
static std::mutex g_ctx_mu;
static std::vector<DeviceCtx*> g_ctx;

static int device_ctx_init(DeviceCtx* c, int dev) {
    SC_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, dev));
    // Twiddle table exp(-2 pi i k / kMaxL) built in FP64 from sin/cos of
    // exactly representable multiples of pi/2^kMaxLog: each FP32 entry is the
    // correctly rounded FP64 value.
    std::vector<float2> t32(kMaxL);
    std::vector<double2> t64(kMaxL);
    std::vector<float4> tdd(kMaxL);  // double-FP32: hi (re, im), lo (re, im)
    for (int k = 0; k < kMaxL; ++k) {
        long double a = -2.0L * 3.141592653589793238462643383279502884L * (long double)k / (long double)kMaxL;
        const long double cl = cosl(a), sl = sinl(a);
        double c = (double)cl, s = (double)sl;
        t64[k] = make_double2(c, s);
        t32[k] = make_float2((float)c, (float)s);
        const float ch = (float)cl, sh = (float)sl;
        tdd[k] = make_float4(ch, sh, (float)(cl - (long double)ch), (float)(sl - (long double)sh));
    }
    SC_CUDA(dev_alloc(&c->tw32, sizeof(float2) * kMaxL));
    SC_CUDA(dev_alloc(&c->tw64, sizeof(double2) * kMaxL));
    SC_CUDA(dev_alloc(&c->twdd, sizeof(float4) * kMaxL));
    SC_CUDA(cudaMemcpy(c->tw32, t32.data(), sizeof(float2) * kMaxL, cudaMemcpyHostToDevice));
    SC_CUDA(cudaMemcpy(c->tw64, t64.data(), sizeof(double2) * kMaxL, cudaMemcpyHostToDevice));
    SC_CUDA(cudaMemcpy(c->twdd, tdd.data(), sizeof(float4) * kMaxL, cudaMemcpyHostToDevice));
    c->partial_blocks = 2 * c->sm_count;
    SC_CUDA(dev_alloc(&c->partials, sizeof(double) * 6 * (c->partial_blocks + 1)));
    SC_CUDA(cudaHostAlloc((void**)&c->ext_host, sizeof(double) * 8, cudaHostAllocMapped));
    SC_CUDA(cudaHostGetDevicePointer((void**)&c->ext_dev, c->ext_host, 0));
    return SC_OK;
}

int device_ctx(DeviceCtx** out) {
    int dev = 0;
    SC_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    if ((int)g_ctx.size() <= dev) g_ctx.resize(dev + 1, nullptr);
    if (g_ctx[dev]) {
        *out = g_ctx[dev];
        return SC_OK;
    }
    DeviceCtx* c = new DeviceCtx();
    c->device = dev;
    const int st = device_ctx_init(c, dev);
    if (st != SC_OK) {
        cudaFree(c->tw32);
        cudaFree(c->tw64);
        cudaFree(c->twdd);
        cudaFree(c->partials);
        if (c->ext_host) cudaFreeHost(c->ext_host);
        delete c;
        return st;
    }
    g_ctx[dev] = c;
    *out = c;
    return SC_OK;
}

bool pdl_enabled() {
    static const bool on = [] {
        const char* e = getenv("SC_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

static std::atomic<int> g_fft_engine{0};
int fft_engine() { return g_fft_engine.load(std::memory_order_relaxed); }

Geom make_geom(const sc_mesh* m) {
    Geom g;
    for (int d = 0; d < 3; ++d) {
        g.n[d] = m->n[d];
        g.lo[d] = m->lo[d];
        g.delta[d] = m->delta[d];
        g.inv[d] = 1.0 / m->delta[d];
    }
    return g;
}

const char* stage_name(int stage) {
    static const char* names[SC_NUM_STAGES] = {"sc:deposit", "sc:green", "sc:fwd_x", "sc:fwd_y", "sc:zpass",
                                               "sc:inv_y",   "sc:inv_x", "sc:gather", "sc:plain_fft"};
    return stage >= 0 && stage < SC_NUM_STAGES ? names[stage] : "sc:stage";
}

void StageTimer::begin(int stage, cudaStream_t s) {
    if (open_stage >= 0) end(s);
    if (used[stage] == ev[stage].size()) {
        Pair p;
        if (cudaEventCreate(&p.a) != cudaSuccess || cudaEventCreate(&p.b) != cudaSuccess) return;
        ev[stage].push_back(p);
    }
    cudaEventRecord(ev[stage][used[stage]].a, s);
    open_stage = stage;
}

void StageTimer::end(cudaStream_t s) {
    if (open_stage < 0) return;
    cudaEventRecord(ev[open_stage][used[open_stage]].b, s);
    used[open_stage]++;
    open_stage = -1;
}

void StageTimer::release() {
    for (int k = 0; k < SC_NUM_STAGES; ++k) {
        for (auto& p : ev[k]) {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
        ev[k].clear();
        used[k] = 0;
    }
}

static int check_grid(const int32_t* g) {
    if (!g) return fail(SC_ERR_INVALID, "grid_size is NULL");
    // src/mesh.jl:106-108
    for (int d = 0; d < 3; ++d)
        if (g[d] <= 1) return fail(SC_ERR_INVALID, "All elements of grid_size must be at least 2.");
    return SC_OK;
}

static int check_dtype(int dtype) {
    if (dtype != SC_F32 && dtype != SC_F64)
        return fail(SC_ERR_INVALID, "dtype must be SC_F32 or SC_F64");
    return SC_OK;
}

static int mesh_alloc(const int32_t* g, const double* lo, const double* hi, const double* delta,
                      double gamma, double total_charge, int precision, sc_mesh** out) {
    if (!out) return fail(SC_ERR_INVALID, "out is NULL");
    if (precision != SC_PREC_PLAIN64 && precision != SC_PREC_FP64 && precision != SC_PREC_MIXED)
        return fail(SC_ERR_INVALID, "unknown precision %d", precision);
    if (!(gamma > 0) || !isfinite(gamma)) return fail(SC_ERR_INVALID, "gamma must be a positive finite number");
    sc_mesh* m = new sc_mesh();
    for (int d = 0; d < 3; ++d) {
        m->n[d] = g[d];
        m->lo[d] = lo[d];
        m->hi[d] = hi[d];
        m->delta[d] = delta[d];
    }
    m->N = (int64_t)g[0] * g[1] * g[2];
    m->gamma = gamma;
    m->total_charge = total_charge;
    m->precision = precision;
    cudaError_t e = cudaGetDevice(&m->device);
    if (e != cudaSuccess) {
        delete m;
        return cuda_fail(e, "cudaGetDevice");
    }
    DeviceCtx* ctx = nullptr;
    int st = device_ctx(&ctx);
    if (st != SC_OK) {
        delete m;
        return st;
    }
    if (precision == SC_PREC_MIXED) m->kick_mode = SC_DEPOSIT_VECTOR;
    if (precision != SC_PREC_PLAIN64) {
        st = native_prepare(m);
        if (st != SC_OK) {
            delete m;
            return st;
        }
    }
    const size_t eb = field_elem_bytes(precision);
    const size_t ncomp = precision == SC_PREC_PLAIN64 ? 3 : 4;
    e = dev_alloc(&m->rho, eb * m->N);
    if (e == cudaSuccess) e = dev_alloc(&m->efield, eb * ncomp * m->N);
    if (e == cudaSuccess) e = dev_alloc(&m->oob, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(m->rho, 0, eb * m->N);
    if (e == cudaSuccess) e = cudaMemset(m->efield, 0, eb * ncomp * m->N);
    if (e == cudaSuccess) e = cudaMemset(m->oob, 0, sizeof(unsigned long long));
    if (e != cudaSuccess) {
        cudaFree(m->rho);
        cudaFree(m->efield);
        cudaFree(m->oob);
        delete m;
        return cuda_fail(e, "mesh allocation");
    }
    *out = m;
    return SC_OK;
}

static int check_mesh(const sc_mesh* m) {
    if (!m) return fail(SC_ERR_INVALID, "mesh is NULL");
    return SC_OK;
}

}  // namespace sc

using namespace sc;

static bool valid_deposit_mode(int mode) {
    return mode == SC_DEPOSIT_ATOMIC || mode == SC_DEPOSIT_SORTED || mode == SC_DEPOSIT_DETERMINISTIC ||
           mode == SC_DEPOSIT_TILED || mode == SC_DEPOSIT_VECTOR;
}

namespace sc {

// The kick as issued stream work: deposit, solve (Green build on the side
// stream when needed), gather.  Arguments are already validated.
int kick_issue(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
               int at_cathode, void* ex, void* ey, void* ez, cudaStream_t s) {
    if (m->precision == SC_PREC_PLAIN64) {
        SC_TRY(sc_deposit(m, x, y, z, q, n, dtype, 1, SC_DEPOSIT_ATOMIC, s));
        SC_TRY(sc_solve(m, at_cathode, s));
        return sc_interpolate_field(m, x, y, z, n, dtype, ex, ey, ez, s);
    }
    DeviceGuard g(m->device);
    const int mode = m->kick_mode;
    // The Green spectra do not depend on the charge: when this solve would
    // build them, they are built on the mesh's side stream during the deposit
    // and the forward x and y transforms; the z pass waits for them.
    cudaEvent_t ready = nullptr;
    if (n > 0) SC_TRY(native_green_async(m, at_cathode, s, &ready));
    int st = sc_deposit(m, x, y, z, q, n, dtype, 1, mode, s);
    if (st == SC_OK) st = native_solve(m, at_cathode, s, ready);
    if (st != SC_OK) {
        // the caller's stream still orders the Green build issued above
        if (ready) cudaStreamWaitEvent(s, ready, 0);
        return st;
    }
    if (n == 0) return SC_OK;
    StageScope sg(m->timer, SC_STAGE_GATHER, s);
    // the tiled deposit binned exactly these particles: gather through the tiles
    if (mode == SC_DEPOSIT_TILED) return gather_tiled_launch(m, x, n, dtype, ex, ey, ez, s);
#ifndef SC_GATHER_EARLY
#define SC_GATHER_EARLY 0
#endif
    // the positions are the caller's, read by the deposit before the solve's
    // passes: no grid of this kick writes them
    return gather_launch(m, x, y, z, n, dtype, ex, ey, ez, s, SC_GATHER_EARLY != 0);
}

// ------------------------------------------------------------ kick graph
// A repeated sc_kick with the same arguments and mesh state replays a CUDA
// graph of the kick instead of issuing its ~15 launches from the host.  A call
// with new arguments runs eagerly (it also allocates workspaces and builds
// cached Green spectra); when the next call brings the same arguments back, it
// runs eagerly again and captures the same work, and later calls replay the
// graph on the caller's stream.  A caller that passes new arrays every call
// (allocating its outputs, say) never pays for a capture.
struct KickGraph {
    cudaStream_t cap = nullptr;  // capture origin (the caller's stream may be the legacy stream)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<int64_t> key;
    std::vector<int64_t> seen;  // arguments of the last eager call (kick_key without epoch and generation)
    int64_t launches = 0;       // kernels one replay runs
};

void mesh_state_key(const sc_mesh* m, std::vector<int64_t>& k, bool with_epoch) {
    k.push_back(m->green_cache);
    k.push_back(m->df32);
    k.push_back(m->kick_mode);
    k.push_back(fft_engine());
    k.push_back(m->nw.engine);
    k.push_back(m->nw.lgW);
    // geometry and gamma: kernel arguments captured by value
    const double geo[7] = {m->lo[0], m->lo[1], m->lo[2], m->delta[0], m->delta[1], m->delta[2], m->gamma};
    for (double v : geo) {
        int64_t b;
        memcpy(&b, &v, sizeof b);
        k.push_back(b);
    }
    if (with_epoch) k.push_back(m->green_epoch);
    k.push_back(alloc_generation());
}

static std::vector<int64_t> kick_key(const sc_mesh* m, const void* const* ptr, int64_t n, int dtype,
                                      int at_cathode) {
    std::vector<int64_t> k;
    for (int i = 0; i < 7; ++i) k.push_back((int64_t)(intptr_t)ptr[i]);
    k.push_back(n);
    k.push_back(dtype);
    k.push_back(at_cathode);
    mesh_state_key(m, k);
    return k;
}

void kick_graph_release(sc_mesh* m) {
    KickGraph* kg = reinterpret_cast<KickGraph*>(m->kickgraph);
    if (!kg) return;
    if (kg->exec) cudaGraphExecDestroy(kg->exec);
    if (kg->graph) cudaGraphDestroy(kg->graph);
    if (kg->cap) cudaStreamDestroy(kg->cap);
    delete kg;
    m->kickgraph = nullptr;
}

static void kick_graph_drop(KickGraph* kg) {
    if (kg->exec) cudaGraphExecDestroy(kg->exec);
    if (kg->graph) cudaGraphDestroy(kg->graph);
    kg->exec = nullptr;
    kg->graph = nullptr;
    kg->key.clear();
}

static int kick_graph_capture(sc_mesh* m, KickGraph* kg, const void* const* p, int64_t n, int dtype,
                              int at_cathode) {
    kick_graph_drop(kg);
    if (!kg->cap) SC_CUDA(cudaStreamCreateWithFlags(&kg->cap, cudaStreamNonBlocking));
    const int64_t l0 = m->launches;
    SC_CUDA(cudaStreamBeginCapture(kg->cap, cudaStreamCaptureModeThreadLocal));
    int st = kick_issue(m, p[0], p[1], p[2], p[3], n, dtype, at_cathode, const_cast<void*>(p[4]),
                        const_cast<void*>(p[5]), const_cast<void*>(p[6]), kg->cap);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(kg->cap, &g);
    kg->launches = m->launches - l0;
    m->launches = l0;  // captured, not run
    if (st == SC_OK && e != cudaSuccess) st = cuda_fail(e, "cudaStreamEndCapture");
    if (st != SC_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    // keep the side stream's priority for the Green build's nodes
    const cudaError_t ei = cudaGraphInstantiateWithFlags(&kg->exec, g, cudaGraphInstantiateFlagUseNodePriority);
    if (ei != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(ei, "cudaGraphInstantiate");
    }
    kg->graph = g;
    // keyed on the state after the capture (a capture that builds the Green
    // spectra moves the epoch)
    kg->key = kick_key(m, p, n, dtype, at_cathode);
    return SC_OK;
}

int mesh_set_geometry(sc_mesh* m, const double lo[3], const double hi[3], const double delta[3]) {
    for (int d = 0; d < 3; ++d) {
        if (!(hi[d] > lo[d]) || !(delta[d] > 0))
            return fail(SC_ERR_INVALID, "max_bounds must be strictly greater than min_bounds for all dimensions.");
        m->lo[d] = lo[d];
        m->hi[d] = hi[d];
        m->delta[d] = delta[d];
    }
    return SC_OK;
}

// ------------------------------------------------------ host-buffer kick
// sc_kick_host: particles and outputs in host memory.  The particles go to
// device staging buffers in chunks on an H2D copy stream and each chunk is
// deposited as soon as it has arrived (atomic and vector deposits; the
// sorted, deterministic and tiled deposits wait for all of them); after the
// solve, each chunk is gathered and copied back on a D2H copy stream while
// the next is gathered (every mode but the tiled one, whose gather reads its
// binning of all particles).  The Green build runs on the side stream from
// the start, beside the copies.  Two chunks: each
// chunk costs seven copies and their events, and with 1M FP64 particles the
// kick took 0.401 ms with 2 chunks, 0.431 with 3, 0.421 with 4 and 0.489
// with 8.
constexpr int kHostChunks = 2;

struct HostPipe {
    void* stage = nullptr;  // x, y, z, q, ex, ey, ez, each cap particles
    int64_t cap = 0;
    size_t elem = 0;
    cudaStream_t h2d = nullptr, d2h = nullptr;
    cudaEvent_t fork = nullptr, done = nullptr;
    cudaEvent_t in[kHostChunks] = {}, out[kHostChunks] = {};
};

void host_pipe_release(sc_mesh* m) {
    HostPipe* hp = reinterpret_cast<HostPipe*>(m->hostpipe);
    if (!hp) return;
    cudaFree(hp->stage);
    if (hp->h2d) cudaStreamDestroy(hp->h2d);
    if (hp->d2h) cudaStreamDestroy(hp->d2h);
    cudaEvent_t evs[] = {hp->fork, hp->done};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    for (int c = 0; c < kHostChunks; ++c) {
        if (hp->in[c]) cudaEventDestroy(hp->in[c]);
        if (hp->out[c]) cudaEventDestroy(hp->out[c]);
    }
    delete hp;
    m->hostpipe = nullptr;
}

static int host_pipe_init(HostPipe* hp) {
    SC_CUDA(cudaStreamCreateWithFlags(&hp->h2d, cudaStreamNonBlocking));
    SC_CUDA(cudaStreamCreateWithFlags(&hp->d2h, cudaStreamNonBlocking));
    SC_CUDA(cudaEventCreateWithFlags(&hp->fork, cudaEventDisableTiming));
    SC_CUDA(cudaEventCreateWithFlags(&hp->done, cudaEventDisableTiming));
    for (int c = 0; c < kHostChunks; ++c) {
        SC_CUDA(cudaEventCreateWithFlags(&hp->in[c], cudaEventDisableTiming));
        SC_CUDA(cudaEventCreateWithFlags(&hp->out[c], cudaEventDisableTiming));
    }
    return SC_OK;
}

static int host_pipe(sc_mesh* m, int64_t n, size_t elem, HostPipe** out) {
    HostPipe* hp = reinterpret_cast<HostPipe*>(m->hostpipe);
    if (!hp) {
        hp = new HostPipe();
        m->hostpipe = hp;
        const int st = host_pipe_init(hp);
        if (st != SC_OK) {
            host_pipe_release(m);
            return st;
        }
    }
    if (hp->cap < n || hp->elem != elem) {
        cudaFree(hp->stage);
        hp->stage = nullptr;
        hp->cap = 0;
        SC_CUDA(dev_alloc(&hp->stage, 7 * elem * (size_t)n));
        hp->cap = n;
        hp->elem = elem;
    }
    *out = hp;
    return SC_OK;
}

// Chunk boundaries of the two halves of the host kick, in multiples of 256
// particles.  The H2D side and the D2H side split the particles
// independently.  The deposit runs about three times faster than the H2D
// link and the gather about four times faster than the D2H link, so the last
// H2D chunk is small (its deposit is the only one not hidden under a copy)
// and so is the first gather chunk (the D2H waits for it).  With 1M FP64
// particles the kick took 0.400 ms with halves on both sides, 0.390 with
// 75/25 in and 25/75 out and 0.387 with 65/35 in and 15/85 out.
constexpr double kHostFirstIn = 0.65, kHostFirstOut = 0.15;

// c[0..K]: K chunks of the n particles, the first one a fraction `first` of
// them and the rest equal
static void host_split(int64_t n, int K, double first, int64_t* c) {
    c[0] = 0;
    for (int k = 1; k < K; ++k) {
        const double f = first + (1.0 - first) * (k - 1) / std::max(1, K - 1);
        c[k] = std::min<int64_t>(n, ((int64_t)(f * (double)n) + 255) / 256 * 256);
        c[k] = std::max(c[k], c[k - 1]);
    }
    c[K] = n;
}

static int kick_host_run(sc_mesh* m, HostPipe* hp, const void* const* hin, int64_t n, int dtype, int at_cathode,
                         void* const* hout, cudaStream_t s, cudaEvent_t* ready) {
    const size_t elem = dtype == SC_F64 ? 8 : 4;
    char* st = (char*)hp->stage;
    char* d[7];
    for (int i = 0; i < 7; ++i) d[i] = st + (size_t)i * elem * (size_t)hp->cap;
    const bool plain = m->precision == SC_PREC_PLAIN64;
    const int mode = plain ? SC_DEPOSIT_ATOMIC : m->kick_mode;
    // sorted, deterministic and tiled deposits need every particle at once;
    // the tiled deposit's gather reads its binning of all of them
    const bool chunk_in = deposit_chunkable(m, mode);
    const bool chunk_out = plain || mode != SC_DEPOSIT_TILED;
    const int K = (int)std::min<int64_t>(kHostChunks, std::max<int64_t>(1, n / 65536));
    const int Kin = chunk_in ? K : 1, Kout = chunk_out ? K : 1;
    int64_t cin[kHostChunks + 1], cout[kHostChunks + 1];
    host_split(n, Kin, Kin == 2 ? kHostFirstIn : 1.0 / Kin, cin);
    host_split(n, Kout, Kout == 2 ? kHostFirstOut : 1.0 / Kout, cout);
    SC_CUDA(cudaEventRecord(hp->fork, s));
    SC_CUDA(cudaStreamWaitEvent(hp->h2d, hp->fork, 0));
    SC_CUDA(cudaStreamWaitEvent(hp->d2h, hp->fork, 0));
    if (!plain) SC_TRY(native_green_async(m, at_cathode, s, ready));
    auto h2d = [&](int c) -> int {
        const int64_t off = cin[c], cnt = cin[c + 1] - cin[c];
        for (int i = 0; i < 4; ++i)
            SC_CUDA(cudaMemcpyAsync(d[i] + off * elem, (const char*)hin[i] + off * elem, elem * (size_t)cnt,
                                    cudaMemcpyHostToDevice, hp->h2d));
        SC_CUDA(cudaEventRecord(hp->in[c], hp->h2d));
        SC_CUDA(cudaStreamWaitEvent(s, hp->in[c], 0));
        return SC_OK;
    };
    if (chunk_in) {
        StageScope sd(m->timer, SC_STAGE_DEPOSIT, s);
        SC_TRY(deposit_chunk_begin(m, mode, s));
        for (int c = 0; c < Kin; ++c) {
            const int64_t off = cin[c], cnt = cin[c + 1] - cin[c];
            if (cnt <= 0) continue;
            SC_TRY(h2d(c));
            SC_TRY(deposit_chunk_add(m, d[0] + off * elem, d[1] + off * elem, d[2] + off * elem,
                                     d[3] + off * elem, cnt, dtype, mode, s));
        }
        SC_TRY(deposit_chunk_finish(m, mode, s));
    } else {
        SC_TRY(h2d(0));
        SC_TRY(sc_deposit(m, d[0], d[1], d[2], d[3], n, dtype, 1, mode, s));
    }
    if (plain) {
        SC_TRY(plain_solve(m, at_cathode, s));
    } else {
        m->green_ahead = true;
        const int st = native_solve(m, at_cathode, s, *ready);
        m->green_ahead = false;
        SC_TRY(st);
    }
    StageScope sg(m->timer, SC_STAGE_GATHER, s);
    for (int c = 0; c < Kout; ++c) {
        const int64_t off = cout[c], cnt = cout[c + 1] - cout[c];
        if (cnt <= 0) continue;
        if (chunk_out)
            SC_TRY(gather_launch(m, d[0] + off * elem, d[1] + off * elem, d[2] + off * elem, cnt, dtype,
                                 d[4] + off * elem, d[5] + off * elem, d[6] + off * elem, s));
        else
            SC_TRY(gather_tiled_launch(m, d[0], n, dtype, d[4], d[5], d[6], s));
        SC_CUDA(cudaEventRecord(hp->out[c], s));
        SC_CUDA(cudaStreamWaitEvent(hp->d2h, hp->out[c], 0));
        for (int i = 0; i < 3; ++i)
            SC_CUDA(cudaMemcpyAsync((char*)hout[i] + off * elem, d[4 + i] + off * elem, elem * (size_t)cnt,
                                    cudaMemcpyDeviceToHost, hp->d2h));
    }
    SC_CUDA(cudaEventRecord(hp->done, hp->d2h));
    SC_CUDA(cudaStreamWaitEvent(s, hp->done, 0));
    return SC_OK;
}

static int kick_host_issue(sc_mesh* m, const void* const* hin, int64_t n, int dtype, int at_cathode,
                           void* const* hout, cudaStream_t s) {
    HostPipe* hp = nullptr;
    SC_TRY(host_pipe(m, n, dtype == SC_F64 ? 8 : 4, &hp));
    cudaEvent_t ready = nullptr;
    const int st = kick_host_run(m, hp, hin, n, dtype, at_cathode, hout, s, &ready);
    if (st != SC_OK) {
        // an error returns with no copy of the caller's host buffers in flight,
        // and with the caller's stream ordered after the Green build
        if (ready) cudaStreamWaitEvent(s, ready, 0);
        cudaStreamSynchronize(hp->h2d);
        cudaStreamSynchronize(hp->d2h);
    }
    return st;
}

}  // namespace sc

using namespace sc;

extern "C" {

int sc_version(void) { return 10000; }

const char* sc_last_error(void) { return g_err; }

int sc_mesh_create(const int32_t grid_size[3], const double min_bounds[3], const double max_bounds[3],
                   double gamma, double total_charge, int precision, sc_mesh** out) {
    SC_TRY(check_grid(grid_size));
    if (!min_bounds || !max_bounds) return fail(SC_ERR_INVALID, "bounds are NULL");
    // src/mesh.jl:209-211
    for (int d = 0; d < 3; ++d)
        if (!(max_bounds[d] > min_bounds[d]))
            return fail(SC_ERR_INVALID, "max_bounds must be strictly greater than min_bounds for all dimensions.");
    double delta[3];
    for (int d = 0; d < 3; ++d) delta[d] = (max_bounds[d] - min_bounds[d]) / (double)(grid_size[d] - 1);  // :220
    return mesh_alloc(grid_size, min_bounds, max_bounds, delta, gamma, total_charge, precision, out);
}

int sc_auto_bounds(const int32_t grid_size[3], const void* x, const void* y, const void* z, int64_t n,
                   int dtype, double min_bounds[3], double max_bounds[3], double delta[3], void* stream) {
    SC_TRY(check_grid(grid_size));
    SC_TRY(check_dtype(dtype));
    if (n <= 0 || !x || !y || !z) return fail(SC_ERR_INVALID, "Particle arrays cannot be empty.");  // :110-112
    double mins[3], maxs[3];
    SC_TRY(bounds_reduce(x, y, z, n, dtype, mins, maxs, (cudaStream_t)stream));
    return sc_bounds_from_extrema(grid_size, mins, maxs, min_bounds, max_bounds, delta);
}

int sc_bounds_from_extrema(const int32_t grid_size[3], const double mins[3], const double maxs[3],
                           double min_bounds[3], double max_bounds[3], double delta[3]) {
    SC_TRY(check_grid(grid_size));
    if (!mins || !maxs) return fail(SC_ERR_INVALID, "extrema are NULL");
    for (int d = 0; d < 3; ++d)
        if (!isfinite(mins[d]) || !isfinite(maxs[d]))
            return fail(SC_ERR_INVALID, "particle coordinates must be finite");
    // src/mesh.jl:125-150, Float64 throughout
    double dl[3], lo[3], hi[3];
    for (int d = 0; d < 3; ++d) dl[d] = (maxs[d] - mins[d]) / (double)(grid_size[d] - 1);
    for (int d = 0; d < 3; ++d) {
        lo[d] = mins[d] - 1e-6 * dl[d];
        hi[d] = maxs[d] + 1e-6 * dl[d];
    }
    for (int d = 0; d < 3; ++d) dl[d] = (hi[d] - lo[d]) / (double)(grid_size[d] - 1);
    for (int d = 0; d < 3; ++d) dl[d] = dl[d] == 0 ? 1e-6 : dl[d];
    for (int d = 0; d < 3; ++d) {
        if (min_bounds) min_bounds[d] = lo[d];
        if (max_bounds) max_bounds[d] = hi[d];
        if (delta) delta[d] = dl[d];
    }
    return SC_OK;
}

int sc_mesh_create_from_particles(const int32_t grid_size[3], const void* x, const void* y, const void* z,
                                  int64_t n, int dtype, double gamma, double total_charge, int precision,
                                  void* stream, sc_mesh** out) {
    double lo[3], hi[3], dl[3];
    SC_TRY(sc_auto_bounds(grid_size, x, y, z, n, dtype, lo, hi, dl, stream));
    return mesh_alloc(grid_size, lo, hi, dl, gamma, total_charge, precision, out);
}

int sc_mesh_set_bounds(sc_mesh* m, const double min_bounds[3], const double max_bounds[3]) {
    SC_TRY(check_mesh(m));
    if (!min_bounds || !max_bounds) return fail(SC_ERR_INVALID, "bounds are NULL");
    double delta[3];
    for (int d = 0; d < 3; ++d) {
        if (!(max_bounds[d] > min_bounds[d]))  // src/mesh.jl:209-211
            return fail(SC_ERR_INVALID, "max_bounds must be strictly greater than min_bounds for all dimensions.");
        delta[d] = (max_bounds[d] - min_bounds[d]) / (double)(m->n[d] - 1);  // :220
    }
    return mesh_set_geometry(m, min_bounds, max_bounds, delta);
}

int sc_mesh_refit(sc_mesh* m, const void* x, const void* y, const void* z, int64_t n, int dtype, void* stream) {
    SC_TRY(check_mesh(m));
    DeviceGuard g(m->device);
    double lo[3], hi[3], dl[3];
    SC_TRY(sc_auto_bounds(m->n, x, y, z, n, dtype, lo, hi, dl, stream));
    return mesh_set_geometry(m, lo, hi, dl);
}

int sc_mesh_destroy(sc_mesh* m) {
    if (!m) return SC_OK;
    DeviceGuard g(m->device);
    if (m->precision == SC_PREC_PLAIN64)
        plain_release(m);
    else
        native_release(m);
    m->timer.release();
    sorted_release(m);
    tiled_release(m);
    kick_graph_release(m);
    host_pipe_release(m);
    cudaFree(m->trackE);
    cudaFree(m->corner);
    if (m->side) cudaStreamDestroy(m->side);
    if (m->side2) cudaStreamDestroy(m->side2);
    if (m->ev_join2) cudaEventDestroy(m->ev_join2);
    if (m->ev_fork) cudaEventDestroy(m->ev_fork);
    if (m->ev_join) cudaEventDestroy(m->ev_join);
    cudaFree(m->rho);
    cudaFree(m->efield);
    cudaFree(m->oob);
    delete m;
    return SC_OK;
}

int sc_mesh_set_profiling(sc_mesh* m, int enabled) {
    SC_TRY(check_mesh(m));
    m->timer.enabled = enabled != 0;
    return SC_OK;
}

int sc_mesh_stage_times(sc_mesh* m, double* ms, int64_t* calls, void* stream) {
    SC_TRY(check_mesh(m));
    DeviceGuard g(m->device);
    SC_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    for (int k = 0; k < SC_NUM_STAGES; ++k) {
        double tot = 0;
        for (size_t i = 0; i < m->timer.used[k]; ++i) {
            float t = 0;
            SC_CUDA(cudaEventElapsedTime(&t, m->timer.ev[k][i].a, m->timer.ev[k][i].b));
            tot += t;
        }
        if (ms) ms[k] = tot;
        if (calls) calls[k] = (int64_t)m->timer.used[k];
        m->timer.used[k] = 0;
    }
    return SC_OK;
}

int sc_mesh_launch_count(const sc_mesh* m, int64_t* count) {
    SC_TRY(check_mesh(m));
    if (count) *count = m->launches;
    return SC_OK;
}

int sc_mesh_get_info(const sc_mesh* m, sc_mesh_info* info) {
    SC_TRY(check_mesh(m));
    if (!info) return fail(SC_ERR_INVALID, "info is NULL");
    memset(info, 0, sizeof(*info));
    for (int d = 0; d < 3; ++d) {
        info->grid_size[d] = m->n[d];
        info->min_bounds[d] = m->lo[d];
        info->max_bounds[d] = m->hi[d];
        info->delta[d] = m->delta[d];
        info->fft_shape[d] = m->precision == SC_PREC_PLAIN64 ? 2 * m->n[d] : m->nw.L[d];
    }
    info->precision = m->precision;
    info->gamma = m->gamma;
    info->total_charge = m->total_charge;
    info->efield_layout = m->precision == SC_PREC_PLAIN64 ? SC_LAYOUT_PLANAR : SC_LAYOUT_PACKED;
    info->elem_bytes = (int32_t)field_elem_bytes(m->precision);
    info->device = m->device;
    return SC_OK;
}

int sc_mesh_rho(sc_mesh* m, void** p) {
    SC_TRY(check_mesh(m));
    if (!p) return fail(SC_ERR_INVALID, "dptr is NULL");
    *p = m->rho;
    return SC_OK;
}

int sc_mesh_efield(sc_mesh* m, void** p) {
    SC_TRY(check_mesh(m));
    if (!p) return fail(SC_ERR_INVALID, "dptr is NULL");
    *p = m->efield;
    return SC_OK;
}

int sc_autotune(sc_mesh* m, void* stream, int* choice) {
    SC_TRY(check_mesh(m));
    DeviceGuard g(m->device);
    return native_autotune(m, (cudaStream_t)stream, choice);
}

int sc_set_fft_engine(int engine) {
    if (engine != SC_FFT_AUTO && engine != SC_FFT_STOCKHAM) return fail(SC_ERR_INVALID, "unknown FFT engine %d", engine);
    g_fft_engine.store(engine);
    return SC_OK;
}

int sc_test_fail_allocations(int64_t after) {
    g_alloc_allow.store(after < 0 ? -1 : after);
    return SC_OK;
}

int sc_mesh_set_green_cache(sc_mesh* m, int enabled) {
    SC_TRY(check_mesh(m));
    m->green_cache = enabled != 0;
    if (!m->green_cache) {
        m->nw.key_free.valid = false;
        m->nw.key_img.valid = false;
    }
    return SC_OK;
}

int sc_mesh_set_fp64_arithmetic(sc_mesh* m, int mode) {
    SC_TRY(check_mesh(m));
    if (m->precision != SC_PREC_FP64) return fail(SC_ERR_INVALID, "FP64 transform modes apply to SC_PREC_FP64 meshes");
    if (mode != SC_FP64_ARITH_FP64 && mode != SC_FP64_ARITH_DF32)
        return fail(SC_ERR_INVALID, "unknown FP64 transform mode %d", mode);
    m->df32 = mode == SC_FP64_ARITH_DF32;
    return SC_OK;
}

int sc_clear_mesh(sc_mesh* m, void* stream) {
    SC_TRY(check_mesh(m));
    DeviceGuard g(m->device);
    SC_CUDA(cudaMemsetAsync(m->rho, 0, field_elem_bytes(m->precision) * m->N, (cudaStream_t)stream));
    return SC_OK;
}

int sc_deposit(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n,
               int dtype, int clear, int mode, void* stream) {
    SC_TRY(check_mesh(m));
    SC_TRY(check_dtype(dtype));
    if (n < 0) return fail(SC_ERR_INVALID, "Particle coordinate and charge arrays must have the same length.");
    if (n > 0 && (!x || !y || !z || !q)) return fail(SC_ERR_INVALID, "particle pointer is NULL");
    if (!valid_deposit_mode(mode)) return fail(SC_ERR_INVALID, "unknown deposit mode %d", mode);
    DeviceGuard g(m->device);
    StageScope st(m->timer, SC_STAGE_DEPOSIT, (cudaStream_t)stream);
    // a clearing vector deposit writes rho whole in its node sum
    const bool assign = clear && n > 0 && deposit_assigns(m, mode);
    if (clear && !assign) SC_TRY(sc_clear_mesh(m, stream));
    if (n == 0) return SC_OK;
    return deposit_launch(m, x, y, z, q, n, dtype, mode, (cudaStream_t)stream, assign);
}

int sc_solve(sc_mesh* m, int at_cathode, void* stream) {
    SC_TRY(check_mesh(m));
    DeviceGuard g(m->device);
    if (m->precision == SC_PREC_PLAIN64) return plain_solve(m, at_cathode, (cudaStream_t)stream);
    return native_solve(m, at_cathode, (cudaStream_t)stream);
}

int sc_interpolate_field(sc_mesh* m, const void* x, const void* y, const void* z, int64_t n, int dtype,
                         void* ex, void* ey, void* ez, void* stream) {
    SC_TRY(check_mesh(m));
    SC_TRY(check_dtype(dtype));
    if (n < 0) return fail(SC_ERR_INVALID, "negative particle count");
    if (n == 0) return SC_OK;
    if (!x || !y || !z || !ex || !ey || !ez) return fail(SC_ERR_INVALID, "particle or output pointer is NULL");
    DeviceGuard g(m->device);
    StageScope st(m->timer, SC_STAGE_GATHER, (cudaStream_t)stream);
    return gather_launch(m, x, y, z, n, dtype, ex, ey, ez, (cudaStream_t)stream);
}

int sc_kick(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
            int at_cathode, void* ex, void* ey, void* ez, void* stream) {
    SC_TRY(check_mesh(m));
    SC_TRY(check_dtype(dtype));
    if (n < 0) return fail(SC_ERR_INVALID, "Particle coordinate and charge arrays must have the same length.");
    if (n > 0 && (!x || !y || !z || !q)) return fail(SC_ERR_INVALID, "particle pointer is NULL");
    if (n > 0 && (!ex || !ey || !ez)) return fail(SC_ERR_INVALID, "particle or output pointer is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return cuda_fail(cudaGetLastError(), "cudaStreamIsCapturing");
    const bool graph = m->kick_graph && m->precision != SC_PREC_PLAIN64 && n > 0 && !m->timer.enabled &&
                       cs == cudaStreamCaptureStatusNone;
    if (!graph) return kick_issue(m, x, y, z, q, n, dtype, at_cathode, ex, ey, ez, s);
    DeviceGuard g(m->device);
    const void* p[7] = {x, y, z, q, ex, ey, ez};
    std::vector<int64_t> key = kick_key(m, p, n, dtype, at_cathode);
    KickGraph* kg = reinterpret_cast<KickGraph*>(m->kickgraph);
    if (kg && kg->exec && kg->key == key) {
        SC_CUDA(cudaGraphLaunch(kg->exec, s));
        m->launches += kg->launches;
        return SC_OK;
    }
    SC_TRY(kick_issue(m, x, y, z, q, n, dtype, at_cathode, ex, ey, ez, s));
    if (!kg) {
        kg = new KickGraph();
        m->kickgraph = kg;
    }
    // the Green epoch and the allocation generation close mesh_state_key: an
    // eager kick may move them, the arguments it was called with stay
    key.resize(key.size() - 2);
    if (key != kg->seen) {
        kg->seen = std::move(key);
        return SC_OK;
    }
    return kick_graph_capture(m, kg, p, n, dtype, at_cathode);
}

int sc_kick_host(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
                 int at_cathode, void* ex, void* ey, void* ez, void* stream) {
    SC_TRY(check_mesh(m));
    SC_TRY(check_dtype(dtype));
    if (n < 0) return fail(SC_ERR_INVALID, "Particle coordinate and charge arrays must have the same length.");
    if (n > 0 && (!x || !y || !z || !q)) return fail(SC_ERR_INVALID, "particle pointer is NULL");
    if (n > 0 && (!ex || !ey || !ez)) return fail(SC_ERR_INVALID, "particle or output pointer is NULL");
    if (n == 0) return sc_kick(m, nullptr, nullptr, nullptr, nullptr, 0, dtype, at_cathode, nullptr, nullptr, nullptr,
                               stream);
    DeviceGuard g(m->device);
    const void* hin[4] = {x, y, z, q};
    void* hout[3] = {ex, ey, ez};
    return kick_host_issue(m, hin, n, dtype, at_cathode, hout, (cudaStream_t)stream);
}

int sc_solve_potential(sc_mesh* m, int at_cathode, void* phi, void* stream) {
    SC_TRY(check_mesh(m));
    if (!phi) return fail(SC_ERR_INVALID, "phi is NULL");
    DeviceGuard g(m->device);
    // the hand-written pipelines take transforms of up to 256 points (axes
    // of up to 128 nodes); longer ones and plain64 meshes use the FP64 cuFFT
    // schedule of the reference
    const NativeWork& w = m->nw;
    if (m->precision != SC_PREC_PLAIN64 && w.log2L[0] <= 8 && w.log2L[1] <= 8 && w.log2L[2] <= 8)
        return native_potential(m, at_cathode, phi, (cudaStream_t)stream);
    return plain_potential(m, at_cathode, phi, (cudaStream_t)stream);
}

int sc_mesh_set_kick_graph(sc_mesh* m, int enabled) {
    SC_TRY(check_mesh(m));
    m->kick_graph = enabled != 0;
    if (!m->kick_graph) {
        KickGraph* kg = reinterpret_cast<KickGraph*>(m->kickgraph);
        if (kg) kick_graph_drop(kg);
    }
    return SC_OK;
}

int sc_mesh_set_kick_mode(sc_mesh* m, int mode) {
    SC_TRY(check_mesh(m));
    if (!valid_deposit_mode(mode)) return fail(SC_ERR_INVALID, "unknown deposit mode %d", mode);
    m->kick_mode = mode;
    return SC_OK;
}

int sc_kick_adjoint(sc_mesh* m, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
                    int at_cathode, const void* gex, const void* gey, const void* gez, const void* ggrid, void* dx,
                    void* dy, void* dz, void* dq, void* stream) {
    SC_TRY(check_mesh(m));
    SC_TRY(check_dtype(dtype));
    if (n < 0) return fail(SC_ERR_INVALID, "negative particle count");
    if (n > 0 && (!x || !y || !z || !q || !dx || !dy || !dz || !dq))
        return fail(SC_ERR_INVALID, "particle or gradient pointer is NULL");
    DeviceGuard g(m->device);
    if (n == 0) return SC_OK;
    return adjoint_launch(m, x, y, z, q, n, dtype, at_cathode, gex, gey, gez, ggrid, dx, dy, dz, dq,
                          (cudaStream_t)stream);
}

int sc_cell_index(sc_mesh* m, const void* x, const void* y, const void* z, int64_t n, int dtype, int32_t* idx,
                  double* frac, void* stream) {
    SC_TRY(check_mesh(m));
    SC_TRY(check_dtype(dtype));
    if (n < 0) return fail(SC_ERR_INVALID, "negative particle count");
    if (n == 0) return SC_OK;
    if (!x || !y || !z || !idx || !frac) return fail(SC_ERR_INVALID, "NULL pointer");
    DeviceGuard g(m->device);
    return cell_index_launch(m, x, y, z, n, dtype, idx, frac, (cudaStream_t)stream);
}

int sc_solve_noalloc(const int32_t grid_size[3], const double delta[3], double gamma, const float* rho,
                     float* efield, void* stream) {
    if (!grid_size || !delta || !rho || !efield) return fail(SC_ERR_INVALID, "NULL argument");
    return native_solve_noalloc(grid_size, delta, gamma, rho, efield, (cudaStream_t)stream);
}

int sc_mesh_out_of_range(sc_mesh* m, int64_t* count, void* stream) {
    SC_TRY(check_mesh(m));
    DeviceGuard g(m->device);
    unsigned long long h = 0;
    SC_CUDA(cudaMemcpyAsync(&h, m->oob, sizeof(h), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    SC_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    SC_CUDA(cudaMemsetAsync(m->oob, 0, sizeof(h), (cudaStream_t)stream));
    if (count) *count = (int64_t)h;
    return SC_OK;
}

}  // extern "C"
