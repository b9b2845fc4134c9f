// Batched kick of many independent bunches (own meshes, uneven particle
// counts and grids).
//
// Staged engine.  Bunches on FP32-mixed meshes whose transforms run on the
// register two-step kernels (lengths <= 256, Lx = Ly) are kicked stage by
// stage in groups: consecutive bunches of one grid class (equal transform
// lengths) whose buffers fit a working-set budget.  Per group, on one
// internal stream, each stage is one launch over all of its bunches:
//   clear (rho, or the vector deposit's corner slots) -> deposit -> node sum
//   -> forward x+y (one fused pass, or an x pass and a y pass) -> z pass
//   with the Green multiply -> inverse y+x -> gather.
// A launch's CTAs find their bunch and their plane, tile or particle block
// in a CtaRef table built on the host (batch.cuh); the bunch descriptors,
// clear segments and CTA tables are uploaded once per set of arguments.  A
// bunch deposits through the vector corner slots when it has at least a
// quarter as many particles as nodes, and with scalar atomics into rho when
// it is sparser (the slots cost 32 bytes per node to clear and read).  The
// budget and the forward-pass choice are picked by sc_batch_autotune.
// Other bunches (FP64 meshes, longer transforms, other deposit modes) run
// their whole kick on the internal streams beside the groups.
//
// The first call with a given set of arguments plans the groups (this
// synchronises `stream` once, allocates every mesh's workspace and builds
// its Green spectrum), runs them eagerly, and captures the same work into a
// CUDA graph; later calls with the same pointers, counts and flags, on
// meshes whose state is unchanged, replay the graph with one launch.  The
// reference has no multi-bunch API; a tracking code calls its kick once per
// bunch (benchmark/full_pipeline_benchmark.jl:64-71 times one at a time).
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "batch.cuh"
#include "sc_internal.cuh"

// Working-set budget of a bunch group and the forward-pass choice before
// sc_batch_autotune (measured on the 64-bunch workload: per-bunch groups and
// two-pass forward transforms).
constexpr int64_t kDefaultGroupBytes = 0;
constexpr bool kDefaultFusedForward = false;

struct sc_batch {
    std::vector<sc_mesh*> meshes;
    int device = 0;
    std::vector<cudaStream_t> streams;
    cudaStream_t cap = nullptr;  // origin stream of the graph capture
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    bool graph_enabled = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t graph_nodes = 0;
    // arguments the graph was captured with
    std::vector<const void*> key_ptr;
    std::vector<int64_t> key_n;
    int key_dtype = -1, key_cath = -1;
    std::vector<int64_t> key_state;  // every mesh's mesh_state_key
    // ---- staged engine
    struct Launch {
        int64_t off = 0, ctas = 0;  // CtaRef range of the launch
    };
    // bunches of one grid class kicked together: one launch per stage over
    // all of them, on one internal stream
    struct Group {
        int logL = 0, logLz = 0;
        size_t plane = 0;  // largest ny * Hx of its bunches
        Launch clear, dep, csum, fwd, fx, fy, z, inv, gather;
        std::vector<int> members;  // staged indices
    };
    bool staged_enabled = true;  // sc_batch_set_staged
    // working-set budget of a group (bytes of field, charge and transform
    // buffers): 0 = one bunch per group, INT64_MAX = one group per class
    int64_t group_bytes = kDefaultGroupBytes;
    bool fwd_fused = kDefaultFusedForward;  // forward x+y as one pass per plane
    // plan for the arguments in plan_*
    bool planned = false;
    std::vector<const void*> plan_ptr;
    std::vector<int64_t> plan_n, plan_state;
    int plan_dtype = -1, plan_cath = -1;
    std::vector<int> staged, others;  // bunch indices
    std::vector<Group> groups;
    void* dev = nullptr;  // BunchDesc[staged] | ClearSeg[staged] | CtaRef[...]
    size_t dev_cap = 0;
    sc::BunchDesc* tab = nullptr;
    sc::ClearSeg* segs = nullptr;
    sc::CtaRef* map = nullptr;
    int64_t launches = 0;  // kernels of the staged part per kick
};

namespace sc {

// Forks the internal streams from `s` and joins them back: their work is
// ordered after the caller's earlier work and before its later work.
static int batch_fork(sc_batch* b, cudaStream_t s) {
    SC_CUDA(cudaEventRecord(b->fork, s));
    for (cudaStream_t st : b->streams) SC_CUDA(cudaStreamWaitEvent(st, b->fork, 0));
    return SC_OK;
}
static int batch_join(sc_batch* b, cudaStream_t s, int st) {
    // join every stream, also after a failure: the caller's stream orders
    // whatever was issued
    for (size_t k = 0; k < b->streams.size(); ++k) {
        cudaError_t e = cudaEventRecord(b->join[k], b->streams[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->join[k], 0);
        if (e != cudaSuccess && st == SC_OK) st = cuda_fail(e, "batch join");
    }
    return st;
}

// The per-bunch path: the whole kick of bunch which[k] on internal stream
// k % nstreams (every bunch, or the ones the staged engine does not take).
static int batch_issue_streams(sc_batch* b, const std::vector<int>& which, const void* const* x,
                               const void* const* y, const void* const* z, const void* const* q, const int64_t* n,
                               int dtype, int at_cathode, void* const* ex, void* const* ey, void* const* ez) {
    const int ns = (int)b->streams.size();
    int st = SC_OK;
    for (size_t k = 0; k < which.size() && st == SC_OK; ++k) {
        // With other bunches on the other streams, a fused inverse pass that
        // takes a whole SM per CTA still pays (64 uneven bunches: 7.07 ->
        // 6.22 ms); alone on the GPU it does not (the 128^3 cathode kick:
        // 0.712 -> 0.724 ms).
        const int i = which[k];
        sc_mesh* m = b->meshes[i];
        const size_t cap = m->fused_smem_cap;
        m->fused_smem_cap = ns > 1 ? 210 * 1024 : cap;
        m->beside_others = ns > 1;
        st = kick_issue(m, x[i], y[i], z[i], q[i], n[i], dtype, at_cathode, ex[i], ey[i], ez[i],
                        b->streams[k % ns]);
        m->fused_smem_cap = cap;
        m->beside_others = false;
    }
    return st;
}

// ------------------------------------------------------------ staged plan
static bool stageable(const sc_mesh* m) {
    if (m->precision != SC_PREC_MIXED) return false;
    const NativeWork& w = m->nw;
    const int eng = w.engine >= 0 ? w.engine : fft_engine();
    if (eng != 0) return false;
    if (w.log2L[0] != w.log2L[1] || w.log2L[0] > 8 || w.log2L[2] > 8) return false;
    return m->kick_mode == SC_DEPOSIT_VECTOR || m->kick_mode == SC_DEPOSIT_ATOMIC;
}

static int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Plans the staged engine for these arguments: sorts the bunches into the
// staged set and the others, allocates the staged meshes' workspaces and
// builds their stale Green spectra on `s`, forms the groups, and uploads the
// bunch descriptors and CTA tables (after synchronising `s`: a graph
// replayed earlier may still read the previous tables).
static int batch_plan(sc_batch* b, const void* const* x, const void* const* y, const void* const* z,
                      const void* const* q, const int64_t* n, int at_cathode, void* const* ex, void* const* ey,
                      void* const* ez, cudaStream_t s) {
    b->planned = false;
    b->staged.clear();
    b->others.clear();
    b->groups.clear();
    const int nb = (int)b->meshes.size();
    for (int i = 0; i < nb; ++i) (stageable(b->meshes[i]) ? b->staged : b->others).push_back(i);
    std::vector<BunchDesc> tab;
    std::vector<ClearSeg> segs;
    for (int i : b->staged) {
        sc_mesh* m = b->meshes[i];
        SC_TRY(alloc_work<float>(m));
        if (native_green_stale(m, at_cathode)) SC_TRY(native_ensure_green(m, at_cathode, s));
        const bool vec = m->kick_mode == SC_DEPOSIT_VECTOR && 4 * n[i] >= m->N;
        if (vec) SC_TRY(corner_alloc(m));
        const NativeWork& w = m->nw;
        BunchDesc d = {};
        d.x = x[i];
        d.y = y[i];
        d.z = z[i];
        d.q = q[i];
        d.ex = ex[i];
        d.ey = ey[i];
        d.ez = ez[i];
        d.n = n[i];
        d.ax = make_axes(m);
        d.rho = (float*)m->rho;
        d.corner = vec ? (float4*)m->corner : nullptr;
        d.efield = (float4*)m->efield;
        d.oob = m->oob;
        d.nx = m->n[0];
        d.ny = m->n[1];
        d.nz = m->n[2];
        d.Hx = w.Hx;
        d.Ly = w.L[1];
        d.A = (float2*)w.A;
        d.B = (float2*)w.B;
        d.C = (float2*)w.C;
        d.gv = make_green_view(w, at_cathode ? 1 : 0);
        tab.push_back(d);
        segs.push_back(vec ? ClearSeg{(float*)m->corner, 8 * m->N} : ClearSeg{(float*)m->rho, m->N});
    }
    std::vector<CtaRef> map;
    auto add = [&](sc_batch::Launch& l, int item, int64_t ctas) {
        if (l.ctas == 0) l.off = (int64_t)map.size();
        for (int64_t c = 0; c < ctas; ++c) map.push_back(CtaRef{item, (int)c});
        l.ctas += ctas;
    };
    const int ns = (int)b->staged.size();
    // grid classes (equal transform lengths), in order of first appearance
    std::vector<std::pair<int, int>> cls;
    std::vector<std::vector<int>> members;
    for (int k = 0; k < ns; ++k) {
        const NativeWork& w = b->meshes[b->staged[k]]->nw;
        const std::pair<int, int> key(w.log2L[0], w.log2L[2]);
        const size_t c = std::find(cls.begin(), cls.end(), key) - cls.begin();
        if (c == cls.size()) {
            cls.push_back(key);
            members.emplace_back();
        }
        members[c].push_back(k);
    }
    // groups: consecutive bunches of a class while their working set (field,
    // charge buffer, B and C) stays within the budget
    for (size_t c = 0; c < cls.size(); ++c) {
        int64_t ws = 0;
        bool open = false;
        for (int k : members[c]) {
            const int64_t N = (int64_t)tab[k].nx * tab[k].ny * tab[k].nz;
            const int64_t wk = 16 * N + (tab[k].corner ? 32 : 4) * N + 32 * (int64_t)tab[k].Hx * tab[k].Ly * tab[k].nz;
            if (!open || ws + wk > b->group_bytes) {
                b->groups.emplace_back();
                b->groups.back().logL = cls[c].first;
                b->groups.back().logLz = cls[c].second;
                ws = 0;
                open = true;
            }
            ws += wk;
            b->groups.back().members.push_back(k);
            b->groups.back().plane = std::max(b->groups.back().plane, (size_t)tab[k].ny * tab[k].Hx);
        }
    }
    for (auto& g : b->groups) {
        for (int k : g.members) add(g.clear, k, ceil_div(segs[k].n, kClearChunk));
        for (int k : g.members) add(g.dep, k, ceil_div(tab[k].n, batch_deposit_particles_per_cta()));
        for (int k : g.members)
            if (tab[k].corner) add(g.csum, k, ceil_div((int64_t)tab[k].nx * tab[k].ny * tab[k].nz, 256));
        for (int k : g.members) add(g.fwd, k, tab[k].nz);
        for (int k : g.members) add(g.fx, k, batch_fwd_x_ctas(g.logL, (int64_t)tab[k].ny * tab[k].nz));
        for (int k : g.members) add(g.fy, k, batch_fwd_y_ctas((int64_t)tab[k].Hx * tab[k].nz));
        for (int k : g.members) add(g.z, k, ceil_div((int64_t)tab[k].Hx * tab[k].Ly, kBatchZCols));
        for (int k : g.members) add(g.inv, k, 3 * (int64_t)tab[k].nz);
        for (int k : g.members) add(g.gather, k, ceil_div(tab[k].n, batch_gather_particles_per_cta()));
        if (batch_plane_smem(g.logL, (int64_t)g.plane) > 227 * 1024)
            return fail(SC_ERR_UNSUPPORTED, "batch: a plane of %zu nodes does not fit in shared memory", g.plane);
    }
    // upload
    const size_t tb = sizeof(BunchDesc) * tab.size(), sb = sizeof(ClearSeg) * segs.size();
    const size_t o_segs = (tb + 255) / 256 * 256, o_map = o_segs + (sb + 255) / 256 * 256;
    const size_t need = o_map + sizeof(CtaRef) * map.size() + 256;
    SC_CUDA(cudaStreamSynchronize(s));
    if (b->dev_cap < need) {
        b->dev_cap = 0;
        SC_CUDA(dev_realloc(&b->dev, need));
        b->dev_cap = need;
    }
    unsigned char* base = (unsigned char*)b->dev;
    b->tab = (BunchDesc*)base;
    b->segs = (ClearSeg*)(base + o_segs);
    b->map = (CtaRef*)(base + o_map);
    if (tb) SC_CUDA(cudaMemcpy(b->tab, tab.data(), tb, cudaMemcpyHostToDevice));
    if (sb) SC_CUDA(cudaMemcpy(b->segs, segs.data(), sb, cudaMemcpyHostToDevice));
    if (!map.empty()) SC_CUDA(cudaMemcpy(b->map, map.data(), sizeof(CtaRef) * map.size(), cudaMemcpyHostToDevice));
    b->planned = true;
    return SC_OK;
}

// The staged kick of the planned groups (forked from the caller's stream by
// batch_fork).  With every Green spectrum cached, all groups go on internal
// stream 0, one after another: each launch already fills the GPU, and the
// classes side by side only share L2 (64 uneven bunches: 5.08 ms on 4-8
// streams, 5.01 ms on one).  A call that builds Green spectra puts group g
// on stream g % nstreams, so that the small bunches' builds overlap.
static int batch_issue_staged(sc_batch* b, int dtype, int at_cathode) {
    int64_t l = 0;
    auto at = [&](const sc_batch::Launch& x) {
        l += x.ctas > 0;
        return b->map + x.off;
    };
    const int nstr = (int)b->streams.size();
    bool builds = false;
    for (const sc_batch::Group& k : b->groups)
        for (int j : k.members) builds = builds || native_green_stale(b->meshes[b->staged[j]], at_cathode);
    int st = SC_OK;
    for (size_t g = 0; g < b->groups.size() && st == SC_OK; ++g) {
        const sc_batch::Group& k = b->groups[g];
        cudaStream_t cs = b->streams[builds ? g % nstr : 0];
        // Green spectra this solve must build (stale, or the cache is off)
        for (size_t j = 0; j < k.members.size() && st == SC_OK; ++j) {
            sc_mesh* m = b->meshes[b->staged[k.members[j]]];
            if (native_green_stale(m, at_cathode)) st = native_ensure_green(m, at_cathode, cs);
        }
        if (st == SC_OK) st = batch_clear_launch(b->segs, at(k.clear), k.clear.ctas, cs);
        if (st == SC_OK) st = batch_deposit_launch(b->tab, at(k.dep), k.dep.ctas, dtype, cs);
        if (st == SC_OK) st = batch_corner_sum_launch(b->tab, at(k.csum), k.csum.ctas, cs);
        if (b->fwd_fused) {
            if (st == SC_OK) st = batch_fwd_xy_launch(k.logL, b->tab, at(k.fwd), k.fwd.ctas, k.plane, cs);
        } else {
            if (st == SC_OK) st = batch_fwd_x_launch(k.logL, b->tab, at(k.fx), k.fx.ctas, cs);
            if (st == SC_OK) st = batch_fwd_y_launch(k.logL, b->tab, at(k.fy), k.fy.ctas, cs);
        }
        if (st == SC_OK) st = batch_zpass_launch(k.logLz, b->tab, at(k.z), k.z.ctas, at_cathode != 0, cs);
        if (st == SC_OK) st = batch_inv_yx_launch(k.logL, b->tab, at(k.inv), k.inv.ctas, k.plane, cs);
        if (st == SC_OK) st = batch_gather_launch(b->tab, at(k.gather), k.gather.ctas, dtype, cs);
    }
    b->launches = l;
    return st;
}

static int batch_issue(sc_batch* b, const void* const* x, const void* const* y, const void* const* z,
                       const void* const* q, const int64_t* n, int dtype, int at_cathode, void* const* ex,
                       void* const* ey, void* const* ez, cudaStream_t s) {
    SC_TRY(batch_fork(b, s));
    int st = SC_OK;
    if (!b->planned) {
        std::vector<int> all(b->meshes.size());
        for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
        st = batch_issue_streams(b, all, x, y, z, q, n, dtype, at_cathode, ex, ey, ez);
    } else {
        // the other bunches on the internal streams, beside the groups
        st = batch_issue_streams(b, b->others, x, y, z, q, n, dtype, at_cathode, ex, ey, ez);
        if (st == SC_OK) st = batch_issue_staged(b, dtype, at_cathode);
    }
    return batch_join(b, s, st);
}

// with_epoch = false: what a stage plan depends on (it holds workspace and
// spectrum addresses, not the spectra's contents)
static std::vector<int64_t> batch_state(const sc_batch* b, bool with_epoch = true) {
    std::vector<int64_t> k;
    for (const sc_mesh* m : b->meshes) mesh_state_key(m, k, with_epoch);
    return k;
}

static void batch_drop_graph(sc_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_nodes = 0;
    b->key_ptr.clear();
    b->key_n.clear();
    b->key_state.clear();
}

}  // namespace sc

using namespace sc;

extern "C" {

int sc_batch_create(sc_mesh* const* meshes, int nbunch, int nstreams, sc_batch** out) {
    if (!out || !meshes || nbunch <= 0) return fail(SC_ERR_INVALID, "sc_batch_create needs at least one mesh");
    if (nstreams <= 0) nstreams = 8;
    if (nstreams > nbunch) nstreams = nbunch;
    sc_batch* b = new sc_batch();
    cudaError_t e = cudaGetDevice(&b->device);
    for (int i = 0; i < nbunch && e == cudaSuccess; ++i) {
        if (!meshes[i]) {
            delete b;
            return fail(SC_ERR_INVALID, "mesh %d is NULL", i);
        }
        if (meshes[i]->device != b->device) {
            delete b;
            return fail(SC_ERR_INVALID, "all meshes of a batch must live on the current device");
        }
        b->meshes.push_back(meshes[i]);
    }
    for (int k = 0; k < nstreams && e == cudaSuccess; ++k) {
        cudaStream_t st;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) b->streams.push_back(st);
        cudaEvent_t ev;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) b->join.push_back(ev);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        for (cudaStream_t st : b->streams) cudaStreamDestroy(st);
        for (cudaEvent_t ev : b->join) cudaEventDestroy(ev);
        delete b;
        return cuda_fail(e, "sc_batch_create");
    }
    *out = b;
    return SC_OK;
}

int sc_batch_set_graph(sc_batch* b, int enabled) {
    if (!b) return fail(SC_ERR_INVALID, "batch is NULL");
    b->graph_enabled = enabled != 0;
    if (!b->graph_enabled) batch_drop_graph(b);
    return SC_OK;
}

int sc_batch_kick(sc_batch* b, const void* const* x, const void* const* y, const void* const* z, const void* const* q,
                  const int64_t* n, int dtype, int at_cathode, void* const* ex, void* const* ey, void* const* ez,
                  void* stream) {
    if (!b) return fail(SC_ERR_INVALID, "batch is NULL");
    if (!x || !y || !z || !q || !n || !ex || !ey || !ez) return fail(SC_ERR_INVALID, "NULL argument array");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nb = b->meshes.size();
    std::vector<const void*> key;
    key.reserve(7 * nb);
    for (size_t i = 0; i < nb; ++i) {
        const void* p[7] = {x[i], y[i], z[i], q[i], ex[i], ey[i], ez[i]};
        key.insert(key.end(), p, p + 7);
    }
    std::vector<int64_t> kn(n, n + nb);
    // the member meshes are the caller's: a refit, a rebuilt spectrum or a
    // reallocated workspace of any of them forces a new capture
    if (b->graph_enabled && b->exec && key == b->key_ptr && kn == b->key_n && dtype == b->key_dtype &&
        at_cathode == b->key_cath && batch_state(b) == b->key_state) {
        SC_CUDA(cudaGraphLaunch(b->exec, s));
        return SC_OK;
    }
    // plan the staged engine for these arguments (meshes' workspaces, stale
    // Green spectra, CTA tables) unless the plan in hand is for them
    if (!b->staged_enabled) {
        b->planned = false;
    } else if (!(b->planned && key == b->plan_ptr && kn == b->plan_n && dtype == b->plan_dtype &&
                 at_cathode == b->plan_cath && batch_state(b, false) == b->plan_state)) {
        SC_TRY(batch_plan(b, x, y, z, q, n, at_cathode, ex, ey, ez, s));
        b->plan_ptr = key;
        b->plan_n = kn;
        b->plan_dtype = dtype;
        b->plan_cath = at_cathode;
        b->plan_state = batch_state(b, false);
    }
    // eager run (allocates workspaces, builds Green spectra, sets attributes)
    SC_TRY(batch_issue(b, x, y, z, q, n, dtype, at_cathode, ex, ey, ez, s));
    if (!b->graph_enabled) return SC_OK;
    batch_drop_graph(b);
    // capture the same work; stage timers are not recorded inside graphs
    std::vector<bool> prof(nb);
    for (size_t i = 0; i < nb; ++i) {
        prof[i] = b->meshes[i]->timer.enabled;
        b->meshes[i]->timer.enabled = false;
    }
    // Capture on an internal stream (the caller's may be the legacy default
    // stream, which cannot be captured); the graph is launched on `stream`.
    cudaError_t e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
    int st = e == cudaSuccess ? SC_OK : cuda_fail(e, "cudaStreamBeginCapture");
    if (st == SC_OK) {
        st = batch_issue(b, x, y, z, q, n, dtype, at_cathode, ex, ey, ez, b->cap);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(b->cap, &g);
        if (st == SC_OK && e != cudaSuccess) st = cuda_fail(e, "cudaStreamEndCapture");
        if (st == SC_OK) {
            e = cudaGraphInstantiateWithFlags(&b->exec, g, cudaGraphInstantiateFlagUseNodePriority);
            if (e != cudaSuccess) {
                st = cuda_fail(e, "cudaGraphInstantiate");
                cudaGraphDestroy(g);
            } else {
                b->graph = g;
                cudaGraphGetNodes(g, nullptr, &b->graph_nodes);
            }
        } else if (g) {
            cudaGraphDestroy(g);
        }
    }
    for (size_t i = 0; i < nb; ++i) b->meshes[i]->timer.enabled = prof[i];
    if (st != SC_OK) return st;
    b->key_ptr = key;
    b->key_n = kn;
    b->key_dtype = dtype;
    b->key_cath = at_cathode;
    b->key_state = batch_state(b);
    return SC_OK;
}

int sc_batch_graph_nodes(const sc_batch* b, int64_t* count) {
    if (!b) return fail(SC_ERR_INVALID, "batch is NULL");
    if (count) *count = (int64_t)b->graph_nodes;
    return SC_OK;
}

int sc_batch_destroy(sc_batch* b) {
    if (!b) return SC_OK;
    batch_drop_graph(b);
    for (cudaStream_t st : b->streams) cudaStreamDestroy(st);
    for (cudaEvent_t ev : b->join) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->cap) cudaStreamDestroy(b->cap);
    cudaFree(b->dev);
    delete b;
    return SC_OK;
}

int sc_batch_set_staged(sc_batch* b, int enabled) {
    if (!b) return fail(SC_ERR_INVALID, "batch is NULL");
    b->staged_enabled = enabled != 0;
    b->planned = false;
    batch_drop_graph(b);
    return SC_OK;
}

int sc_batch_set_group_bytes(sc_batch* b, int64_t bytes) {
    if (!b) return fail(SC_ERR_INVALID, "batch is NULL");
    if (bytes < 0) return fail(SC_ERR_INVALID, "group_bytes must be >= 0");
    b->group_bytes = bytes;
    b->planned = false;
    batch_drop_graph(b);
    return SC_OK;
}

int sc_batch_set_fused_forward(sc_batch* b, int enabled) {
    if (!b) return fail(SC_ERR_INVALID, "batch is NULL");
    b->fwd_fused = enabled != 0;
    b->planned = false;
    batch_drop_graph(b);
    return SC_OK;
}

int sc_batch_autotune(sc_batch* b, const void* const* x, const void* const* y, const void* const* z,
                      const void* const* q, const int64_t* n, int dtype, int at_cathode, void* const* ex,
                      void* const* ey, void* const* ez, void* stream, int64_t* group_bytes, int* fused_forward) {
    if (!b) return fail(SC_ERR_INVALID, "batch is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t cand[] = {0, 48ll << 20, 128ll << 20, 512ll << 20, INT64_MAX};
    const bool graph = b->graph_enabled;
    const bool staged = b->staged_enabled;
    b->graph_enabled = true;
    b->staged_enabled = true;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int st = SC_OK;
    cudaError_t ec = cudaEventCreate(&e0);
    if (ec == cudaSuccess) ec = cudaEventCreate(&e1);
    if (ec != cudaSuccess) st = cuda_fail(ec, "cudaEventCreate");
    float best = 1e30f;
    int64_t pick = b->group_bytes;
    bool pick_fused = b->fwd_fused;
    for (int v = 0; v < 10 && st == SC_OK; ++v) {
        const int64_t c = cand[v % 5];
        const bool fused = v >= 5;
        st = sc_batch_set_group_bytes(b, c);
        if (st == SC_OK) st = sc_batch_set_fused_forward(b, fused ? 1 : 0);
        // plan + eager + capture, then one replay to warm up
        for (int r = 0; r < 2 && st == SC_OK; ++r) st = sc_batch_kick(b, x, y, z, q, n, dtype, at_cathode, ex, ey, ez, s);
        if (st != SC_OK) break;
        cudaError_t e = cudaEventRecord(e0, s);
        for (int r = 0; r < 3 && st == SC_OK; ++r) st = sc_batch_kick(b, x, y, z, q, n, dtype, at_cathode, ex, ey, ez, s);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (st == SC_OK && e != cudaSuccess) st = cuda_fail(e, "batch autotune timing");
        if (st != SC_OK) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            pick = c;
            pick_fused = fused;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    b->graph_enabled = graph;
    b->staged_enabled = staged;
    b->fwd_fused = pick_fused;
    const int st2 = sc_batch_set_group_bytes(b, pick);
    if (st != SC_OK) return st;
    if (group_bytes) *group_bytes = pick;
    if (fused_forward) *fused_forward = pick_fused ? 1 : 0;
    return st2;
}

int sc_batch_staged_count(const sc_batch* b, int* staged, int64_t* launches) {
    if (!b) return fail(SC_ERR_INVALID, "batch is NULL");
    if (staged) *staged = b->planned ? (int)b->staged.size() : 0;
    if (launches) *launches = b->planned ? b->launches : 0;
    return SC_OK;
}

}  // extern "C"
