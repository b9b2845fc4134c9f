// Batched kick of many independent bunches (own meshes, uneven particle
// counts and grids) and the FFT autotuner.
//
// sc_batch_kick forks the bunches' deposit -> solve -> interpolate pipelines
// onto nstreams internal streams (fork/join through events on the caller's
// stream), so independent bunches overlap on the GPU.  The first call with a
// given set of arguments runs eagerly (this also allocates every mesh's
// workspace and builds its Green spectrum) and then captures the same work
// into a CUDA graph; later calls with the same pointers, counts and flags
// replay the graph with one launch.  The reference has no multi-bunch API;
// a tracking code calls its kick once per bunch.
#include <string.h>

#include <vector>

#include "sc_internal.cuh"

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
};

namespace sc {

static int batch_issue(sc_batch* b, const void* const* x, const void* const* y, const void* const* z,
                       const void* const* q, const int64_t* n, int dtype, int at_cathode, void* const* ex,
                       void* const* ey, void* const* ez, cudaStream_t s) {
    SC_CUDA(cudaEventRecord(b->fork, s));
    for (cudaStream_t st : b->streams) SC_CUDA(cudaStreamWaitEvent(st, b->fork, 0));
    const int ns = (int)b->streams.size();
    int st = SC_OK;
    for (size_t i = 0; i < b->meshes.size() && st == SC_OK; ++i) {
        // With other bunches on the other streams, a fused inverse pass that
        // takes a whole SM per CTA still pays (64 uneven bunches: 7.07 ->
        // 6.22 ms); alone on the GPU it does not (the 128^3 cathode kick:
        // 0.712 -> 0.724 ms).
        sc_mesh* m = b->meshes[i];
        const size_t cap = m->fused_smem_cap;
        m->fused_smem_cap = ns > 1 ? 210 * 1024 : cap;
        m->beside_others = ns > 1;
        st = kick_issue(m, x[i], y[i], z[i], q[i], n[i], dtype, at_cathode, ex[i], ey[i], ez[i], b->streams[i % ns]);
        m->fused_smem_cap = cap;
        m->beside_others = false;
    }
    // join every stream, also after a failed bunch: the caller's stream
    // orders whatever was issued
    for (int k = 0; k < ns; ++k) {
        cudaError_t e = cudaEventRecord(b->join[k], b->streams[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->join[k], 0);
        if (e != cudaSuccess && st == SC_OK) st = cuda_fail(e, "batch join");
    }
    return st;
}

static std::vector<int64_t> batch_state(const sc_batch* b) {
    std::vector<int64_t> k;
    for (const sc_mesh* m : b->meshes) mesh_state_key(m, k);
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
    delete b;
    return SC_OK;
}

}  // extern "C"
