// C ABI of libgbc: device-resident graphs, betweenness / closeness / per-source
// counts through the lane or plain engine, with status codes and stats.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <mutex>

#include "engine.h"

using namespace gbc;

struct gbc_graph_s {
    DevGraph g;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::unique_ptr<LaneEngine> eng;
    gbc_run_stats last{};
    int32_t* d_src = nullptr;
    int64_t src_cap = 0;
    unsigned long long* d_ccb = nullptr;
    int64_t ccb_cap = 0;
    double* d_bc = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<int32_t> last_src;
    // lane assignment: per-vertex level-profile key (computed once)
    std::vector<uint32_t> key;
    int32_t key_depth = 0;        // levels of that BFS (0: not run)
    int32_t* d_pos = nullptr;
    int64_t pos_cap = 0;
    // internal ids are by descending degree: order[new] = old, inv[old] = new
    int32_t* d_order = nullptr;
    int32_t* d_inv = nullptr;
    // per-level profile of the last batch of the last call (gbc_graph_last_levels)
    std::vector<int64_t> last_level_entries;
    std::vector<float> last_fwd_launch_ms, last_bwd_launch_ms;
    std::vector<int32_t> h_inv;
    double* d_bc_out = nullptr;   // BC in the caller's ids (gbc_bc)
    // vertex weights set by gbc_graph_set_weights, in internal ids (nullable)
    int32_t* d_w = nullptr;
    int64_t* d_ff = nullptr;
    // settings chosen by gbc_autotune; used where the options ask for autotuning
    struct {
        bool done = false;
        int32_t lanes = 0, sparse = -1, light = -1, lpg = 0, group = 0;
        int32_t block = 0;    // threads per CTA of the level kernels (0: default)
        int32_t share = -1;   // closeness direction-switch share (0: top-down only; -1: default)
    } tuned;
    ~gbc_graph_s() {
        eng.reset();
        if (stream) cudaStreamSynchronize(stream);
        // the CSR and id maps go back to the lane-state cache (graphs created in a loop reuse them)
        dev_release(g.row, sizeof(int64_t) * ((size_t)g.n + 1));
        dev_release(g.col, sizeof(int32_t) * std::max<int64_t>(g.m, 1));
        g.row = nullptr;
        g.col = nullptr;
        cudaFree(d_src);
        cudaFree(d_ccb);
        cudaFree(d_bc);
        cudaFree(d_pos);
        dev_release(d_order, sizeof(int32_t) * (size_t)g.n);
        dev_release(d_inv, sizeof(int32_t) * (size_t)g.n);
        cudaFree(d_bc_out);
        cudaFree(d_w);
        cudaFree(d_ff);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace gbc {

// Component ids and per-component undirected edge counts of a host CSR.
static void host_components(const int64_t* row, const int32_t* col, int32_t n, DevGraph& g) {
    HostCSR h;
    h.n = n;
    h.row.assign(row, row + n + 1);
    h.col.assign(col, col + row[n]);
    std::vector<int64_t> sizes;
    const int32_t nc = components(h, g.comp, sizes);
    g.comp_edges.assign(nc, 0);
    int32_t md = 0;
    for (int32_t v = 0; v < n; v++) {
        g.comp_edges[g.comp[v]] += row[v + 1] - row[v];
        md = std::max<int32_t>(md, (int32_t)(row[v + 1] - row[v]));
    }
    for (auto& e : g.comp_edges) e /= 2;
    g.max_degree = md;
}

static gbc_status graph_alloc(int32_t n, int64_t m, gbc_graph_s* G) {
    DevGraph& g = G->g;
    g.n = n;
    g.m = m;
    GBC_CUDA(cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking));
    GBC_CUDA(cudaEventCreate(&G->ev0));
    GBC_CUDA(cudaEventCreate(&G->ev1));
    if (dev_alloc((void**)&g.row, sizeof(int64_t) * ((size_t)n + 1)) != cudaSuccess ||
        dev_alloc((void**)&g.col, sizeof(int32_t) * std::max<int64_t>(g.m, 1)) != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation for the CSR failed");
        return GBC_ERR_NOMEM;
    }
    return GBC_OK;
}

// Host CSR to the device, on the graph's stream (not waited for).
static gbc_status graph_upload(const int64_t* row, const int32_t* col, int32_t n, gbc_graph_s* G) {
    GBC_TRY(graph_alloc(n, row[n], G));
    DevGraph& g = G->g;
    GBC_CUDA(cudaMemcpyAsync(g.row, row, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, G->stream));
    if (g.m) GBC_CUDA(cudaMemcpyAsync(g.col, col, sizeof(int32_t) * g.m, cudaMemcpyHostToDevice, G->stream));
    return GBC_OK;
}

// bad[0] = smallest v with row[v+1] < row[v], bad[1] = smallest e with col[e]
// outside [0, n); both stay 0xFFFFFFFF when there is none (indices < 2^31).
// Whole blocks step together so that every lane takes part in the warp minimum.
__global__ void csr_check_kernel(const int64_t* __restrict__ row, const int32_t* __restrict__ col, int32_t n,
                                 int64_t m, unsigned* __restrict__ bad) {
    const int64_t len = (int64_t)n > m ? (int64_t)n : m;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < len; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        unsigned br = ~0u, bc = ~0u;
        if (i < n && row[i + 1] < row[i]) br = (unsigned)i;
        if (i < m && (uint32_t)col[i] >= (uint32_t)n) bc = (unsigned)i;
        br = __reduce_min_sync(0xFFFFFFFFu, br);
        bc = __reduce_min_sync(0xFFFFFFFFu, bc);
        if ((threadIdx.x & 31) == 0) {
            if (br != ~0u) atomicMin(&bad[0], br);
            if (bc != ~0u) atomicMin(&bad[1], bc);
        }
    }
}

// The per-entry checks of validate_csr on the device copy (0.6 GB of CSR
// takes well under a millisecond here against ~10 ms for 16 host threads),
// with the same messages and the same first offending index.  host_col, when
// given, supplies the offending value for the message.  Waits for the upload.
static gbc_status validate_device(gbc_graph_s* G, const int32_t* host_col) {
    const DevGraph& g = G->g;
    unsigned* d_bad = nullptr;
    if (dev_alloc((void**)&d_bad, 2 * sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        set_error("validation flag");
        return GBC_ERR_NOMEM;
    }
    std::unique_ptr<unsigned, void (*)(unsigned*)> keep(d_bad, [](unsigned* p) { dev_release(p, 2 * sizeof(unsigned)); });
    int dev = 0, sm = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    GBC_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
    GBC_CUDA(cudaMemsetAsync(d_bad, 0xFF, 2 * sizeof(unsigned), G->stream));
    csr_check_kernel<<<sm * 8, 256, 0, G->stream>>>(g.row, g.col, g.n, g.m, d_bad);
    GBC_CUDA(cudaGetLastError());
    unsigned bad[2] = {~0u, ~0u};
    GBC_CUDA(cudaMemcpyAsync(bad, d_bad, sizeof bad, cudaMemcpyDeviceToHost, G->stream));
    GBC_CUDA(cudaStreamSynchronize(G->stream));
    if (bad[0] != ~0u) { set_error("row offsets decrease at %lld", (long long)bad[0]); return GBC_ERR_ARG; }
    if (bad[1] != ~0u) {
        int32_t val = 0;
        if (host_col) val = host_col[bad[1]];
        else GBC_CUDA(cudaMemcpy(&val, g.col + bad[1], sizeof val, cudaMemcpyDeviceToHost));
        set_error("col[%lld]=%d out of range", (long long)bad[1], val);
        return GBC_ERR_ARG;
    }
    return GBC_OK;
}

// Component information is needed only for the statistics (edges per
// source's component); it is computed on first request from a copy of the
// device CSR, outside the compute calls.
static gbc_status ensure_components(gbc_graph_s* G) {
    DevGraph& g = G->g;
    if (!g.comp.empty()) return GBC_OK;
    std::vector<int64_t> row(g.n + 1);
    std::vector<int32_t> col(std::max<int64_t>(g.m, 1));
    GBC_CUDA(cudaMemcpy(row.data(), g.row, sizeof(int64_t) * (g.n + 1), cudaMemcpyDeviceToHost));
    if (g.m) GBC_CUDA(cudaMemcpy(col.data(), g.col, sizeof(int32_t) * g.m, cudaMemcpyDeviceToHost));
    host_components(row.data(), col.data(), g.n, g);
    return GBC_OK;
}

static gbc_status ensure_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device available (%s)", cudaGetErrorString(e));
        return GBC_ERR_NO_DEVICE;
    }
    return GBC_OK;
}

static gbc_status resolve_options(const gbc_options* opt, gbc_options& o) {
    gbc_options_default(&o);
    if (opt) o = *opt;
    if (o.semantics != GBC_BC_BRANDES && o.semantics != GBC_BC_REFERENCE) { set_error("bad semantics"); return GBC_ERR_ARG; }
    if (o.delta_precision != GBC_DELTA_F32 && o.delta_precision != GBC_DELTA_F64) { set_error("bad delta precision"); return GBC_ERR_ARG; }
    if (o.sigma_mode < GBC_SIGMA_AUTO || o.sigma_mode > GBC_SIGMA_WIDE) { set_error("bad sigma mode"); return GBC_ERR_ARG; }
    if (o.engine < GBC_ENGINE_AUTO || o.engine > GBC_ENGINE_LANES) { set_error("bad engine"); return GBC_ERR_ARG; }
    if (o.lanes != 0 && (o.lanes < 32 || o.lanes > 1024 || o.lanes % 32)) { set_error("lanes must be 0 or a multiple of 32 in [32,1024]"); return GBC_ERR_ARG; }
    if (o.group_lanes != 0 && o.group_lanes != 1 && o.group_lanes != 32 && o.group_lanes != 128) {
        set_error("group_lanes must be 0, 1, 32 or 128");
        return GBC_ERR_ARG;
    }
    if (o.group_lanes == 128 && o.lanes % 128) { set_error("group_lanes 128 needs lanes = 0 or a multiple of 128"); return GBC_ERR_ARG; }
    if (o.direction != 0 && o.direction != 1) { set_error("direction must be 0 or 1"); return GBC_ERR_ARG; }
    if (o.block_threads != 0 && o.block_threads != 128 && o.block_threads != 256 && o.block_threads != 512) {
        set_error("block_threads must be 0, 128, 256 or 512");
        return GBC_ERR_ARG;
    }
    if (o.bu_share < 0 || o.bu_share > 4096) { set_error("bu_share must be in [0,4096]"); return GBC_ERR_ARG; }
    return GBC_OK;
}

// Calls on a graph with vertex weights: the lane engine only (the plain
// engine has none), and for betweenness the Brandes semantics only (the
// reference's per-predecessor count does not combine with pair weights).
static gbc_status check_weighted(const gbc_graph_s* G, const gbc_options& o, bool bc) {
    if (!G->g.w && !G->g.ff) return GBC_OK;
    if (o.engine == GBC_ENGINE_PLAIN) { set_error("the plain engine has no vertex weights (gbc_graph_set_weights)"); return GBC_ERR_ARG; }
    if (bc && o.semantics != GBC_BC_BRANDES) {
        set_error("betweenness with vertex weights supports GBC_BC_BRANDES only");
        return GBC_ERR_ARG;
    }
    return GBC_OK;
}

// Autotune lanes: as wide as the sources and the memory budget allow; an
// existing engine that is wide enough is kept.
// Lanes per group of a call: the option, else the tuned value, else 128 on
// small-world graphs (the source-ordering BFS from the hubs ended within 32
// levels: sources grouped by level profile keep many lanes active per task;
// R-MAT scale 22 BC 103 -> 126 GTEPS, closeness 258 -> 490 GTEPS), one lane per
// task on deeper graphs of degree at most 64 (grids, meshes, roads: a lane
// group's sampled sources rarely share a level; 1024^2 grid BC 3.9 -> 5.2
// GTEPS), and 32 on other deep graphs.  The max degree is known from graph
// creation for graphs of fewer than 2^22 vertices.
static int32_t group_of(const gbc_graph_s* G, const gbc_options& o) {
    if (o.group_lanes) return o.group_lanes;
    if (G->tuned.done && G->tuned.group) return G->tuned.group;
    if (G->key_depth > 0 && G->key_depth <= SMALL_WORLD_DEPTH) return 128;
    if (G->key_depth > SMALL_WORLD_DEPTH && G->g.max_degree <= ONE_LANE_MAX_DEGREE && G->g.n < ONE_LANE_MAX_N)
        return 1;
    return 32;
}

static int32_t pick_lanes(const gbc_graph_s* G, int64_t k, bool bc, int32_t requested, int32_t group) {
    if (requested) return requested;
    const DevGraph& g = G->g;
    const int32_t unit = group == 1 ? 32 : group;   // batches stay a multiple of 32 lanes
    int32_t lanes = (int32_t)std::min<int64_t>(G->tuned.lanes ? G->tuned.lanes : 1024, ((k + unit - 1) / unit) * unit);
    lanes = std::max(lanes, unit);
    if (G->eng && (G->eng->has_bc() || !bc) && G->eng->lanes() >= lanes && G->eng->group_lanes() == group)
        return G->eng->lanes();
    const size_t fr = dev_free_bytes();
    const size_t budget = (fr + (G->eng ? G->eng->device_bytes() : 0)) / 2;
    while (lanes > unit && LaneEngine::bytes_needed(g.n, lanes, bc, group) > budget) lanes -= unit;
    return lanes;
}

// Expansion settings of a call: the options' values, or the graph's tuned ones
// where the options leave them to autotuning.
struct Tuning { int sparse, light, lpg, block, share; };
static Tuning tuning_of(const gbc_graph_s* G, const gbc_options& o) {
    const bool t = G->tuned.done;
    Tuning u;
    u.sparse = (o.sparse_lanes < 0 && t) ? G->tuned.sparse : o.sparse_lanes;
    u.light = (o.light_steps < 0 && t) ? G->tuned.light : o.light_steps;
    u.lpg = (o.levels_per_graph <= 0 && t) ? G->tuned.lpg : o.levels_per_graph;
    u.block = (o.block_threads == 0 && t) ? G->tuned.block : o.block_threads;
    u.share = o.bu_share > 0 ? o.bu_share : (t ? G->tuned.share : -1);
    return u;
}

static gbc_status get_engine(gbc_graph_s* G, int32_t lanes, bool bc, const gbc_options& o, LaneEngine** out) {
    const Tuning u = tuning_of(G, o);
    const int32_t gw = group_of(G, o);
    const int32_t group = (gw == 1 || lanes % 128 == 0) ? gw : 32;
    if (G->eng && G->eng->lanes() == lanes && (G->eng->has_bc() || !bc) && G->eng->group_lanes() == group) {
        G->eng->set_tuning(u.sparse, u.light, u.lpg, u.block, u.share);
        *out = G->eng.get();
        return GBC_OK;
    }
    G->eng.reset();
    auto e = std::make_unique<LaneEngine>();
    GBC_TRY(e->init(&G->g, lanes, bc, u.sparse, u.lpg, G->stream, group));
    e->set_tuning(u.sparse, u.light, u.lpg, u.block, u.share);
    G->eng = std::move(e);
    *out = G->eng.get();
    return GBC_OK;
}

// Level-profile key of every vertex: one forward batch from the 32 highest-
// degree vertices; key = (level from the top vertex, nearest of the others).
// The graph's ids must be in descending degree order (every device graph of
// this library is relabelled so), so the 32 highest-degree vertices are ids
// 0..31.  depth = levels of that batch.
gbc_status level_profile_key(const DevGraph& g, cudaStream_t stream, std::vector<uint32_t>& key, int32_t& depth) {
    // its own narrow engine: the main engine's group width depends on the depth found here
    LaneEngine E;
    GBC_TRY(E.init(&g, 32, false, -1, 0, stream, 32));
    const int32_t kb = std::min<int32_t>(32, g.n);
    std::vector<int32_t> idx(kb);
    for (int32_t v = 0; v < kb; v++) idx[v] = v;
    int32_t* d_hub = nullptr;
    uint32_t* d_key = nullptr;
    const size_t skey = sizeof(uint32_t) * (size_t)g.n;
    if (dev_alloc((void**)&d_hub, sizeof(int32_t) * 32) != cudaSuccess || dev_alloc((void**)&d_key, skey) != cudaSuccess) {
        cudaGetLastError();
        dev_release(d_hub, sizeof(int32_t) * 32);
        set_error("order key buffers");
        return GBC_ERR_NOMEM;
    }
    // handed back once the stream is idle
    struct Bufs {
        cudaStream_t s; int32_t* hub; uint32_t* key; size_t skey;
        ~Bufs() { cudaStreamSynchronize(s); dev_release(hub, sizeof(int32_t) * 32); dev_release(key, skey); }
    } bufs{stream, d_hub, d_key, skey};
    GBC_CUDA(cudaMemcpyAsync(d_hub, idx.data(), sizeof(int32_t) * kb, cudaMemcpyHostToDevice, stream));
    LaneRequest rq;
    rq.job = LaneJob::CC;
    rq.d_src = d_hub;
    rq.kb = kb;
    rq.d_profile_key = d_key;
    LaneResult res;
    GBC_TRY(E.run(rq, res));
    depth = (int32_t)res.levels;
    key.resize(g.n);
    GBC_CUDA(cudaMemcpyAsync(key.data(), d_key, sizeof(uint32_t) * g.n, cudaMemcpyDeviceToHost, stream));
    GBC_CUDA(cudaStreamSynchronize(stream));
    return GBC_OK;
}

static gbc_status ensure_order_key(gbc_graph_s* G) {
    if (!G->key.empty()) return GBC_OK;
    return level_profile_key(G->g, G->stream, G->key, G->key_depth);
}

// Reorder sources so that each 32-lane group holds sources with similar BFS
// level profiles (denser lane masks, fewer frontier entries).  pos[i] = index
// in the caller's list of the i-th ordered source.
static gbc_status order_sources(gbc_graph_s* G, const gbc_options& o, bool bc, std::vector<int32_t>& hsrc,
                                std::vector<int32_t>& pos) {
    const int64_t k = (int64_t)hsrc.size();
    pos.resize(k);
    for (int64_t i = 0; i < k; i++) pos[i] = (int32_t)i;
    if (o.engine == GBC_ENGINE_PLAIN || o.source_order != 0 || k <= 32) return GBC_OK;
    GBC_TRY(ensure_order_key(G));
    const std::vector<uint32_t>& key = G->key;
    // ties: lower id first, which is higher degree first (ids are in descending degree order)
    std::stable_sort(pos.begin(), pos.end(), [&](int32_t a, int32_t b) {
        const int32_t x = hsrc[a], y = hsrc[b];
        if (key[x] != key[y]) return key[x] < key[y];
        return x < y;
    });
    std::vector<int32_t> ordered(k);
    for (int64_t i = 0; i < k; i++) ordered[i] = hsrc[pos[i]];
    hsrc.swap(ordered);
    return GBC_OK;
}

static gbc_status upload_sources(gbc_graph_s* G, const std::vector<int32_t>& hsrc) {
    if ((int64_t)hsrc.size() > G->src_cap) {
        cudaFree(G->d_src);
        G->d_src = nullptr;
        if (cudaMalloc(&G->d_src, sizeof(int32_t) * hsrc.size()) != cudaSuccess) { cudaGetLastError(); set_error("source buffer"); return GBC_ERR_NOMEM; }
        G->src_cap = (int64_t)hsrc.size();
    }
    GBC_CUDA(cudaMemcpyAsync(G->d_src, hsrc.data(), sizeof(int32_t) * hsrc.size(), cudaMemcpyHostToDevice, G->stream));
    return GBC_OK;
}

__global__ void scatter_cc_kernel(const unsigned long long* __restrict__ in, const int32_t* __restrict__ pos, int32_t k,
                                  int64_t* __restrict__ out) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) out[pos[i]] = (int64_t)in[i];
}

static gbc_status resolve_sources(gbc_graph_s* G, const int32_t* sources, int32_t k, std::vector<int32_t>& hsrc) {
    const DevGraph& g = G->g;
    if (k < 0) { set_error("k < 0"); return GBC_ERR_ARG; }
    if (k == 0) {
        if (sources) { set_error("k = 0 with a non-NULL source list"); return GBC_ERR_ARG; }
        hsrc.resize(g.n);
        for (int32_t i = 0; i < g.n; i++) hsrc[i] = i;
    } else {
        if (!sources) { set_error("sources is NULL"); return GBC_ERR_ARG; }
        hsrc.assign(sources, sources + k);
        for (int32_t i = 0; i < k; i++)
            if (hsrc[i] < 0 || hsrc[i] >= g.n) { set_error("source %d out of range [0,%d)", hsrc[i], g.n); return GBC_ERR_ARG; }
    }
    for (auto& x : hsrc) x = G->h_inv[x];   // to internal ids
    return GBC_OK;
}

// Caller's source ids (already range-checked) to internal ids.
static void map_sources(const gbc_graph_s* G, std::vector<int32_t>& hsrc) {
    for (auto& x : hsrc) x = G->h_inv[x];
}

// After the CSR is on the device: relabelling (degree order, or Cuthill-McKee
// on deep graphs of low degree) and the id maps.
static gbc_status finish_graph(gbc_graph_s* G) {
    GBC_TRY(relabel_graph(G->g, G->stream, &G->d_order, &G->d_inv));
    G->h_inv.resize(G->g.n);
    GBC_CUDA(cudaMemcpy(G->h_inv.data(), G->d_inv, sizeof(int32_t) * G->g.n, cudaMemcpyDeviceToHost));
    return GBC_OK;
}

static gbc_status ensure_bc_buffer(double** p, int32_t n) {
    if (*p) return GBC_OK;
    if (cudaMalloc(p, sizeof(double) * n) != cudaSuccess) { cudaGetLastError(); set_error("bc buffer"); return GBC_ERR_NOMEM; }
    return GBC_OK;
}

static void finish_stats(gbc_graph_s* G, const LaneResult& r, int64_t k, int64_t batches, int32_t lanes, int sigma_used,
                         const std::vector<int32_t>& hsrc, double ms_kernel, double ms_total) {
    gbc_run_stats& s = G->last;
    std::memset(&s, 0, sizeof s);
    s.sources = k;
    s.batches = batches;
    s.levels = r.levels;
    s.kernel_launches = r.kernel_launches;
    s.graph_launches = r.graph_launches;
    s.frontier_entries = r.frontier_entries;
    s.sigma_overflow_lanes = r.overflow_count;
    s.kernel_ms = ms_kernel;
    s.total_ms = ms_total;
    s.lanes = lanes;
    s.sigma_mode_used = sigma_used;
    s.fwd_ms = r.fwd_ms;
    s.bwd_ms = r.bwd_ms;
    s.fwd_kernels = r.fwd_kernels;
    s.bwd_kernels = r.bwd_kernels;
    s.edges_traversed = -1;   // filled in lazily by gbc_graph_last_stats
    s.group_lanes = lanes == 1 ? 1 : (G->eng ? G->eng->group_lanes() : 32);
    s.bottom_up_levels = (int32_t)r.bottom_up_levels;
    s.sigma_bytes = r.sigma_bytes;
    s.neighbour_visits = r.neighbour_visits;
    G->last_src = hsrc;
    G->last_level_entries = r.level_entries;
    G->last_fwd_launch_ms = r.fwd_launch_ms;
    G->last_bwd_launch_ms = r.bwd_launch_ms;
}

// Betweenness over device-staged sources d_src[0..k) into d_bc[n].
static gbc_status bc_core(gbc_graph_s* G, const int32_t* d_src, int32_t k, const gbc_options& o, double* d_bc,
                          LaneResult& res, int32_t& lanes_used, int& sigma_used, int64_t& batches) {
    const DevGraph& g = G->g;
    if (o.engine == GBC_ENGINE_PLAIN) {
        std::vector<int32_t> h(k);
        GBC_CUDA(cudaMemcpyAsync(h.data(), d_src, sizeof(int32_t) * k, cudaMemcpyDeviceToHost, G->stream));
        GBC_CUDA(cudaStreamSynchronize(G->stream));
        GBC_CUDA(cudaMemsetAsync(d_bc, 0, sizeof(double) * g.n, G->stream));
        GBC_TRY(plain_bc(&g, h.data(), k, o.semantics, o.delta_precision == GBC_DELTA_F64, d_bc, G->stream, res));
        lanes_used = 1;
        sigma_used = GBC_SIGMA_EXACT;
        batches = k;
        if (res.overflow_count && o.sigma_mode != GBC_SIGMA_WIDE) {
            set_error("exact path counts overflowed uint64 for %d sources (plain engine has no wide form)", res.overflow_count);
            return GBC_ERR_OVERFLOW;
        }
        return GBC_OK;
    }
    const int32_t lanes = pick_lanes(G, k, true, o.lanes, group_of(G, o));
    LaneEngine* E = nullptr;
    GBC_TRY(get_engine(G, lanes, true, o, &E));
    lanes_used = lanes;
    GBC_TRY(E->bc_begin());
    sigma_used = o.sigma_mode == GBC_SIGMA_WIDE ? GBC_SIGMA_WIDE : GBC_SIGMA_EXACT;
    batches = 0;
    // AUTO: once a batch of this call has overflowed, the later ones start in wide form
    bool wide = (o.sigma_mode == GBC_SIGMA_WIDE);
    for (int32_t b0 = 0; b0 < k; b0 += lanes) {
        LaneRequest rq;
        rq.job = LaneJob::BC;
        rq.d_src = d_src + b0;
        rq.kb = std::min(lanes, k - b0);
        rq.delta_f64 = o.delta_precision == GBC_DELTA_F64;
        rq.semantics = o.semantics;
        rq.sigma_wide = wide;
        rq.abort_on_overflow = !rq.sigma_wide;
        gbc_status st = E->run(rq, res);
        if (st == GBC_ERR_OVERFLOW && o.sigma_mode == GBC_SIGMA_AUTO && !wide) {
            wide = true;
            rq.sigma_wide = 1;
            rq.abort_on_overflow = false;
            st = E->run(rq, res);
        }
        if (wide) sigma_used = GBC_SIGMA_WIDE;
        if (st != GBC_OK) return st;
        batches++;
    }
    return E->bc_finish(d_bc);
}

static gbc_status cc_core(gbc_graph_s* G, const int32_t* d_src, const int32_t* h_src, int32_t k, const gbc_options& o,
                          unsigned long long* d_cc, int64_t* h_cc_plain, LaneResult& res, int32_t& lanes_used,
                          int64_t& batches) {
    const DevGraph& g = G->g;
    if (o.engine == GBC_ENGINE_PLAIN) {
        GBC_TRY(plain_cc(&g, h_src, k, h_cc_plain, G->stream, res));
        lanes_used = 1;
        batches = k;
        return GBC_OK;
    }
    const int32_t lanes = pick_lanes(G, k, false, o.lanes, group_of(G, o));
    LaneEngine* E = nullptr;
    GBC_TRY(get_engine(G, lanes, false, o, &E));
    lanes_used = lanes;
    batches = 0;
    for (int32_t b0 = 0; b0 < k; b0 += lanes) {
        LaneRequest rq;
        rq.job = LaneJob::CC;
        rq.d_src = d_src + b0;
        rq.kb = std::min(lanes, k - b0);
        rq.d_cc = d_cc + b0;
        rq.top_down_only = o.direction == 1;
        GBC_TRY(E->run(rq, res));
        batches++;
    }
    return GBC_OK;
}

}  // namespace gbc

static double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

extern "C" {

const char* gbc_version(void) { return "gbc 0.1 (sm_103a)"; }

int gbc_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
    return n;
}

gbc_status gbc_set_device(int device) {
    const int n = gbc_device_count();
    if (n == 0) { set_error("no CUDA device"); return GBC_ERR_NO_DEVICE; }
    if (device < 0 || device >= n) { set_error("device %d out of range [0,%d)", device, n); return GBC_ERR_ARG; }
    GBC_CUDA(cudaSetDevice(device));
    return GBC_OK;
}

void gbc_options_default(gbc_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->semantics = GBC_BC_BRANDES;
    o->delta_precision = GBC_DELTA_F64;
    o->sigma_mode = GBC_SIGMA_AUTO;
    o->engine = GBC_ENGINE_AUTO;
    o->lanes = 0;
    o->sparse_lanes = -1;
    o->levels_per_graph = 0;
    o->source_order = 0;
    o->light_steps = -1;
    o->group_lanes = 0;
}

gbc_status gbc_graph_create(const int64_t* row, const int32_t* col, int32_t n, gbc_graph* out) {
    if (!out) { set_error("out is NULL"); return GBC_ERR_ARG; }
    *out = nullptr;
    GBC_TRY(validate_csr_header(row, col, n));
    if (ensure_device() != GBC_OK) {
        // no device to check on: the host check, so that a bad CSR is still reported as such
        GBC_TRY(validate_csr(row, col, n));
        return ensure_device();
    }
    auto G = std::make_unique<gbc_graph_s>();
    GBC_TRY(graph_upload(row, col, n, G.get()));
    GBC_TRY(validate_device(G.get(), col));
    GBC_TRY(finish_graph(G.get()));
    *out = G.release();
    return GBC_OK;
}

gbc_status gbc_graph_from_edges_device(const int32_t* d_u, const int32_t* d_v, int64_t m, int32_t n, gbc_graph* out) {
    if (!out || n <= 0 || m < 0 || (m > 0 && (!d_u || !d_v))) { set_error("bad arguments"); return GBC_ERR_ARG; }
    *out = nullptr;
    GBC_TRY(ensure_device());
    auto G = std::make_unique<gbc_graph_s>();
    GBC_CUDA(cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking));
    GBC_CUDA(cudaEventCreate(&G->ev0));
    GBC_CUDA(cudaEventCreate(&G->ev1));
    int64_t M = 0;
    GBC_TRY(csr_from_edges_device(d_u, d_v, m, n, G->stream, &G->g.row, &G->g.col, &M));
    G->g.n = n;
    G->g.m = M;
    GBC_TRY(finish_graph(G.get()));
    *out = G.release();
    return GBC_OK;
}

gbc_status gbc_graph_from_edges(const int32_t* u, const int32_t* v, int64_t m, int32_t n, gbc_graph* out) {
    if (!out || n <= 0 || m < 0 || (m > 0 && (!u || !v))) { set_error("bad arguments"); return GBC_ERR_ARG; }
    GBC_TRY(ensure_device());
    int32_t *du = nullptr, *dv = nullptr;
    if (cudaMalloc(&du, sizeof(int32_t) * std::max<int64_t>(m, 1)) != cudaSuccess ||
        cudaMalloc(&dv, sizeof(int32_t) * std::max<int64_t>(m, 1)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(du);
        set_error("edge list upload buffers");
        return GBC_ERR_NOMEM;
    }
    gbc_status st = GBC_OK;
    if (m && (cudaMemcpy(du, u, sizeof(int32_t) * m, cudaMemcpyHostToDevice) != cudaSuccess ||
              cudaMemcpy(dv, v, sizeof(int32_t) * m, cudaMemcpyHostToDevice) != cudaSuccess)) {
        cudaGetLastError();
        set_error("edge list upload failed");
        st = GBC_ERR_CUDA;
    }
    if (st == GBC_OK) st = gbc_graph_from_edges_device(du, dv, m, n, out);
    cudaFree(du);
    cudaFree(dv);
    return st;
}

gbc_status gbc_graph_export(gbc_graph G, int64_t** row, int32_t** col, int32_t* n) {
    if (!G || !row || !col || !n) { set_error("NULL argument"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    const int32_t nn = G->g.n;
    std::vector<int64_t> irow((size_t)nn + 1);
    std::vector<int32_t> icol(std::max<int64_t>(G->g.m, 1)), order(nn);
    GBC_CUDA(cudaMemcpy(irow.data(), G->g.row, sizeof(int64_t) * (nn + 1), cudaMemcpyDeviceToHost));
    if (G->g.m) GBC_CUDA(cudaMemcpy(icol.data(), G->g.col, sizeof(int32_t) * G->g.m, cudaMemcpyDeviceToHost));
    GBC_CUDA(cudaMemcpy(order.data(), G->d_order, sizeof(int32_t) * nn, cudaMemcpyDeviceToHost));
    // rows back in the caller's ids, ascending
    HostCSR h;
    h.n = nn;
    h.row.assign((size_t)nn + 1, 0);
    for (int32_t v = 0; v < nn; v++) {
        const int32_t u = G->h_inv[v];
        h.row[v + 1] = h.row[v] + (irow[u + 1] - irow[u]);
    }
    h.col.resize(G->g.m);
    for (int32_t v = 0; v < nn; v++) {
        const int32_t u = G->h_inv[v];
        int32_t* dst = h.col.data() + h.row[v];
        for (int64_t j = irow[u]; j < irow[u + 1]; j++) *dst++ = order[icol[j]];
        std::sort(h.col.data() + h.row[v], dst);
    }
    *n = nn;
    return export_csr(h, row, col);
}

gbc_status gbc_graph_create_device(const int64_t* d_row, const int32_t* d_col, int32_t n, int64_t m, gbc_graph* out) {
    if (!out || !d_row || (m > 0 && !d_col) || n <= 0 || m < 0) { set_error("bad arguments"); return GBC_ERR_ARG; }
    *out = nullptr;
    GBC_TRY(ensure_device());
    int64_t r0 = 0, rn = 0;
    GBC_CUDA(cudaMemcpy(&r0, d_row, sizeof r0, cudaMemcpyDeviceToHost));
    GBC_CUDA(cudaMemcpy(&rn, d_row + n, sizeof rn, cudaMemcpyDeviceToHost));
    if (rn != m) { set_error("row[n] != m"); return GBC_ERR_ARG; }
    if (r0 != 0) { set_error("row[0] must be 0"); return GBC_ERR_ARG; }
    if (m >= ((int64_t)1 << 31)) { set_error("more than 2^31-1 directed edges (%lld)", (long long)m); return GBC_ERR_ARG; }
    auto G = std::make_unique<gbc_graph_s>();
    GBC_TRY(graph_alloc(n, m, G.get()));
    GBC_CUDA(cudaMemcpyAsync(G->g.row, d_row, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToDevice, G->stream));
    if (m) GBC_CUDA(cudaMemcpyAsync(G->g.col, d_col, sizeof(int32_t) * m, cudaMemcpyDeviceToDevice, G->stream));
    GBC_TRY(validate_device(G.get(), nullptr));
    GBC_TRY(finish_graph(G.get()));
    *out = G.release();
    return GBC_OK;
}

gbc_status gbc_graph_set_weights(gbc_graph G, const int32_t* w, const int64_t* ff) {
    if (!G) { set_error("graph is NULL"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    const int32_t n = G->g.n;
    if (w)
        for (int32_t v = 0; v < n; v++)
            if (w[v] < 0) { set_error("weight w[%d] = %d is negative", v, w[v]); return GBC_ERR_ARG; }
    if (ff)
        for (int32_t v = 0; v < n; v++)
            if (ff[v] < 0) { set_error("ff[%d] = %lld is negative", v, (long long)ff[v]); return GBC_ERR_ARG; }
    // the captured level loops hold the old pointers
    G->eng.reset();
    G->g.w = nullptr;
    G->g.ff = nullptr;
    cudaFree(G->d_w);
    cudaFree(G->d_ff);
    G->d_w = nullptr;
    G->d_ff = nullptr;
    if (!w && !ff) return GBC_OK;
    // caller ids -> internal ids: internal[new] = caller[order[new]]
    void* tmp = nullptr;
    if (cudaMalloc(&tmp, sizeof(int64_t) * std::max<int32_t>(n, 1)) != cudaSuccess) {
        cudaGetLastError();
        set_error("weight staging buffer");
        return GBC_ERR_NOMEM;
    }
    std::unique_ptr<void, void (*)(void*)> keep(tmp, [](void* p) { cudaFree(p); });
    if (w) {
        if (cudaMalloc(&G->d_w, sizeof(int32_t) * std::max<int32_t>(n, 1)) != cudaSuccess) {
            cudaGetLastError();
            set_error("weight buffer");
            return GBC_ERR_NOMEM;
        }
        GBC_CUDA(cudaMemcpyAsync(tmp, w, sizeof(int32_t) * n, cudaMemcpyHostToDevice, G->stream));
        GBC_TRY(gather_to_caller<int32_t>(static_cast<const int32_t*>(tmp), G->d_order, n, 1, G->d_w, G->stream));
        G->g.w = G->d_w;
    }
    if (ff) {
        if (cudaMalloc(&G->d_ff, sizeof(int64_t) * std::max<int32_t>(n, 1)) != cudaSuccess) {
            cudaGetLastError();
            set_error("ff buffer");
            return GBC_ERR_NOMEM;
        }
        GBC_CUDA(cudaMemcpyAsync(tmp, ff, sizeof(int64_t) * n, cudaMemcpyHostToDevice, G->stream));
        GBC_TRY(gather_to_caller<uint64_t>(static_cast<const uint64_t*>(tmp), G->d_order, n, 1,
                                           reinterpret_cast<uint64_t*>(G->d_ff), G->stream));
        G->g.ff = G->d_ff;
    }
    GBC_CUDA(cudaStreamSynchronize(G->stream));
    return GBC_OK;
}

gbc_status gbc_graph_destroy(gbc_graph g) {
    if (!g) { set_error("graph is NULL"); return GBC_ERR_ARG; }
    delete g;
    return GBC_OK;
}

gbc_status gbc_graph_info(gbc_graph G, int32_t* n, int64_t* m, size_t* bytes) {
    if (!G) { set_error("graph is NULL"); return GBC_ERR_ARG; }
    if (n) *n = G->g.n;
    if (m) *m = G->g.m;
    if (bytes) *bytes = sizeof(int64_t) * (G->g.n + 1) + sizeof(int32_t) * G->g.m + (G->eng ? G->eng->device_bytes() : 0);
    return GBC_OK;
}

gbc_status gbc_graph_last_levels(gbc_graph G, int64_t* entries, int32_t entries_cap, float* fwd_ms, float* bwd_ms,
                                 int32_t launch_cap, int32_t* levels, int32_t* fwd_launches, int32_t* bwd_launches) {
    if (!G) { set_error("graph is NULL"); return GBC_ERR_ARG; }
    if (entries_cap < 0 || launch_cap < 0) { set_error("negative capacity"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    const int32_t nl = (int32_t)G->last_level_entries.size();
    const int32_t nf = (int32_t)G->last_fwd_launch_ms.size(), nb = (int32_t)G->last_bwd_launch_ms.size();
    if (levels) *levels = nl;
    if (fwd_launches) *fwd_launches = nf;
    if (bwd_launches) *bwd_launches = nb;
    if (entries) std::memcpy(entries, G->last_level_entries.data(), sizeof(int64_t) * std::min(nl, entries_cap));
    if (fwd_ms) std::memcpy(fwd_ms, G->last_fwd_launch_ms.data(), sizeof(float) * std::min(nf, launch_cap));
    if (bwd_ms) std::memcpy(bwd_ms, G->last_bwd_launch_ms.data(), sizeof(float) * std::min(nb, launch_cap));
    return GBC_OK;
}

gbc_status gbc_graph_last_stats(gbc_graph G, gbc_run_stats* st) {
    if (!G || !st) { set_error("NULL argument"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    if (G->last.edges_traversed < 0) {
        GBC_TRY(ensure_components(G));
        int64_t e = 0;
        for (int32_t x : G->last_src) e += G->g.comp_edges[G->g.comp[x]];
        G->last.edges_traversed = e;
    }
    *st = G->last;
    return GBC_OK;
}

gbc_status gbc_bc(gbc_graph G, const int32_t* sources, int32_t k, const gbc_options* opt, double* bc) {
    if (!G || !bc) { set_error("NULL graph or output"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    const double t0 = now_ms();
    gbc_options o;
    GBC_TRY(resolve_options(opt, o));
    GBC_TRY(check_weighted(G, o, true));
    std::vector<int32_t> hsrc, pos;
    GBC_TRY(resolve_sources(G, sources, k, hsrc));
    GBC_TRY(order_sources(G, o, true, hsrc, pos));
    GBC_TRY(upload_sources(G, hsrc));
    const int32_t kk = (int32_t)hsrc.size();
    GBC_TRY(ensure_bc_buffer(&G->d_bc, G->g.n));
    GBC_TRY(ensure_bc_buffer(&G->d_bc_out, G->g.n));
    LaneResult res;
    int32_t lanes = 0;
    int sig = 0;
    int64_t batches = 0;
    GBC_CUDA(cudaEventRecord(G->ev0, G->stream));
    GBC_TRY(bc_core(G, G->d_src, kk, o, G->d_bc, res, lanes, sig, batches));
    GBC_TRY(gather_to_caller<double>(G->d_bc, G->d_inv, G->g.n, 1, G->d_bc_out, G->stream));
    GBC_CUDA(cudaEventRecord(G->ev1, G->stream));
    GBC_CUDA(cudaMemcpyAsync(bc, G->d_bc_out, sizeof(double) * G->g.n, cudaMemcpyDeviceToHost, G->stream));
    GBC_CUDA(cudaStreamSynchronize(G->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, G->ev0, G->ev1);
    finish_stats(G, res, kk, batches, lanes, sig, hsrc, ms, now_ms() - t0);
    return GBC_OK;
}

gbc_status gbc_bc_device(gbc_graph G, const int32_t* d_sources, int32_t k, const gbc_options* opt, double* d_bc,
                         void* stream) {
    if (!G || !d_bc || !d_sources || k <= 0) { set_error("bad arguments"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    const double t0 = now_ms();
    gbc_options o;
    GBC_TRY(resolve_options(opt, o));
    GBC_TRY(check_weighted(G, o, true));
    cudaStream_t us = (cudaStream_t)stream;
    GBC_CUDA(cudaEventRecord(G->ev0, us));
    GBC_CUDA(cudaStreamWaitEvent(G->stream, G->ev0, 0));
    // the source list comes to the host (k ints) to be validated and grouped
    std::vector<int32_t> hsrc(k), pos;
    GBC_CUDA(cudaMemcpyAsync(hsrc.data(), d_sources, sizeof(int32_t) * k, cudaMemcpyDeviceToHost, G->stream));
    GBC_CUDA(cudaStreamSynchronize(G->stream));
    for (int32_t i = 0; i < k; i++)
        if (hsrc[i] < 0 || hsrc[i] >= G->g.n) { set_error("source %d out of range [0,%d)", hsrc[i], G->g.n); return GBC_ERR_ARG; }
    map_sources(G, hsrc);
    GBC_TRY(order_sources(G, o, true, hsrc, pos));
    GBC_TRY(upload_sources(G, hsrc));
    LaneResult res;
    int32_t lanes = 0;
    int sig = 0;
    int64_t batches = 0;
    GBC_CUDA(cudaEventRecord(G->ev0, G->stream));
    GBC_TRY(ensure_bc_buffer(&G->d_bc, G->g.n));
    GBC_TRY(bc_core(G, G->d_src, k, o, G->d_bc, res, lanes, sig, batches));
    GBC_TRY(gather_to_caller<double>(G->d_bc, G->d_inv, G->g.n, 1, d_bc, G->stream));
    GBC_CUDA(cudaEventRecord(G->ev1, G->stream));
    GBC_CUDA(cudaStreamWaitEvent(us, G->ev1, 0));
    GBC_CUDA(cudaEventSynchronize(G->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, G->ev0, G->ev1);
    finish_stats(G, res, k, batches, lanes, sig, hsrc, ms, now_ms() - t0);
    return GBC_OK;
}

// Device time (forward + dependency sweep) of one betweenness batch of the
// staged sources d_src[0..kb) with the given expansion settings.
static gbc_status tune_batch(gbc_graph_s* G, int32_t lanes, int32_t kb, const gbc_options& o, int sparse, int light,
                             int lpg, int group, int block, double& ms) {
    LaneEngine* E = nullptr;
    gbc_options og = o;
    og.group_lanes = group;
    GBC_TRY(get_engine(G, lanes, true, og, &E));
    E->set_tuning(sparse, light, lpg, block, -1);
    GBC_TRY(E->bc_begin());
    LaneRequest rq;
    rq.job = LaneJob::BC;
    rq.d_src = G->d_src;
    rq.kb = kb;
    rq.delta_f64 = o.delta_precision == GBC_DELTA_F64;
    rq.semantics = o.semantics;
    rq.sigma_wide = o.sigma_mode == GBC_SIGMA_WIDE;
    rq.abort_on_overflow = !rq.sigma_wide;
    LaneResult res;
    gbc_status st = E->run(rq, res);
    if (st == GBC_ERR_OVERFLOW && o.sigma_mode == GBC_SIGMA_AUTO) {
        rq.sigma_wide = 1;
        rq.abort_on_overflow = false;
        LaneResult r2;
        st = E->run(rq, r2);
        res = r2;
    }
    if (st != GBC_OK) return st;
    GBC_CUDA(cudaStreamSynchronize(G->stream));
    ms = res.fwd_ms + res.bwd_ms;
    return GBC_OK;
}

// One closeness batch on the tuned engine with direction-switch share `share`
// (0: top-down only); its forward device time.
static gbc_status tune_cc_batch(gbc_graph_s* G, int32_t kb, int share, double& ms) {
    LaneEngine* E = G->eng.get();
    E->set_tuning(G->tuned.sparse, G->tuned.light, G->tuned.lpg, G->tuned.block, share);
    LaneRequest rq;
    rq.job = LaneJob::CC;
    rq.d_src = G->d_src;
    rq.kb = kb;
    LaneResult res;
    GBC_TRY(E->run(rq, res));
    GBC_CUDA(cudaStreamSynchronize(G->stream));
    ms = res.fwd_ms;
    return GBC_OK;
}

gbc_status gbc_autotune(gbc_graph G, const int32_t* sources, int32_t k, const gbc_options* opt, gbc_options* chosen) {
    if (!G) { set_error("graph is NULL"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    gbc_options o;
    GBC_TRY(resolve_options(opt, o));
    GBC_TRY(check_weighted(G, o, true));
    if (o.engine == GBC_ENGINE_PLAIN) { set_error("autotuning applies to the lane engine"); return GBC_ERR_ARG; }
    std::vector<int32_t> hsrc, pos;
    GBC_TRY(resolve_sources(G, sources, k, hsrc));
    G->tuned.done = false;
    const int32_t k0 = (int32_t)hsrc.size();
    int32_t lanes = pick_lanes(G, k0, true, o.lanes, group_of(G, o));
    GBC_TRY(order_sources(G, o, true, hsrc, pos));
    GBC_TRY(upload_sources(G, hsrc));
    // candidate settings; the options' explicit values are kept fixed
    const int sp0 = o.sparse_lanes >= 0 ? o.sparse_lanes : 2;
    const int li0 = o.light_steps >= 0 ? o.light_steps : 16;
    const int lp0 = o.levels_per_graph > 0 ? o.levels_per_graph : 16;
    const int gr0 = o.group_lanes ? o.group_lanes : 32;
    const int bt0 = o.block_threads ? o.block_threads : 256;
    int best_sp = sp0, best_li = li0, best_lp = lp0, best_gr = gr0, best_bt = bt0;
    double best = 0;
    const int32_t kb = std::min(lanes, k0);
    GBC_TRY(tune_batch(G, lanes, kb, o, sp0, li0, lp0, gr0, bt0, best));   // warm-up: level width, queue size, graph capture
    // a candidate's time: the better of two batches (single batches vary by a few percent, about
    // as much as neighbouring settings differ)
    auto timed = [&](int32_t w, int32_t kk, int sp, int li, int lp, int gr, int bt, double& ms) -> gbc_status {
        double a = 0, b = 0;
        GBC_TRY(tune_batch(G, w, kk, o, sp, li, lp, gr, bt, a));
        GBC_TRY(tune_batch(G, w, kk, o, sp, li, lp, gr, bt, b));
        ms = std::min(a, b);
        return GBC_OK;
    };
    auto consider = [&](int sp, int li, int lp, int bt) -> gbc_status {
        double ms = 0;
        GBC_TRY(timed(lanes, kb, sp, li, lp, best_gr, bt, ms));
        if (ms < best) { best = ms; best_sp = sp; best_li = li; best_lp = lp; best_bt = bt; }
        return GBC_OK;
    };
    GBC_TRY(timed(lanes, kb, sp0, li0, lp0, gr0, bt0, best));
    // lanes per group first: 128-lane groups (four lanes per thread) against 32, and on deep graphs
    // of low degree one lane per task (lanes whose sources lie far apart rarely share a level)
    if (o.group_lanes == 0 && lanes % 128 == 0) {
        double ms = 0;
        GBC_TRY(tune_batch(G, lanes, kb, o, sp0, li0, lp0, 128, bt0, ms));   // warm-up of the 128-lane engine
        GBC_TRY(timed(lanes, kb, sp0, li0, lp0, 128, bt0, ms));
        if (ms < best) { best = ms; best_gr = 128; }
    }
    if (o.group_lanes == 0 && G->key_depth > SMALL_WORLD_DEPTH && G->g.max_degree <= ONE_LANE_MAX_DEGREE &&
        G->g.n < ONE_LANE_MAX_N) {
        double ms = 0;
        GBC_TRY(tune_batch(G, lanes, kb, o, sp0, li0, lp0, 1, bt0, ms));   // warm-up of the one-lane engine
        GBC_TRY(timed(lanes, kb, sp0, li0, lp0, 1, bt0, ms));
        if (ms < best) { best = ms; best_gr = 1; }
    }
    // one-thread tasks, then the edge-parallel threshold, then the level-loop graph length
    if (o.light_steps < 0 && best_gr == 32)   // only 32-lane groups have one-thread tasks
        for (int li : {0, 8, 32}) GBC_TRY(consider(best_sp, li, best_lp, best_bt));
    if (o.sparse_lanes < 0 && best_gr != 1)   // one lane per task has no lane-parallel expansion
        for (int sp : {1, 4}) GBC_TRY(consider(sp, best_li, best_lp, best_bt));
    if (o.levels_per_graph <= 0 && G->eng && G->eng->level_bytes() == 2) GBC_TRY(consider(best_sp, best_li, 64, best_bt));
    // CTA shape of the level kernels
    if (o.block_threads == 0)
        for (int bt : {128, 512}) GBC_TRY(consider(best_sp, best_li, best_lp, bt));
    // batch width: halve while the time per source drops (down to 32 lanes)
    int32_t best_lanes = lanes;
    if (o.lanes == 0 && kb == lanes) {
        double per_src = best / lanes;
        for (int32_t w = lanes / 2; w >= 32; w /= 2) {
            double ms = 0;
            const int gw = (best_gr == 1 || w % 128 == 0) ? best_gr : 32;
            GBC_TRY(tune_batch(G, w, w, o, best_sp, best_li, best_lp, gw, best_bt, ms));   // warm-up of the narrower engine
            GBC_TRY(timed(w, w, best_sp, best_li, best_lp, gw, best_bt, ms));
            if (ms / w >= per_src) break;
            per_src = ms / w;
            best_lanes = w;
        }
    }
    G->tuned.lanes = o.lanes ? 0 : best_lanes;
    G->tuned.sparse = best_sp;
    G->tuned.light = best_li;
    G->tuned.lpg = best_lp;
    G->tuned.group = best_gr;
    G->tuned.block = best_bt;
    G->tuned.share = -1;
    // closeness direction threshold (128-lane groups only switch direction):
    // one closeness batch of the same sources per share, 0 = top-down only
    int best_share = o.bu_share > 0 ? o.bu_share : 16;
    bool bu_tuned = false;
    if (o.bu_share == 0 && o.direction == 0 && best_gr == 128 && G->eng && G->eng->group_lanes() == 128) {
        const int32_t kc = std::min(G->eng->lanes(), k0);
        double ms = 0, ms2 = 0, best_cc = 0;
        GBC_TRY(tune_cc_batch(G, kc, 16, ms));        // warm-up: component labels, graph capture
        GBC_TRY(tune_cc_batch(G, kc, 16, best_cc));
        GBC_TRY(tune_cc_batch(G, kc, 16, ms2));
        best_cc = std::min(best_cc, ms2);
        for (int sh : {0, 4, 8, 32, 64}) {
            GBC_TRY(tune_cc_batch(G, kc, sh, ms));
            GBC_TRY(tune_cc_batch(G, kc, sh, ms2));
            ms = std::min(ms, ms2);
            if (ms < best_cc) { best_cc = ms; best_share = sh; }
        }
        G->tuned.share = best_share;
        bu_tuned = true;
    }
    G->tuned.done = true;
    if (chosen) {
        *chosen = o;
        chosen->lanes = best_lanes;
        chosen->sparse_lanes = best_sp;
        chosen->light_steps = best_li;
        chosen->levels_per_graph = best_lp;
        chosen->group_lanes = best_gr;
        chosen->block_threads = best_bt;
        chosen->bu_share = best_share;
        if (bu_tuned && best_share == 0) chosen->direction = 1;
    }
    return GBC_OK;
}

gbc_status gbc_cc(gbc_graph G, const int32_t* sources, int32_t k, const gbc_options* opt, int64_t* cc) {
    if (!G || !cc) { set_error("NULL graph or output"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    const double t0 = now_ms();
    gbc_options o;
    GBC_TRY(resolve_options(opt, o));
    GBC_TRY(check_weighted(G, o, false));
    std::vector<int32_t> hsrc, pos;
    GBC_TRY(resolve_sources(G, sources, k, hsrc));
    GBC_TRY(order_sources(G, o, false, hsrc, pos));
    GBC_TRY(upload_sources(G, hsrc));
    const int32_t kk = (int32_t)hsrc.size();
    if (kk > G->ccb_cap) {
        cudaFree(G->d_ccb);
        G->d_ccb = nullptr;
        if (cudaMalloc(&G->d_ccb, sizeof(unsigned long long) * kk) != cudaSuccess) { cudaGetLastError(); set_error("cc buffer"); return GBC_ERR_NOMEM; }
        G->ccb_cap = kk;
    }
    LaneResult res;
    int32_t lanes = 0;
    int64_t batches = 0;
    GBC_CUDA(cudaEventRecord(G->ev0, G->stream));
    std::vector<int64_t> ordered(kk);
    GBC_TRY(cc_core(G, G->d_src, hsrc.data(), kk, o, G->d_ccb, ordered.data(), res, lanes, batches));
    GBC_CUDA(cudaEventRecord(G->ev1, G->stream));
    if (o.engine != GBC_ENGINE_PLAIN)
        GBC_CUDA(cudaMemcpyAsync(ordered.data(), G->d_ccb, sizeof(int64_t) * kk, cudaMemcpyDeviceToHost, G->stream));
    GBC_CUDA(cudaStreamSynchronize(G->stream));
    for (int32_t i = 0; i < kk; i++) cc[pos[i]] = ordered[i];
    float ms = 0;
    cudaEventElapsedTime(&ms, G->ev0, G->ev1);
    finish_stats(G, res, kk, batches, lanes, GBC_SIGMA_EXACT, hsrc, ms, now_ms() - t0);
    return GBC_OK;
}

gbc_status gbc_cc_device(gbc_graph G, const int32_t* d_sources, int32_t k, const gbc_options* opt, int64_t* d_cc,
                         void* stream) {
    if (!G || !d_cc || !d_sources || k <= 0) { set_error("bad arguments"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    const double t0 = now_ms();
    gbc_options o;
    GBC_TRY(resolve_options(opt, o));
    GBC_TRY(check_weighted(G, o, false));
    if (o.engine == GBC_ENGINE_PLAIN) { set_error("gbc_cc_device runs the lane engine only"); return GBC_ERR_ARG; }
    cudaStream_t us = (cudaStream_t)stream;
    GBC_CUDA(cudaEventRecord(G->ev0, us));
    GBC_CUDA(cudaStreamWaitEvent(G->stream, G->ev0, 0));
    std::vector<int32_t> hsrc(k), pos;
    GBC_CUDA(cudaMemcpyAsync(hsrc.data(), d_sources, sizeof(int32_t) * k, cudaMemcpyDeviceToHost, G->stream));
    GBC_CUDA(cudaStreamSynchronize(G->stream));
    for (int32_t i = 0; i < k; i++)
        if (hsrc[i] < 0 || hsrc[i] >= G->g.n) { set_error("source %d out of range [0,%d)", hsrc[i], G->g.n); return GBC_ERR_ARG; }
    map_sources(G, hsrc);
    GBC_TRY(order_sources(G, o, false, hsrc, pos));
    GBC_TRY(upload_sources(G, hsrc));
    if (k > G->ccb_cap) {
        cudaFree(G->d_ccb);
        G->d_ccb = nullptr;
        if (cudaMalloc(&G->d_ccb, sizeof(unsigned long long) * k) != cudaSuccess) { cudaGetLastError(); set_error("cc buffer"); return GBC_ERR_NOMEM; }
        G->ccb_cap = k;
    }
    if (k > G->pos_cap) {
        cudaFree(G->d_pos);
        G->d_pos = nullptr;
        if (cudaMalloc(&G->d_pos, sizeof(int32_t) * k) != cudaSuccess) { cudaGetLastError(); set_error("position buffer"); return GBC_ERR_NOMEM; }
        G->pos_cap = k;
    }
    GBC_CUDA(cudaMemcpyAsync(G->d_pos, pos.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice, G->stream));
    LaneResult res;
    int32_t lanes = 0;
    int64_t batches = 0;
    GBC_CUDA(cudaEventRecord(G->ev0, G->stream));
    GBC_TRY(cc_core(G, G->d_src, nullptr, k, o, G->d_ccb, nullptr, res, lanes, batches));
    scatter_cc_kernel<<<std::max(1, std::min(1024, (k + 255) / 256)), 256, 0, G->stream>>>(G->d_ccb, G->d_pos, k, d_cc);
    GBC_CUDA(cudaGetLastError());
    GBC_CUDA(cudaEventRecord(G->ev1, G->stream));
    GBC_CUDA(cudaStreamWaitEvent(us, G->ev1, 0));
    GBC_CUDA(cudaEventSynchronize(G->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, G->ev0, G->ev1);
    finish_stats(G, res, k, batches, lanes, GBC_SIGMA_EXACT, hsrc, ms, now_ms() - t0);
    return GBC_OK;
}

gbc_status gbc_sssp(gbc_graph G, const int32_t* sources, int32_t k, const gbc_options* opt, int32_t* dist,
                    uint64_t* sigma, uint8_t* ovf) {
    if (!G || !sources || k <= 0) { set_error("bad arguments"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(G->mu);
    gbc_options o;
    GBC_TRY(resolve_options(opt, o));
    std::vector<int32_t> hsrc;
    GBC_TRY(resolve_sources(G, sources, k, hsrc));
    GBC_TRY(upload_sources(G, hsrc));
    const int32_t n = G->g.n;
    const int32_t grp = group_of(G, o) == 1 ? 32 : group_of(G, o);   // batches stay a multiple of 32 lanes
    const int32_t lanes = o.lanes ? o.lanes : std::min<int32_t>(1024, ((k + grp - 1) / grp) * grp);
    LaneEngine* E = nullptr;
    GBC_TRY(get_engine(G, lanes, true, o, &E));
    int32_t* d_dist = nullptr;
    uint64_t* d_sig = nullptr;
    const size_t cells = (size_t)std::min(lanes, k) * n;
    if (cudaMalloc(&d_dist, 2 * cells * sizeof(int32_t)) != cudaSuccess || cudaMalloc(&d_sig, 2 * cells * sizeof(uint64_t)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_dist);
        set_error("sssp output buffers");
        return GBC_ERR_NOMEM;
    }
    std::unique_ptr<void, void (*)(void*)> f1(d_dist, [](void* p) { cudaFree(p); });
    std::unique_ptr<void, void (*)(void*)> f2(d_sig, [](void* p) { cudaFree(p); });
    LaneResult res;
    for (int32_t b0 = 0; b0 < k; b0 += lanes) {
        LaneRequest rq;
        rq.job = LaneJob::SSSP;
        rq.d_src = G->d_src + b0;
        rq.kb = std::min(lanes, k - b0);
        rq.d_dist = d_dist;
        rq.d_sigma = d_sig;
        GBC_TRY(E->run(rq, res));
        const size_t c = (size_t)rq.kb * n;
        // per-vertex rows back to the caller's ids, through the second halves of the buffers
        GBC_TRY(gather_to_caller<int32_t>(d_dist, G->d_inv, n, rq.kb, d_dist + cells, G->stream));
        GBC_TRY(gather_to_caller<uint64_t>(d_sig, G->d_inv, n, rq.kb, d_sig + cells, G->stream));
        if (dist) GBC_CUDA(cudaMemcpyAsync(dist + (size_t)b0 * n, d_dist + cells, c * sizeof(int32_t), cudaMemcpyDeviceToHost, G->stream));
        if (sigma) GBC_CUDA(cudaMemcpyAsync(sigma + (size_t)b0 * n, d_sig + cells, c * sizeof(uint64_t), cudaMemcpyDeviceToHost, G->stream));
        GBC_CUDA(cudaStreamSynchronize(G->stream));
        if (ovf)
            for (int32_t l = 0; l < rq.kb; l++) ovf[b0 + l] = (res.ovf_bits[l >> 5] >> (l & 31)) & 1u;
    }
    return GBC_OK;
}

}  // extern "C"
