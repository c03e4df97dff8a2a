// D1 folding + articulation-point (block) reduction for closeness and
// betweenness.
//
// Folding (as Lib/D1Process/D1Process.c:32-73): degree-1 vertices are peeled
// repeatedly into their neighbour, which accumulates reach r (vertices it
// stands for) and ff (sum of distances from it to the vertices folded into
// it).  A vertex whose last neighbour was folded into it is the root of a
// tree component and stays.
//
// Splitting: the folded graph is cut into biconnected blocks (Hopcroft-Tarjan
// with an edge stack).  For a block B and a vertex b of B that is an
// articulation point, the clone weight w'_B(b) = r(b) + reach of every vertex
// separated from B by b (the AP clones of Lib/AP_Process/AP_Process.c:916-1020
// carry the same reach).  Then for every vertex v and any block B holding v
//     CC(v) = FF_B + D_B(v),   D_B(v) = sum_{u in B} d_B(v,u) * w'_B(u)
// where FF_B = sum_{u in B} ff'_B(u) and ff'_B(b) folds the distance sums of
// everything behind b.  D_B is a weighted distance sum computed for every
// (block, vertex) slot by the lane engine on the disjoint union of the
// blocks; FF_B follows from two passes over the block-cut tree on the host.
// Folded vertices are recovered in reverse folding order with
//     CC(d1) = CC(parent) + N_c - 2 r(d1)
// (Seq_CC/CC.cpp:2037-2049) where N_c is the size of d1's connected
// component (the reference uses the global vertex count, which is only right
// for connected graphs).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>

#include "engine.h"
#include "reduce.h"

namespace gbc {

struct Reduction {
    int32_t n = 0, start = 0;
    // folding
    std::vector<int64_t> r, ff;       // reach and folded distance sums
    std::vector<int32_t> parent;      // folded vertex -> vertex it was folded into
    std::vector<int32_t> fold_order;
    std::vector<int64_t> fold_rp;     // reach of the parent just before it absorbed fold_order[i]
    std::vector<uint8_t> folded, is_ap;
    // folded graph ("core": unfolded vertices, live edges) for betweenness
    HostCSR core;
    std::vector<int32_t> core_v;      // core id -> vertex
    std::vector<int32_t> core_w;      // reach of each core vertex
    int32_t n_hub = 0;
    // connected components of the folded graph (alive vertices)
    std::vector<int32_t> comp;        // per vertex slot (-1 for the phantom slot)
    std::vector<int64_t> comp_w;      // total reach per component
    int32_t n_comp = 0;
    // blocks
    int32_t n_blocks = 0;
    std::vector<int64_t> bvoff;       // block -> first slot
    std::vector<int32_t> slot_v;      // slot -> vertex
    std::vector<int32_t> slot_w;      // slot -> clone weight w'
    std::vector<int32_t> vslot;       // vertex -> one slot holding it (its only slot unless AP)
    HostCSR bg;                       // block graph over slots
    // block-cut tree
    std::vector<int32_t> bparent_ap;  // block -> parent AP vertex (-1 for a root block)
    std::vector<int32_t> ap_parent_block;  // vertex -> parent block (APs only)
    std::vector<std::vector<int32_t>> ap_child_blocks;  // per AP vertex (index by vertex via map)
    std::vector<int32_t> ap_index;    // vertex -> index into ap_child_blocks (-1 if not AP)
    std::vector<int32_t> border;      // blocks in BFS order from the roots
    int32_t max_block = 0;
    // device path: the folded graph and the block graph as the device built
    // them; core / bg above then hold only n until an export asks for the rows
    int64_t* d_core_row = nullptr;
    int32_t* d_core_col = nullptr;
    int64_t core_m = 0;
    int64_t* d_bg_row = nullptr;
    int32_t* d_bg_col = nullptr;
    int64_t bg_m = 0;
    // where the reduction ran, and the device path's round and level counts
    bool on_device = false;
    int32_t fold_rounds = 0, forest_levels = 0;
    // device copy of the block graph
    std::unique_ptr<DevGraph> dg;
    int32_t* d_w = nullptr;
    std::vector<int32_t> b_inv;       // slot -> internal id of the degree-relabelled device block graph
    cudaStream_t stream = nullptr;
    std::unique_ptr<LaneEngine> eng;  // lane engine on the block graph (closeness; betweenness state once asked for)
    // lane grouping of the block graph: level-profile order of its slots
    // (internal ids) and the group width it implies
    std::vector<int32_t> b_order;
    int32_t b_group = 0;
    std::mutex mu;
    ~Reduction() {
        eng.reset();
        if (dg) { cudaFree(dg->row); cudaFree(dg->col); }
        cudaFree(d_w);
        cudaFree(d_core_row);
        cudaFree(d_core_col);
        cudaFree(d_bg_row);
        cudaFree(d_bg_col);
        if (stream) cudaStreamDestroy(stream);
    }
};

// Directed entries of the two graphs, wherever their rows are.
static int64_t core_entries(const Reduction& R) { return R.d_core_row ? R.core_m : R.core.m(); }
static int64_t bg_entries(const Reduction& R) { return R.d_bg_row ? R.bg_m : R.bg.m(); }

// Host rows of a graph that the device path left on the device (for exports).
static gbc_status host_rows(HostCSR& h, const int64_t* d_row, const int32_t* d_col, int64_t m) {
    if (!h.row.empty()) return GBC_OK;
    if (!d_row) {   // an empty graph
        h.row.assign((size_t)h.n + 1, 0);
        return GBC_OK;
    }
    h.row.resize((size_t)h.n + 1);
    h.col.resize((size_t)m);
    GBC_CUDA(cudaMemcpy(h.row.data(), d_row, sizeof(int64_t) * ((size_t)h.n + 1), cudaMemcpyDeviceToHost));
    if (m) GBC_CUDA(cudaMemcpy(h.col.data(), d_col, sizeof(int32_t) * m, cudaMemcpyDeviceToHost));
    return GBC_OK;
}

// A device graph for the lane engine: a copy of the device-built rows, or an upload of the host rows.
static gbc_status graph_rows(DevGraph& g, const HostCSR& h, const int64_t* d_row, const int32_t* d_col) {
    const cudaMemcpyKind k = d_row ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    GBC_CUDA(cudaMemcpy(g.row, d_row ? (const void*)d_row : (const void*)h.row.data(), sizeof(int64_t) * (g.n + 1), k));
    if (g.m) GBC_CUDA(cudaMemcpy(g.col, d_row ? (const void*)d_col : (const void*)h.col.data(), sizeof(int32_t) * g.m, k));
    return GBC_OK;
}

// ---------------------------------------------------------------- fold ----
static void fold(const int64_t* row, const int32_t* col, Reduction& R, std::vector<int32_t>& livecol,
                 std::vector<int64_t>& lo) {
    const int32_t n = R.n;
    livecol.assign(col, col + row[n]);
    lo.assign(row, row + n);
    std::vector<int64_t> deg(n);
    R.r.assign(n, 1);
    R.ff.assign(n, 0);
    R.parent.assign(n, -1);
    R.folded.assign(n, 0);
    std::vector<uint8_t> hub(n, 0);
    std::vector<int32_t> q;
    q.reserve(n);
    for (int32_t v = 0; v < n; v++) {
        deg[v] = row[v + 1] - row[v];
        if (v >= R.start && deg[v] == 1) q.push_back(v);
    }
    for (size_t h = 0; h < q.size(); h++) {
        const int32_t d1 = q[h];
        if (deg[d1] != 1) continue;           // root of a tree component
        const int32_t p = livecol[lo[d1]];
        R.folded[d1] = 1;
        R.parent[d1] = p;
        hub[p] = 1;
        R.fold_rp.push_back(R.r[p]);
        R.r[p] += R.r[d1];
        R.ff[p] += R.r[d1] + R.ff[d1];
        for (int64_t e = lo[p]; e < row[p + 1]; e++)
            if (livecol[e] == d1) { std::swap(livecol[e], livecol[lo[p]]); break; }
        lo[p]++;
        deg[d1] = 0;
        if (--deg[p] == 1) q.push_back(p);
        R.fold_order.push_back(d1);
    }
    R.n_hub = 0;
    for (int32_t v = R.start; v < n; v++) R.n_hub += (hub[v] && !R.folded[v]);
}

// Block-cut tree over the slots (BFS over blocks and articulation points from
// the first block of each component) and the clone weight w' of every slot.
static gbc_status block_tree(Reduction& R) {
    const int32_t n = R.n;
    R.ap_index.assign(n, -1);
    int32_t nap = 0;
    for (int32_t v = 0; v < n; v++) if (R.is_ap[v]) R.ap_index[v] = nap++;
    std::vector<std::vector<int32_t>> ap_blocks(nap);
    for (int32_t b = 0; b < R.n_blocks; b++)
        for (int64_t s = R.bvoff[b]; s < R.bvoff[b + 1]; s++)
            if (R.is_ap[R.slot_v[s]]) ap_blocks[R.ap_index[R.slot_v[s]]].push_back(b);
    R.bparent_ap.assign(R.n_blocks, -2);
    R.ap_parent_block.assign(n, -1);
    R.ap_child_blocks.assign(nap, {});
    R.border.clear();
    for (int32_t b0 = 0; b0 < R.n_blocks; b0++) {
        if (R.bparent_ap[b0] != -2) continue;
        R.bparent_ap[b0] = -1;
        size_t h = R.border.size();
        R.border.push_back(b0);
        while (h < R.border.size()) {
            const int32_t b = R.border[h++];
            for (int64_t s = R.bvoff[b]; s < R.bvoff[b + 1]; s++) {
                const int32_t v = R.slot_v[s];
                if (!R.is_ap[v] || v == R.bparent_ap[b]) continue;
                R.ap_parent_block[v] = b;
                for (int32_t b2 : ap_blocks[R.ap_index[v]]) {
                    if (b2 == b) continue;
                    R.bparent_ap[b2] = v;
                    R.ap_child_blocks[R.ap_index[v]].push_back(b2);
                    R.border.push_back(b2);
                }
            }
        }
    }
    // clone weights: W_sub bottom-up, then w' per slot
    std::vector<int64_t> wsub(R.n_blocks, 0);
    for (int64_t h = (int64_t)R.border.size() - 1; h >= 0; h--) {
        const int32_t b = R.border[h];
        int64_t sum = 0;
        for (int64_t s = R.bvoff[b]; s < R.bvoff[b + 1]; s++) {
            const int32_t v = R.slot_v[s];
            if (v == R.bparent_ap[b]) continue;
            sum += R.r[v];
            if (R.is_ap[v]) for (int32_t b2 : R.ap_child_blocks[R.ap_index[v]]) sum += wsub[b2];
        }
        wsub[b] = sum;
    }
    R.slot_w.resize(R.bg.n);
    for (int32_t b = 0; b < R.n_blocks; b++) {
        for (int64_t s = R.bvoff[b]; s < R.bvoff[b + 1]; s++) {
            const int32_t v = R.slot_v[s];
            int64_t w = R.r[v];
            if (R.is_ap[v]) {
                if (v == R.bparent_ap[b]) w = R.comp_w[R.comp[v]] - wsub[b];
                else for (int32_t b2 : R.ap_child_blocks[R.ap_index[v]]) w += wsub[b2];
            }
            if (w > INT32_MAX) { set_error("clone weight exceeds int32"); return GBC_ERR_ARG; }
            R.slot_w[s] = (int32_t)w;
        }
    }
    return GBC_OK;
}

// ----------------------------------------------------- blocks (Tarjan) ----
static gbc_status split(const int64_t* row, Reduction& R, const std::vector<int32_t>& lc, const std::vector<int64_t>& lo) {
    const int32_t n = R.n;
    std::vector<int32_t> disc(n, 0), low(n, 0), nchild(n, 0);
    std::vector<int64_t> it(n), pedge(n, -1);
    std::vector<int32_t> par(n, -1), stk;
    std::vector<std::pair<int32_t, int32_t>> es;   // edge stack
    std::vector<std::vector<std::pair<int32_t, int32_t>>> block_edges;
    std::vector<std::vector<int32_t>> block_verts;
    R.is_ap.assign(n, 0);
    R.comp.assign(n, -1);
    std::vector<int32_t> mark(n, -1);
    int32_t timer = 0;
    auto close_block = [&](int32_t v, int32_t u) {
        std::vector<std::pair<int32_t, int32_t>> edges;
        std::vector<int32_t> verts;
        const int32_t b = (int32_t)block_edges.size();
        while (!es.empty()) {
            auto e = es.back();
            es.pop_back();
            edges.push_back(e);
            for (int32_t x : {e.first, e.second})
                if (mark[x] != b) { mark[x] = b; verts.push_back(x); }
            if (e.first == v && e.second == u) break;
        }
        std::sort(verts.begin(), verts.end());
        block_edges.push_back(std::move(edges));
        block_verts.push_back(std::move(verts));
    };
    for (int32_t rt = R.start; rt < n; rt++) {
        if (R.folded[rt] || disc[rt]) continue;
        const int32_t c = R.n_comp++;
        R.comp_w.push_back(0);
        if (lo[rt] == row[rt + 1]) {   // isolated alive vertex: a block of its own
            disc[rt] = ++timer;
            R.comp[rt] = c;
            R.comp_w[c] += R.r[rt];
            block_edges.emplace_back();
            block_verts.push_back({rt});
            mark[rt] = (int32_t)block_verts.size() - 1;
            continue;
        }
        stk.clear();
        stk.push_back(rt);
        disc[rt] = low[rt] = ++timer;
        it[rt] = lo[rt];
        R.comp[rt] = c;
        R.comp_w[c] += R.r[rt];
        while (!stk.empty()) {
            const int32_t v = stk.back();
            if (it[v] < row[v + 1]) {
                const int64_t e = it[v]++;
                const int32_t u = lc[e];
                if (u == v) continue;
                if (!disc[u]) {
                    par[u] = v;
                    pedge[u] = e;
                    disc[u] = low[u] = ++timer;
                    it[u] = lo[u];
                    R.comp[u] = c;
                    R.comp_w[c] += R.r[u];
                    nchild[v]++;
                    es.push_back({v, u});
                    stk.push_back(u);
                } else if (disc[u] < disc[v]) {
                    // back edge (the tree edge to the parent is skipped by position,
                    // so a parallel edge to the parent counts as a back edge)
                    bool is_tree = (u == par[v]);
                    if (is_tree) {
                        // find whether e is the reverse of the tree edge: the first
                        // occurrence of par[v] in v's live list is treated as it
                        int64_t first = -1;
                        for (int64_t f = lo[v]; f < row[v + 1]; f++) if (lc[f] == u) { first = f; break; }
                        is_tree = (first == e);
                    }
                    if (!is_tree) {
                        es.push_back({v, u});
                        low[v] = std::min(low[v], disc[u]);
                    }
                }
            } else {
                stk.pop_back();
                const int32_t p = par[v];
                if (p >= 0) {
                    low[p] = std::min(low[p], low[v]);
                    if (low[v] >= disc[p]) {
                        if (par[p] >= 0 || nchild[p] > 1) R.is_ap[p] = 1;
                        close_block(p, v);
                    }
                }
            }
        }
    }
    // slots: blocks in order, vertices sorted within a block
    R.n_blocks = (int32_t)block_verts.size();
    R.bvoff.assign(R.n_blocks + 1, 0);
    for (int32_t b = 0; b < R.n_blocks; b++) R.bvoff[b + 1] = R.bvoff[b] + (int64_t)block_verts[b].size();
    const int64_t ns = R.bvoff[R.n_blocks];
    if (ns >= ((int64_t)1 << 27)) { set_error("block graph too large (%lld slots)", (long long)ns); return GBC_ERR_ARG; }
    R.slot_v.resize(ns);
    R.vslot.assign(n, -1);
    R.max_block = 0;
    for (int32_t b = 0; b < R.n_blocks; b++) {
        R.max_block = std::max<int32_t>(R.max_block, (int32_t)block_verts[b].size());
        for (size_t i = 0; i < block_verts[b].size(); i++) {
            const int32_t v = block_verts[b][i];
            R.slot_v[R.bvoff[b] + i] = v;
            if (R.vslot[v] < 0) R.vslot[v] = (int32_t)(R.bvoff[b] + i);
        }
    }
    // block graph CSR over slots
    // a vertex that is not an articulation point has exactly one slot
    auto slot_of = [&](int32_t b, int32_t v) -> int32_t {
        if (!R.is_ap[v]) return R.vslot[v];
        const auto& V = block_verts[b];
        return (int32_t)(R.bvoff[b] + (std::lower_bound(V.begin(), V.end(), v) - V.begin()));
    };
    std::vector<int64_t> deg(ns + 1, 0);
    for (int32_t b = 0; b < R.n_blocks; b++)
        for (auto& e : block_edges[b]) { deg[slot_of(b, e.first)]++; deg[slot_of(b, e.second)]++; }
    R.bg.n = (int32_t)ns;
    R.bg.row.assign(ns + 1, 0);
    for (int64_t s = 0; s < ns; s++) R.bg.row[s + 1] = R.bg.row[s] + deg[s];
    R.bg.col.resize(R.bg.row[ns]);
    std::vector<int64_t> fill(R.bg.row.begin(), R.bg.row.end() - 1);
    for (int32_t b = 0; b < R.n_blocks; b++)
        for (auto& e : block_edges[b]) {
            const int32_t x = slot_of(b, e.first), y = slot_of(b, e.second);
            R.bg.col[fill[x]++] = y;
            R.bg.col[fill[y]++] = x;
        }
    return block_tree(R);
}

// Degree relabelling of a weighted device graph: the weights move with their
// vertices; inv[old] = new on the host.
static gbc_status relabel_weighted(DevGraph& g, cudaStream_t s, int32_t** d_w, std::vector<int32_t>& inv) {
    inv.resize(g.n);
    if (g.n == 0) return GBC_OK;
    int32_t *d_order = nullptr, *d_inv = nullptr, *w2 = nullptr;
    GBC_TRY(relabel_by_degree(g, s, &d_order, &d_inv));
    std::unique_ptr<void, void (*)(void*)> f1(d_order, [](void* p) { cudaFree(p); });
    std::unique_ptr<void, void (*)(void*)> f2(d_inv, [](void* p) { cudaFree(p); });
    if (cudaMalloc(&w2, sizeof(int32_t) * g.n) != cudaSuccess) { cudaGetLastError(); set_error("weights"); return GBC_ERR_NOMEM; }
    GBC_TRY(gather_to_caller<int32_t>(*d_w, d_order, g.n, 1, w2, s));   // w2[new] = w[order[new]]
    GBC_CUDA(cudaMemcpyAsync(inv.data(), d_inv, sizeof(int32_t) * g.n, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    cudaFree(*d_w);
    *d_w = w2;
    return GBC_OK;
}

static gbc_status upload(Reduction& R) {
    if (R.dg) return GBC_OK;
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) { cudaGetLastError(); set_error("no CUDA device"); return GBC_ERR_NO_DEVICE; }
    GBC_CUDA(cudaStreamCreateWithFlags(&R.stream, cudaStreamNonBlocking));
    auto g = std::make_unique<DevGraph>();
    g->n = R.bg.n;
    g->m = bg_entries(R);
    bool ok = cudaMalloc(&g->row, sizeof(int64_t) * (g->n + 1)) == cudaSuccess;
    ok &= cudaMalloc(&g->col, sizeof(int32_t) * std::max<int64_t>(g->m, 1)) == cudaSuccess;
    ok &= cudaMalloc(&R.d_w, sizeof(int32_t) * std::max<int32_t>(g->n, 1)) == cudaSuccess;
    if (!ok) { cudaGetLastError(); set_error("block graph allocation"); cudaFree(g->row); cudaFree(g->col); return GBC_ERR_NOMEM; }
    GBC_TRY(graph_rows(*g, R.bg, R.d_bg_row, R.d_bg_col));
    GBC_CUDA(cudaMemcpy(R.d_w, R.slot_w.data(), sizeof(int32_t) * g->n, cudaMemcpyHostToDevice));
    GBC_TRY(relabel_weighted(*g, R.stream, &R.d_w, R.b_inv));
    g->w = R.d_w;
    g->ff = nullptr;
    R.dg = std::move(g);
    return GBC_OK;
}

// Internal ids of a degree-relabelled device graph in level-profile order
// (ties: lower id first) and the lane-group width for it, as the graph
// handles of the API choose them.
static gbc_status profile_order(const DevGraph& g, cudaStream_t s, std::vector<int32_t>& order, int32_t& group) {
    std::vector<uint32_t> key;
    int32_t depth = 0;
    GBC_TRY(level_profile_key(g, s, key, depth));
    order.resize(g.n);
    for (int32_t i = 0; i < g.n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });
    group = (depth > 0 && depth <= SMALL_WORLD_DEPTH) ? 128 : 32;
    return GBC_OK;
}

// The lane engine over the block graph for a call: lanes and group width
// from the options or the slot count and the memory budget, as graph handles
// choose them; an engine with betweenness state also serves closeness.
static gbc_status block_engine(Reduction& R, const gbc_options& o, bool bc, LaneEngine** out) {
    const int32_t ns = R.bg.n;
    if (R.b_order.empty()) GBC_TRY(profile_order(*R.dg, R.stream, R.b_order, R.b_group));
    // the block graph runs on lane groups (one lane per task is for whole deep graphs)
    int32_t group = o.group_lanes > 1 ? o.group_lanes : R.b_group;
    if (o.lanes % group) group = 32;
    int32_t lanes = o.lanes ? o.lanes : std::min<int32_t>(1024, ((ns + group - 1) / group) * group);
    const size_t fr = dev_free_bytes() + (R.eng ? R.eng->device_bytes() : 0);
    while (!o.lanes && lanes > group && LaneEngine::bytes_needed(ns, lanes, bc) > fr / 2) lanes -= group;
    if (!R.eng || R.eng->lanes() != lanes || R.eng->group_lanes() != group || (bc && !R.eng->has_bc())) {
        R.eng.reset();
        auto e = std::make_unique<LaneEngine>();
        GBC_TRY(e->init(R.dg.get(), lanes, bc, o.sparse_lanes, o.levels_per_graph, R.stream, group));
        R.eng = std::move(e);
    }
    R.eng->set_tuning(o.sparse_lanes, o.light_steps, o.levels_per_graph, o.block_threads, o.bu_share > 0 ? o.bu_share : -1);
    *out = R.eng.get();
    return GBC_OK;
}

// D_B(slot) for every slot, by the lane engine over the block graph.
static gbc_status weighted_sums(Reduction& R, const gbc_options& o, std::vector<int64_t>& D) {
    GBC_TRY(upload(R));
    const int32_t ns = R.bg.n;
    D.assign(ns, 0);
    if (ns == 0) return GBC_OK;
    LaneEngine* E = nullptr;
    GBC_TRY(block_engine(R, o, false, &E));
    const int32_t lanes = E->lanes();
    int32_t* d_src = nullptr;
    unsigned long long* d_cc = nullptr;
    if (cudaMalloc(&d_src, sizeof(int32_t) * ns) != cudaSuccess || cudaMalloc(&d_cc, sizeof(unsigned long long) * ns) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_src);
        set_error("slot buffers");
        return GBC_ERR_NOMEM;
    }
    std::unique_ptr<void, void (*)(void*)> f1(d_src, [](void* p) { cudaFree(p); });
    std::unique_ptr<void, void (*)(void*)> f2(d_cc, [](void* p) { cudaFree(p); });
    // lane i holds the i-th internal id in level-profile order; slot_of_id maps it back
    std::vector<int32_t> slot_of_id(ns);
    for (int32_t sl = 0; sl < ns; sl++) slot_of_id[R.b_inv[sl]] = sl;
    GBC_CUDA(cudaMemcpyAsync(d_src, R.b_order.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, R.stream));
    LaneResult res;
    for (int32_t b0 = 0; b0 < ns; b0 += lanes) {
        LaneRequest rq;
        rq.job = LaneJob::CC;
        rq.d_src = d_src + b0;
        rq.kb = std::min(lanes, ns - b0);
        rq.d_cc = d_cc + b0;
        rq.top_down_only = o.direction == 1;
        GBC_TRY(E->run(rq, res));
    }
    std::vector<int64_t> Dl(ns);
    GBC_CUDA(cudaMemcpyAsync(Dl.data(), d_cc, sizeof(int64_t) * ns, cudaMemcpyDeviceToHost, R.stream));
    GBC_CUDA(cudaStreamSynchronize(R.stream));
    for (int32_t i = 0; i < ns; i++) D[slot_of_id[R.b_order[i]]] = Dl[i];
    return GBC_OK;
}

// Host DP over the block-cut tree, then recovery of the folded vertices.
static gbc_status assemble_cc(Reduction& R, const std::vector<int64_t>& D, int64_t* cc) {
    const int32_t n = R.n, nb = R.n_blocks;
    auto slot_of = [&](int32_t b, int32_t v) -> int64_t {
        auto first = R.slot_v.begin() + R.bvoff[b], last = R.slot_v.begin() + R.bvoff[b + 1];
        return std::lower_bound(first, last, v) - R.slot_v.begin();
    };
    const int32_t nap = (int32_t)R.ap_child_blocks.size();
    std::vector<int64_t> base(nb, 0), xdown(nap, 0), sdown(nb, 0), xup(nb, 0), FF(nb, 0);
    for (int32_t b = 0; b < nb; b++)
        for (int64_t s = R.bvoff[b]; s < R.bvoff[b + 1]; s++) base[b] += R.ff[R.slot_v[s]];
    // down: S_B(p) = base(B) - ff[p] + sum_{child APs c of B} X_down(c) + D_B(p)
    for (int64_t h = (int64_t)R.border.size() - 1; h >= 0; h--) {
        const int32_t b = R.border[h];
        int64_t xs = 0;
        for (int64_t s = R.bvoff[b]; s < R.bvoff[b + 1]; s++) {
            const int32_t v = R.slot_v[s];
            if (R.is_ap[v] && v != R.bparent_ap[b]) xs += xdown[R.ap_index[v]];
        }
        const int32_t p = R.bparent_ap[b];
        if (p >= 0) {
            sdown[b] = base[b] - R.ff[p] + xs + D[slot_of(b, p)];
            xdown[R.ap_index[p]] += sdown[b];
        }
        FF[b] = base[b] + xs;   // completed with the up term below
    }
    // up: X_up(B) = S_P(p) + X_down(p) - S_B(p) with S_P(p) = FF_P - ff[p] - X_down(p) + D_P(p)
    for (size_t h = 0; h < R.border.size(); h++) {
        const int32_t b = R.border[h];
        const int32_t p = R.bparent_ap[b];
        if (p >= 0) {
            const int32_t P = R.ap_parent_block[p];
            const int64_t xd = xdown[R.ap_index[p]];
            const int64_t sP = FF[P] - R.ff[p] - xd + D[slot_of(P, p)];
            xup[b] = sP + xd - sdown[b];
            FF[b] += xup[b];
        }
    }
    for (int32_t v = 0; v < n; v++) cc[v] = 0;
    for (int32_t b = 0; b < nb; b++)
        for (int64_t s = R.bvoff[b]; s < R.bvoff[b + 1]; s++) {
            const int32_t v = R.slot_v[s];
            const int64_t val = FF[b] + D[s];
            if (R.vslot[v] == s) cc[v] = val;
            else if (cc[v] != val) {
                set_error("internal: closeness of articulation point %d differs between blocks (%lld vs %lld)", v,
                          (long long)cc[v], (long long)val);
                return GBC_ERR_LIMIT;
            }
        }
    // folded vertices, reverse folding order
    for (int64_t i = (int64_t)R.fold_order.size() - 1; i >= 0; i--) {
        const int32_t d1 = R.fold_order[i];
        const int64_t Nc = R.comp_w[R.comp[d1]];
        cc[d1] = cc[R.parent[d1]] + Nc - 2 * R.r[d1];
    }
    return GBC_OK;
}

// Betweenness through D1 folding.  Folding a degree-1 vertex u (reach r_u)
// into v (reach r_v before absorbing u) in a component of N vertices puts v
// on the shortest paths of exactly the 2 r_u (N - r_u - r_v) ordered pairs
// between u's vertices and the vertices not yet folded into v; summing over
// folding events covers every pair with an endpoint in a pendant tree once.
// Pairs of distinct core vertices s, t stand for r_s r_t original pairs, so
// the core contributes reach-weighted Brandes: delta_s(v) = sum over
// successors w of sigma_sv/sigma_sw (r_w + delta_s(w)), BC(v) += r_s delta_s(v).
static void fold_bc(const Reduction& R, std::vector<double>& bc) {
    bc.assign(R.n, 0.0);
    for (size_t i = 0; i < R.fold_order.size(); i++) {
        const int32_t d1 = R.fold_order[i];
        const int32_t p = R.parent[d1];
        const int64_t N = R.comp_w[R.comp[d1]];
        const int64_t ru = R.r[d1];
        bc[p] += 2.0 * (double)ru * (double)(N - ru - R.fold_rp[i]);
    }
}

// Betweenness through the block split.  A shortest path between vertices on
// different sides of an articulation point b passes through b, and its part
// inside a block B runs between the two vertices of B through which its ends
// reach B.  The clone weight w'_B(a) counts every vertex that reaches B
// through a (a's own reach for a vertex that is no articulation point), so
// reach-weighted Brandes inside every block, every slot a source,
//     BC_B(v) = sum over a != v != c in B of w'_B(a) w'_B(c) sigma^B_ac(v) / sigma^B_ac,
// counts every pair of unfolded vertices whose shortest paths cross B with v
// inside.  An articulation point v also lies on every path between two of the
// sides it separates.  With N the total reach of v's component, the side
// behind block B holds R_B = N - w'_B(v), and those sides hold N - r_v in all,
// so the separated ordered pairs add (N - r_v)^2 - sum_B R_B^2.  With the
// folded pendant trees' pair counts (fold_bc):
//     BC(v) = fold(v) + sum_{B holding v} BC_B(v) + [v is an AP] ((N - r_v)^2 - sum_B (N - w'_B(v))^2).
// The reference has no betweenness through these reductions; its AP clones
// (Lib/AP_Process/AP_Process.c:916-1020) carry the same reach w'.
static gbc_status block_bc(Reduction& R, const gbc_options& o, std::vector<double>& out) {
    GBC_TRY(upload(R));
    const int32_t ns = R.bg.n;
    out.assign(ns, 0.0);
    if (ns == 0) return GBC_OK;
    LaneEngine* E = nullptr;
    GBC_TRY(block_engine(R, o, true, &E));
    const int32_t lanes = E->lanes();
    int32_t* d_src = nullptr;
    double* d_bc = nullptr;
    if (cudaMalloc(&d_src, sizeof(int32_t) * ns) != cudaSuccess || cudaMalloc(&d_bc, sizeof(double) * ns) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_src);
        set_error("slot buffers");
        return GBC_ERR_NOMEM;
    }
    std::unique_ptr<void, void (*)(void*)> f1(d_src, [](void* p) { cudaFree(p); });
    std::unique_ptr<void, void (*)(void*)> f2(d_bc, [](void* p) { cudaFree(p); });
    // every slot once, in level-profile order (internal ids)
    GBC_CUDA(cudaMemcpyAsync(d_src, R.b_order.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, R.stream));
    GBC_TRY(E->bc_begin());
    LaneResult res;
    bool wide = o.sigma_mode == GBC_SIGMA_WIDE;   // AUTO: later batches start wide after an overflow
    for (int32_t b0 = 0; b0 < ns; b0 += lanes) {
        LaneRequest rq;
        rq.job = LaneJob::BC;
        rq.d_src = d_src + b0;
        rq.kb = std::min(lanes, ns - b0);
        rq.delta_f64 = o.delta_precision == GBC_DELTA_F64;
        rq.semantics = GBC_BC_BRANDES;
        rq.sigma_wide = wide;
        rq.abort_on_overflow = !rq.sigma_wide;
        gbc_status st = E->run(rq, res);
        if (st == GBC_ERR_OVERFLOW && o.sigma_mode == GBC_SIGMA_AUTO && !wide) {
            wide = true;
            rq.sigma_wide = 1;
            rq.abort_on_overflow = false;
            st = E->run(rq, res);
        }
        if (st != GBC_OK) return st;
    }
    GBC_TRY(E->bc_finish(d_bc));
    std::vector<double> h(ns);
    GBC_CUDA(cudaMemcpyAsync(h.data(), d_bc, sizeof(double) * ns, cudaMemcpyDeviceToHost, R.stream));
    GBC_CUDA(cudaStreamSynchronize(R.stream));
    for (int32_t sl = 0; sl < ns; sl++) out[sl] = h[R.b_inv[sl]];
    return GBC_OK;
}

// bc[n] from the per-slot block terms, the separated pairs of the
// articulation points and the folded pair counts.
static void assemble_block_bc(const Reduction& R, const std::vector<double>& slot_bc, double* bc) {
    std::vector<double> fb;
    fold_bc(R, fb);
    for (int32_t v = 0; v < R.n; v++) bc[v] = fb[v];
    std::vector<double> sq(R.ap_child_blocks.size(), 0.0);
    for (int64_t sl = 0; sl < (int64_t)R.slot_v.size(); sl++) {
        const int32_t v = R.slot_v[sl];
        bc[v] += slot_bc[sl];
        if (R.is_ap[v]) {
            const double side = (double)(R.comp_w[R.comp[v]] - R.slot_w[sl]);
            sq[R.ap_index[v]] += side * side;
        }
    }
    for (int32_t v = 0; v < R.n; v++) {
        if (!R.is_ap[v]) continue;
        const double others = (double)(R.comp_w[R.comp[v]] - R.r[v]);
        bc[v] += others * others - sq[R.ap_index[v]];
    }
}

}  // namespace gbc

using namespace gbc;

struct gbc_reduced_s {
    Reduction R;
};

// The reduction on the host: O(n + m) folding and a Hopcroft-Tarjan DFS, the
// reference's placement of this step.
static gbc_status reduce_on_host(const int64_t* row, const int32_t* col, Reduction& R) {
    const int32_t n = R.n, start = R.start;
    std::vector<int32_t> lc;
    std::vector<int64_t> lo;
    fold(row, col, R, lc, lo);
    std::vector<int32_t> cid(n, -1);
    for (int32_t v = start; v < n; v++)
        if (!R.folded[v]) { cid[v] = (int32_t)R.core_v.size(); R.core_v.push_back(v); }
    const int32_t nc = (int32_t)R.core_v.size();
    R.core.n = nc;
    R.core.row.assign(nc + 1, 0);
    R.core_w.resize(nc);
    for (int32_t i = 0; i < nc; i++) {
        const int32_t v = R.core_v[i];
        R.core.row[i + 1] = R.core.row[i] + (row[v + 1] - lo[v]);
        if (R.r[v] > INT32_MAX) { set_error("reach exceeds int32"); return GBC_ERR_ARG; }
        R.core_w[i] = (int32_t)R.r[v];
    }
    R.core.col.resize(R.core.row[nc]);
    for (int32_t i = 0; i < nc; i++) {
        const int32_t v = R.core_v[i];
        int64_t o = R.core.row[i];
        for (int64_t e = lo[v]; e < row[v + 1]; e++) R.core.col[o++] = cid[lc[e]];
    }
    return split(row, R, lc, lo);
}

// The reduction on the device (reduce_dev.cu); the host keeps the O(#folded)
// bookkeeping of the folding order and the O(#slots) block-cut tree.
static gbc_status device_ready(Reduction& R) {
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) { cudaGetLastError(); set_error("no CUDA device"); return GBC_ERR_NO_DEVICE; }
    if (!R.stream) GBC_CUDA(cudaStreamCreateWithFlags(&R.stream, cudaStreamNonBlocking));
    return GBC_OK;
}

static gbc_status reduce_device_csr(const int64_t* d_row, const int32_t* d_col, int64_t M, const int32_t* host_col,
                                    Reduction& R);

// Host CSR: upload, then the device reduction.
static gbc_status reduce_on_device(const int64_t* row, const int32_t* col, Reduction& R) {
    GBC_TRY(device_ready(R));
    const int32_t n = R.n;
    const int64_t M = row[n];
    int64_t* d_row = nullptr;
    int32_t* d_col = nullptr;
    if (cudaMalloc(&d_row, sizeof(int64_t) * ((size_t)n + 1)) != cudaSuccess ||
        cudaMalloc(&d_col, sizeof(int32_t) * std::max<int64_t>(M, 1)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_row);
        set_error("reduction: graph allocation");
        return GBC_ERR_NOMEM;
    }
    std::unique_ptr<void, void (*)(void*)> f1(d_row, [](void* p) { cudaFree(p); });
    std::unique_ptr<void, void (*)(void*)> f2(d_col, [](void* p) { cudaFree(p); });
    GBC_CUDA(cudaMemcpyAsync(d_row, row, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, R.stream));
    if (M) GBC_CUDA(cudaMemcpyAsync(d_col, col, sizeof(int32_t) * M, cudaMemcpyHostToDevice, R.stream));
    return reduce_device_csr(d_row, d_col, M, col, R);
}

// The reduction of a device CSR, its entries checked on the device first.
static gbc_status reduce_device_csr(const int64_t* d_row, const int32_t* d_col, int64_t M, const int32_t* host_col,
                                    Reduction& R) {
    const int32_t n = R.n;
    GBC_TRY(check_csr_device(d_row, d_col, n, M, host_col, R.stream));
    if (R.start == 1) {
        int64_t r1 = 0;
        GBC_CUDA(cudaMemcpy(&r1, d_row + 1, sizeof r1, cudaMemcpyDeviceToHost));
        if (r1 != 0) { set_error("phantom slot 0 must have no edges"); return GBC_ERR_ARG; }
    }
    FoldSplit F;
    GBC_TRY(fold_split_device(d_row, d_col, n, M, R.start, R.stream, F));
    R.d_core_row = F.d_core_row;
    R.d_core_col = F.d_core_col;
    R.core_m = F.core_m;
    R.d_bg_row = F.d_bg_row;
    R.d_bg_col = F.d_bg_col;
    R.bg_m = F.bg_m;
    // folding: order by round, then vertex id; parents' reach before each absorption
    R.r = std::move(F.r);
    R.ff = std::move(F.ff);
    R.parent = std::move(F.parent);
    R.folded.assign(n, 0);
    std::vector<int64_t> pos((size_t)F.rounds + 1, 0);
    for (int32_t v = 0; v < n; v++)
        if (F.fround[v] >= 0) { R.folded[v] = 1; pos[F.fround[v] + 1]++; }
    for (int32_t k = 0; k < F.rounds; k++) pos[k + 1] += pos[k];
    R.fold_order.resize(pos[F.rounds]);
    for (int32_t v = 0; v < n; v++)
        if (F.fround[v] >= 0) R.fold_order[pos[F.fround[v]]++] = v;
    std::vector<int64_t> rc(n, 1);
    std::vector<uint8_t> hub(n, 0);
    R.fold_rp.resize(R.fold_order.size());
    for (size_t i = 0; i < R.fold_order.size(); i++) {
        const int32_t d1 = R.fold_order[i], p = R.parent[d1];
        R.fold_rp[i] = rc[p];
        rc[p] += rc[d1];
        hub[p] = 1;
    }
    R.n_hub = 0;
    for (int32_t v = R.start; v < n; v++) R.n_hub += (hub[v] && !R.folded[v]);
    // the folded graph and its components
    R.core = std::move(F.core);
    R.core_v = std::move(F.core_v);
    const int32_t nc = R.core.n;
    R.core_w.resize(nc);
    R.comp.assign(n, -1);
    R.n_comp = F.n_comp;
    R.comp_w.assign(R.n_comp, 0);
    R.is_ap.assign(n, 0);
    R.vslot.assign(n, -1);
    for (int32_t i = 0; i < nc; i++) {
        const int32_t v = R.core_v[i];
        if (R.r[v] > INT32_MAX) { set_error("reach exceeds int32"); return GBC_ERR_ARG; }
        R.core_w[i] = (int32_t)R.r[v];
        R.comp[v] = F.core_comp[i];
        R.comp_w[F.core_comp[i]] += R.r[v];
        R.is_ap[v] = F.core_ap[i];
        R.vslot[v] = F.core_vslot[i];
    }
    // blocks
    R.n_blocks = (int32_t)F.bvoff.size() - 1;
    R.bvoff = std::move(F.bvoff);
    R.slot_v.resize(F.slot_core.size());
    for (size_t k = 0; k < F.slot_core.size(); k++) R.slot_v[k] = R.core_v[F.slot_core[k]];
    R.max_block = 0;
    for (int32_t b = 0; b < R.n_blocks; b++) R.max_block = std::max<int32_t>(R.max_block, (int32_t)(R.bvoff[b + 1] - R.bvoff[b]));
    R.bg = std::move(F.bg);
    R.fold_rounds = F.rounds;
    R.forest_levels = F.levels;
    return block_tree(R);
}

// Components of folded vertices follow their root.
static void folded_components(Reduction& R) {
    for (int64_t i = (int64_t)R.fold_order.size() - 1; i >= 0; i--) {
        const int32_t d1 = R.fold_order[i];
        R.comp[d1] = R.comp[R.parent[d1]];
    }
}

static gbc_status reduce_entry(const int64_t* row, const int32_t* col, int32_t n, int32_t start, gbc_reduced* out,
                               bool on_device) {
    if (!out) { set_error("out is NULL"); return GBC_ERR_ARG; }
    *out = nullptr;
    // the device path checks the entries on its device copy
    GBC_TRY(on_device ? validate_csr_header(row, col, n) : validate_csr(row, col, n));
    if (start < 0 || start > 1 || start >= n) { set_error("start must be 0 or 1"); return GBC_ERR_ARG; }
    if (!on_device) {
        if (start == 1 && row[1] != 0) { set_error("phantom slot 0 must have no edges"); return GBC_ERR_ARG; }
        for (int32_t v = 0; v < n; v++)
            for (int64_t e = row[v]; e < row[v + 1]; e++)
                if (col[e] == v) { set_error("self-loop at vertex %d", v); return GBC_ERR_ARG; }
    }
    auto H = std::make_unique<gbc_reduced_s>();
    Reduction& R = H->R;
    R.n = n;
    R.start = start;
    R.on_device = on_device;
    GBC_TRY(on_device ? reduce_on_device(row, col, R) : reduce_on_host(row, col, R));
    folded_components(R);
    *out = H.release();
    return GBC_OK;
}

extern "C" {

gbc_status gbc_reduce(const int64_t* row, const int32_t* col, int32_t n, int32_t start, gbc_reduced* out) {
    return reduce_entry(row, col, n, start, out, true);
}

gbc_status gbc_reduce_host(const int64_t* row, const int32_t* col, int32_t n, int32_t start, gbc_reduced* out) {
    return reduce_entry(row, col, n, start, out, false);
}

gbc_status gbc_reduce_device(const int64_t* d_row, const int32_t* d_col, int32_t n, int32_t start, gbc_reduced* out) {
    if (!out) { set_error("out is NULL"); return GBC_ERR_ARG; }
    *out = nullptr;
    if (n <= 0 || !d_row) { set_error("invalid CSR arguments (n=%d)", n); return GBC_ERR_ARG; }
    if (start < 0 || start > 1 || start >= n) { set_error("start must be 0 or 1"); return GBC_ERR_ARG; }
    auto H = std::make_unique<gbc_reduced_s>();
    Reduction& R = H->R;
    R.n = n;
    R.start = start;
    R.on_device = true;
    GBC_TRY(device_ready(R));
    // the header checks of the host path, on the two offsets they need
    int64_t ends[2] = {0, 0};
    GBC_CUDA(cudaMemcpy(&ends[0], d_row, sizeof(int64_t), cudaMemcpyDeviceToHost));
    GBC_CUDA(cudaMemcpy(&ends[1], d_row + n, sizeof(int64_t), cudaMemcpyDeviceToHost));
    if (ends[0] != 0) { set_error("row[0] must be 0"); return GBC_ERR_ARG; }
    if (ends[1] < 0 || ends[1] >= ((int64_t)1 << 31)) { set_error("row[n]=%lld out of range", (long long)ends[1]); return GBC_ERR_ARG; }
    if (ends[1] > 0 && !d_col) { set_error("invalid CSR arguments (n=%d)", n); return GBC_ERR_ARG; }
    GBC_TRY(reduce_device_csr(d_row, d_col, ends[1], nullptr, R));
    folded_components(R);
    *out = H.release();
    return GBC_OK;
}

gbc_status gbc_reduced_info_get(gbc_reduced h, gbc_reduced_info* info) {
    if (!h || !info) { set_error("NULL argument"); return GBC_ERR_ARG; }
    const Reduction& R = h->R;
    std::memset(info, 0, sizeof *info);
    info->n = R.n;
    info->d1_folded = (int32_t)R.fold_order.size();
    info->d1_hubs = R.n_hub;
    info->alive = (R.n - R.start) - info->d1_folded;
    int32_t ap = 0;
    for (uint8_t a : R.is_ap) ap += a;
    info->articulation_points = ap;
    info->blocks = R.n_blocks;
    info->max_block = R.max_block;
    info->block_slots = R.bg.n;
    info->block_edges = bg_entries(R);
    info->components = R.n_comp;
    info->on_device = R.on_device;
    info->fold_rounds = R.fold_rounds;
    info->forest_levels = R.forest_levels;
    return GBC_OK;
}

gbc_status gbc_cc_reduced(gbc_reduced h, const gbc_options* opt, int64_t* cc) {
    if (!h || !cc) { set_error("NULL argument"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(h->R.mu);
    gbc_options o;
    gbc_options_default(&o);
    if (opt) o = *opt;
    if (o.lanes != 0 && (o.lanes < 32 || o.lanes > 1024 || o.lanes % 32)) { set_error("bad lanes"); return GBC_ERR_ARG; }
    std::vector<int64_t> D;
    GBC_TRY(weighted_sums(h->R, o, D));
    return assemble_cc(h->R, D, cc);
}

gbc_status gbc_bc_reduced(gbc_reduced h, const gbc_options* opt, double* bc) {
    if (!h || !bc) { set_error("NULL argument"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(h->R.mu);
    gbc_options o;
    gbc_options_default(&o);
    if (opt) o = *opt;
    if (o.semantics != GBC_BC_BRANDES) {
        set_error("betweenness through the reduction supports GBC_BC_BRANDES only");
        return GBC_ERR_ARG;
    }
    if (o.lanes != 0 && (o.lanes < 32 || o.lanes > 1024 || o.lanes % 32)) { set_error("bad lanes"); return GBC_ERR_ARG; }
    std::vector<double> sb;
    GBC_TRY(block_bc(h->R, o, sb));
    assemble_block_bc(h->R, sb, bc);
    return GBC_OK;
}

gbc_status gbc_reduced_core_graph(gbc_reduced h, int64_t** row, int32_t** col, int32_t** weight, int32_t** vertex,
                                  int32_t* n_core) {
    if (!h || !row || !col || !weight || !vertex || !n_core) { set_error("NULL argument"); return GBC_ERR_ARG; }
    Reduction& R = h->R;
    std::lock_guard<std::mutex> lk(R.mu);
    GBC_TRY(host_rows(R.core, R.d_core_row, R.d_core_col, R.core_m));
    GBC_TRY(export_csr(R.core, row, col));
    const size_t nc = std::max<size_t>(R.core.n, 1);
    *weight = (int32_t*)malloc(sizeof(int32_t) * nc);
    *vertex = (int32_t*)malloc(sizeof(int32_t) * nc);
    if (!*weight || !*vertex) { free(*row); free(*col); free(*weight); free(*vertex); set_error("host allocation"); return GBC_ERR_NOMEM; }
    if (R.core.n) {
        std::memcpy(*weight, R.core_w.data(), sizeof(int32_t) * R.core.n);
        std::memcpy(*vertex, R.core_v.data(), sizeof(int32_t) * R.core.n);
    }
    *n_core = R.core.n;
    return GBC_OK;
}

gbc_status gbc_reduced_assemble_bc(gbc_reduced h, const double* core_bc, double* bc) {
    if (!h || (!core_bc && h->R.core.n) || !bc) { set_error("NULL argument"); return GBC_ERR_ARG; }
    std::vector<double> fb;
    fold_bc(h->R, fb);
    for (int32_t v = 0; v < h->R.n; v++) bc[v] = fb[v];
    for (size_t i = 0; i < h->R.core_v.size(); i++) bc[h->R.core_v[i]] += core_bc[i];
    return GBC_OK;
}

gbc_status gbc_reduced_block_graph(gbc_reduced h, int64_t** row, int32_t** col, int32_t** weight, int32_t* n_slots) {
    if (!h || !row || !col || !weight || !n_slots) { set_error("NULL argument"); return GBC_ERR_ARG; }
    Reduction& R = h->R;
    std::lock_guard<std::mutex> lk(R.mu);
    GBC_TRY(host_rows(R.bg, R.d_bg_row, R.d_bg_col, R.bg_m));
    GBC_TRY(export_csr(R.bg, row, col));
    *weight = (int32_t*)malloc(sizeof(int32_t) * std::max<int32_t>(R.bg.n, 1));
    if (!*weight) { free(*row); free(*col); set_error("host allocation"); return GBC_ERR_NOMEM; }
    if (R.bg.n) std::memcpy(*weight, R.slot_w.data(), sizeof(int32_t) * R.bg.n);
    *n_slots = R.bg.n;
    return GBC_OK;
}

gbc_status gbc_reduced_assemble_cc(gbc_reduced h, const int64_t* D, int64_t* cc) {
    if (!h || (!D && h->R.bg.n) || !cc) { set_error("NULL argument"); return GBC_ERR_ARG; }
    std::vector<int64_t> d(D, D + h->R.bg.n);
    return assemble_cc(h->R, d, cc);
}

gbc_status gbc_reduced_destroy(gbc_reduced h) {
    if (!h) { set_error("NULL handle"); return GBC_ERR_ARG; }
    delete h;
    return GBC_OK;
}

}  // extern "C"
