// Serving: continuous batching of centrality queries over device-resident
// graphs (the query loop the reference does not have; its drivers run one
// computation per process, Seq_CC/CC.cpp:2687, parallel_CC/para_CC.cu:383).
//
// A few worker threads run lane batches; each graph is worked on by at most
// one of them at a time, on the graph's own stream, so batches of different
// graphs overlap on the device and in the host gaps between level-loop
// launches.  Each registered graph keeps its CSR in HBM and, while it has
// work, one lane engine sized to its pending sources.  A lane batch is filled
// from every admitted request on one graph that wants the same kind of sweep
// (closeness or betweenness), oldest first, in lane groups of 128 lanes on
// small-world graphs, else 32, as graph handles choose them.  A request takes
// whole 32-lane parts: the level kernels keep betweenness partials per 32
// lanes for both group widths, so one 128-lane group can carry up to four
// requests, and each request's partials are added into its own FP64 result
// vector after each batch.  Its sources run in level-profile order.
// Requests that arrive while a batch runs join the next batch.
//
// Device memory is admitted against one budget: a request is admitted, in
// arrival order, only while the result vectors of the admitted (not yet
// fetched) requests, the engines of the graphs with admitted work (or the
// narrowest engine a graph could run with, while it has none) and its own
// share fit.  Later requests wait behind one that does not fit; one that
// could never fit fails.  Result vectors come from the library's device-buffer
// cache when the request's first batch runs, not at submission.  Engines are
// created under the same budget and idle ones are released when another
// graph needs room.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "engine.h"

using namespace gbc;

namespace {
constexpr int32_t PART = 32;   // lanes of one betweenness partial: a request's unit of a lane batch
}

namespace {

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct SGraph {
    DevGraph g;
    std::unique_ptr<LaneEngine> eng;
    int32_t lanes = 0;
    int32_t* d_src = nullptr;
    double** d_dst = nullptr;    // device table: lane group -> destination result vector
    cudaStream_t stream = nullptr;
    bool running = false;        // a worker holds this graph (its engine, buffers and stream)
    // the device CSR is relabelled by descending degree: inv[caller id] = internal id
    int32_t* d_order = nullptr;
    int32_t* d_inv = nullptr;
    std::vector<int32_t> h_inv;
    // level-profile key of every internal id: a request's sources are sorted by
    // it, so that each 32-lane group holds sources whose BFS levels move together
    std::vector<uint32_t> key;
    std::vector<int32_t> all_sorted;   // every caller id in that order (exact queries), isolated vertices last
    size_t n_with_edges = 0;           // leading entries of all_sorted that have edges
    // A source without edges (an isolated vertex) reaches nothing: it adds
    // nothing to betweenness and its closeness sum is 0, so it takes no lane.
    bool isolated(int32_t v) const { return g.comp_edges[g.comp[v]] == 0; }
    int32_t group = 32;          // lanes per lane group: 128 on small-world graphs, as on graph handles
    // device bytes of the narrowest lane engine this graph runs with
    int32_t unit() const { return group == 1 ? 32 : group; }   // lanes an engine grows by
    size_t engine_floor() const { return LaneEngine::bytes_needed(g.n, unit(), true, group); }
    ~SGraph() {
        eng.reset();
        cudaFree(g.row);
        cudaFree(g.col);
        cudaFree(d_src);
        cudaFree(d_dst);
        cudaFree(d_order);
        cudaFree(d_inv);
        if (stream) cudaStreamDestroy(stream);
    }
};

struct Req {
    int64_t id = 0;
    int32_t gid = 0;
    int32_t kind = GBC_Q_CC;
    gbc_options opt{};
    std::vector<int32_t> src;    // the sources, those with edges first (in run order), then any without
    size_t nlane = 0;            // sources with edges: only these take lanes
    size_t next = 0;             // next source to hand out
    size_t done = 0;             // sources whose lanes finished
    int32_t state = GBC_REQ_QUEUED;
    gbc_status err = GBC_OK;
    std::string msg;
    double t_submit = 0, t_done = 0, deadline = 0;
    double* d_bc = nullptr;      // device FP64 result (BC kinds), from the buffer cache at the first batch
    size_t res_bytes = 0;        // device bytes of that result (admission charges them until fetched)
    std::vector<int64_t> cc;     // host result (CC), indexed by vertex
    bool admitted = false;
    int32_t inflight = 0;        // lane batches holding this request's sources or result buffer
    ~Req() { dev_release(d_bc, res_bytes); }
    bool bc() const { return kind != GBC_Q_CC; }
};

}  // namespace

struct gbc_server_s {
    gbc_server_config cfg{};
    size_t budget = 0;
    int32_t max_lanes = 1024;
    int32_t max_inflight = 64;
    int32_t nworkers = 8;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<std::unique_ptr<SGraph>> graphs;
    std::map<int64_t, std::unique_ptr<Req>> reqs;
    std::deque<int64_t> fifo;    // admitted or queued requests in arrival order
    int64_t next_id = 1;
    bool stop = false;
    std::vector<std::thread> workers;
    int32_t rr = 0;              // round-robin position over graphs
    // counters; busy_ms is the time during which at least one batch ran
    int64_t completed = 0, batches = 0, shared_batches = 0, edges = 0;
    double busy_ms = 0, busy_t0 = 0;
    int32_t active = 0;

    void run();
    size_t engines_bytes() const {
        size_t b = 0;
        for (auto& g : graphs) if (g->eng) b += g->eng->device_bytes();
        return b;
    }
    // result bytes of admitted requests not yet fetched
    size_t results_bytes() const {
        size_t b = 0;
        for (auto& kv : reqs) if (kv.second->admitted) b += kv.second->res_bytes;
        return b;
    }
    void admit();
    void fail(Req& r, gbc_status st, const char* why) {
        r.state = GBC_REQ_FAILED;
        r.err = st;
        r.msg = why;
        r.t_done = now_ms();
    }
};

namespace {

// Engine for graph gi, as wide as its pending sources need (up to max_lanes)
// and the budget allows, counting the result vectors of admitted requests.
// Idle engines (graphs that neither have admitted work nor are held by a
// worker) are released to make room.  A graph's engine is replaced only by a
// wider one that fits; its buffers go to the cache.
gbc_status ensure_engine(gbc_server_s* S, int32_t gi, const std::vector<bool>& graph_busy, int64_t pending) {
    SGraph& G = *S->graphs[gi];
    const int32_t gr = G.unit();
    const int32_t cap = S->max_lanes / gr * gr;
    const int32_t want = (int32_t)std::min<int64_t>(cap, std::max<int64_t>(gr, (pending + gr - 1) / gr * gr));
    if (G.eng && (G.eng->lanes() >= want || G.eng->lanes() >= cap)) return GBC_OK;
    // bytes that stay held: results plus the engines of other graphs that are not idle
    size_t held = S->results_bytes();
    for (size_t j = 0; j < S->graphs.size(); j++)
        if ((int32_t)j != gi && S->graphs[j]->eng && graph_busy[j]) held += S->graphs[j]->eng->device_bytes();
    int32_t lanes = want;
    while (lanes > gr && held + LaneEngine::bytes_needed(G.g.n, lanes, true, G.group) > S->budget)
        lanes = std::max(gr, lanes / 2 / gr * gr);
    if (held + LaneEngine::bytes_needed(G.g.n, lanes, true, G.group) > S->budget) {
        if (G.eng) return GBC_OK;   // keep the engine it has
        set_error("graph does not fit the HBM budget");
        return GBC_ERR_BUSY;
    }
    if (G.eng && G.eng->lanes() >= lanes) return GBC_OK;   // nothing wider fits
    G.eng.reset();
    size_t used = S->engines_bytes() + S->results_bytes();
    const size_t need = LaneEngine::bytes_needed(G.g.n, lanes, true, G.group);
    for (size_t j = 0; j < S->graphs.size() && used + need > S->budget; j++) {
        if ((int32_t)j == gi || !S->graphs[j]->eng || graph_busy[j]) continue;
        used -= S->graphs[j]->eng->device_bytes();
        S->graphs[j]->eng.reset();
    }
    auto e = std::make_unique<LaneEngine>();
    GBC_TRY(e->init(&G.g, lanes, true, -1, 0, G.stream, G.group));
    if (G.lanes != lanes) {
        cudaFree(G.d_src);
        cudaFree(G.d_dst);
        G.d_src = nullptr;
        G.d_dst = nullptr;
        if (cudaMalloc(&G.d_src, sizeof(int32_t) * lanes) != cudaSuccess ||
            cudaMalloc(&G.d_dst, sizeof(double*) * (lanes / 32)) != cudaSuccess) {
            cudaGetLastError();
            set_error("server batch buffers");
            return GBC_ERR_NOMEM;
        }
        G.lanes = lanes;
    }
    G.eng = std::move(e);
    return GBC_OK;
}

}  // namespace

// Admit queued requests in arrival order while their device bytes fit the
// budget (and fewer than max_inflight hold sources).  Charged: the result
// vectors of every admitted request not yet fetched, and per graph with
// admitted work its engine, or the narrowest engine it could run with.
// Called with mu held.
void gbc_server_s::admit() {
    int32_t inflight = 0;
    for (int64_t id : fifo) inflight += reqs[id]->admitted;
    std::vector<char> charged(graphs.size(), 0);
    size_t reserved = results_bytes();
    auto engine_bytes = [&](int32_t gi) {
        const SGraph& G = *graphs[gi];
        return G.eng ? std::max(G.eng->device_bytes(), G.engine_floor()) : G.engine_floor();
    };
    for (int64_t id : fifo) {
        Req* r = reqs[id].get();
        if (r->admitted && !charged[r->gid]) {
            charged[r->gid] = 1;
            reserved += engine_bytes(r->gid);
        }
    }
    for (int64_t id : fifo) {
        Req* r = reqs[id].get();
        if (r->admitted || r->state != GBC_REQ_QUEUED) continue;
        if (inflight >= max_inflight) break;
        const size_t own = r->res_bytes + graphs[r->gid]->engine_floor();
        if (own > budget) {
            fail(*r, GBC_ERR_NOMEM, "the request's result and its graph's narrowest engine exceed the server's HBM budget");
            cv_done.notify_all();
            continue;
        }
        const size_t need = r->res_bytes + (charged[r->gid] ? 0 : engine_bytes(r->gid));
        if (reserved + need > budget) break;   // first come, first served: later requests wait behind it
        r->admitted = true;
        r->state = GBC_REQ_RUNNING;
        inflight++;
        reserved += need;
        charged[r->gid] = 1;
    }
}

void gbc_server_s::run() {
    std::vector<int32_t> hsrc;
    std::vector<double*> hdst;
    std::vector<unsigned long long> hcc;
    struct Slot { Req* r; size_t first; int32_t count; int32_t lane0; };
    for (;;) {
        std::vector<Slot> slots;
        int32_t gi = -1, kind = 0, lanes = 0;
        SGraph* Gp = nullptr;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                if (stop) return;
                // expire deadlines, drop finished ids from the fifo
                const double t = now_ms();
                for (auto it = fifo.begin(); it != fifo.end();) {
                    Req* r = reqs.count(*it) ? reqs[*it].get() : nullptr;
                    if (!r || r->state == GBC_REQ_DONE || r->state == GBC_REQ_FAILED || r->state == GBC_REQ_CANCELLED) {
                        it = fifo.erase(it);
                        continue;
                    }
                    if (r->deadline > 0 && t > r->deadline && r->done < r->nlane) {
                        fail(*r, GBC_ERR_TIMEOUT, "deadline passed");
                        cv_done.notify_all();
                        it = fifo.erase(it);
                        continue;
                    }
                    ++it;
                }
                admit();
                // pick a graph with pending sources that no other worker holds, round robin
                std::vector<bool> busy(graphs.size(), false);
                for (int64_t id : fifo) {
                    Req* r = reqs[id].get();
                    if (r->admitted && r->next < r->nlane) busy[r->gid] = true;
                }
                for (size_t k = 0; k < graphs.size(); k++) {
                    const int32_t cand = (int32_t)((rr + k) % graphs.size());
                    if (busy[cand] && !graphs[cand]->running) { gi = cand; break; }
                }
                if (gi < 0) { cv_work.wait_for(lk, std::chrono::milliseconds(50)); continue; }
                rr = gi + 1;
                for (size_t j = 0; j < graphs.size(); j++) busy[j] = busy[j] || graphs[j]->running;
                int64_t pending = 0;
                for (int64_t id : fifo) {
                    Req* r = reqs[id].get();
                    if (r->gid == gi && r->admitted) pending += (int64_t)(r->nlane - r->next);
                }
                gbc_status st = ensure_engine(this, gi, busy, pending);
                if (st != GBC_OK) {
                    for (int64_t id : fifo) {
                        Req* r = reqs[id].get();
                        if (r->gid == gi && r->admitted) fail(*r, st, last_error());
                    }
                    cv_done.notify_all();
                    gi = -1;
                    continue;
                }
                lanes = graphs[gi]->lanes;
                // fill the batch: oldest request's kind, whole 32-lane parts per request
                kind = -1;
                int32_t used = 0;
                for (int64_t id : fifo) {
                    Req* r = reqs[id].get();
                    if (r->gid != gi || !r->admitted || r->next >= r->nlane) continue;
                    // requests share a batch only when they need the same sweep
                    const int32_t rk = r->bc() ? 1 + r->opt.semantics * 2 + (r->opt.delta_precision == GBC_DELTA_F64) : 0;
                    if (kind < 0) kind = rk;
                    if (rk != kind) continue;
                    const int32_t room = lanes - used;
                    if (room < PART) break;
                    const int32_t take = (int32_t)std::min<size_t>(room, r->nlane - r->next);
                    slots.push_back({r, r->next, take, used});
                    r->next += take;
                    r->inflight++;
                    used += ((take + PART - 1) / PART) * PART;
                }
                Gp = graphs[gi].get();
                Gp->running = true;
                if (active++ == 0) busy_t0 = now_ms();
                break;
            }
        }
        // device work outside the lock
        SGraph& G = *Gp;
        cudaStream_t stream = G.stream;
        const int32_t grp = G.group;
        const int32_t np = lanes / PART;
        hsrc.assign(lanes, -1);
        hdst.assign(np, nullptr);
        int32_t kb = 0;
        const bool bc_batch = kind > 0;
        gbc_status st = GBC_OK;
        // result vectors of requests in their first batch: from the buffer cache, zeroed on this stream
        for (auto& sl : slots) {
            Req* r = sl.r;
            if (!bc_batch || r->d_bc || st != GBC_OK) continue;
            double* p = nullptr;
            if (dev_alloc((void**)&p, r->res_bytes) != cudaSuccess) {
                cudaGetLastError();
                set_error("result vector of %zu bytes", r->res_bytes);
                st = GBC_ERR_NOMEM;
            } else if (cudaMemsetAsync(p, 0, r->res_bytes, stream) != cudaSuccess) {
                cudaGetLastError();
                dev_release(p, r->res_bytes);
                set_error("result vector reset failed");
                st = GBC_ERR_CUDA;
            } else {
                r->d_bc = p;   // only the worker holding this graph touches it until the request is fetched
            }
        }
        for (auto& sl : slots) {
            for (int32_t i = 0; i < sl.count; i++) hsrc[sl.lane0 + i] = G.h_inv[sl.r->src[sl.first + i]];
            for (int32_t p = sl.lane0 / PART; p < (sl.lane0 + sl.count + PART - 1) / PART; p++) hdst[p] = sl.r->d_bc;
            kb = std::max(kb, ((sl.lane0 + sl.count + grp - 1) / grp) * grp);
        }
        if (st == GBC_OK &&
            cudaMemcpyAsync(G.d_src, hsrc.data(), sizeof(int32_t) * kb, cudaMemcpyHostToDevice, stream) != cudaSuccess) {
            cudaGetLastError();
            st = GBC_ERR_CUDA;
            set_error("source upload failed");
        }
        LaneResult res;
        if (st == GBC_OK && bc_batch) {
            if (cudaMemcpyAsync(G.d_dst, hdst.data(), sizeof(double*) * np, cudaMemcpyHostToDevice, stream) != cudaSuccess) {
                cudaGetLastError();
                st = GBC_ERR_CUDA;
            }
            if (st == GBC_OK) st = G.eng->bc_begin();
            LaneRequest rq;
            rq.job = LaneJob::BC;
            rq.d_src = G.d_src;
            rq.kb = kb;
            rq.delta_f64 = slots[0].r->opt.delta_precision == GBC_DELTA_F64;
            rq.semantics = slots[0].r->opt.semantics;
            rq.abort_on_overflow = true;
            if (st == GBC_OK) st = G.eng->run(rq, res);
            if (st == GBC_ERR_OVERFLOW) {
                rq.sigma_wide = 1;
                rq.abort_on_overflow = false;
                st = G.eng->run(rq, res);
            }
            if (st == GBC_OK) st = G.eng->bc_scatter(G.d_dst);
            if (st == GBC_OK && cudaStreamSynchronize(stream) != cudaSuccess) { cudaGetLastError(); st = GBC_ERR_CUDA; }
        } else if (st == GBC_OK) {
            LaneRequest rq;
            rq.job = LaneJob::CC;
            rq.d_src = G.d_src;
            rq.kb = kb;
            st = G.eng->run(rq, res);
            hcc.assign(kb, 0);
            if (st == GBC_OK) st = G.eng->cc_read(hcc.data(), kb);
        }
        // a failed batch may leave copies or kernels queued: let them finish before
        // its requests' buffers can go back to the cache
        if (st != GBC_OK && cudaStreamSynchronize(stream) != cudaSuccess) cudaGetLastError();
        {
            std::lock_guard<std::mutex> lk(mu);
            G.running = false;
            if (--active == 0) busy_ms += now_ms() - busy_t0;
            batches++;
            if (slots.size() > 1) shared_batches++;
            for (auto& sl : slots) {
                Req* r = sl.r;
                r->inflight--;
                if (r->state != GBC_REQ_RUNNING) continue;   // cancelled or expired meanwhile
                if (st != GBC_OK) { fail(*r, st, last_error()); continue; }
                for (int32_t i = 0; i < sl.count; i++) {
                    const int32_t v = r->src[sl.first + i];
                    edges += G.g.comp_edges.empty() ? 0 : G.g.comp_edges[G.g.comp[v]];
                    if (!bc_batch) r->cc[v] = (int64_t)hcc[sl.lane0 + i];
                }
                r->done += sl.count;
                if (r->done == r->nlane) {
                    r->state = GBC_REQ_DONE;
                    r->t_done = now_ms();
                    completed++;
                }
            }
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

extern "C" {

gbc_status gbc_server_create(const gbc_server_config* cfg, gbc_server* out) {
    if (!out) { set_error("out is NULL"); return GBC_ERR_ARG; }
    *out = nullptr;
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) { cudaGetLastError(); set_error("no CUDA device"); return GBC_ERR_NO_DEVICE; }
    auto S = std::make_unique<gbc_server_s>();
    if (cfg) S->cfg = *cfg;
    if (S->cfg.max_lanes != 0 && (S->cfg.max_lanes < 32 || S->cfg.max_lanes > 1024 || S->cfg.max_lanes % 32)) {
        set_error("max_lanes must be 0 or a multiple of 32 in [32,1024]");
        return GBC_ERR_ARG;
    }
    S->max_lanes = S->cfg.max_lanes ? S->cfg.max_lanes : 1024;
    S->max_inflight = S->cfg.max_inflight > 0 ? S->cfg.max_inflight : 64;
    if (S->cfg.workers < 0 || S->cfg.workers > 16) { set_error("workers must be in [0,16]"); return GBC_ERR_ARG; }
    // 8 by default: with 4, small queries of a mixed stream waited behind large batches (40 q/s on
    // the serving mix: p50 / p99 148 / 1754 ms with 4 workers, 61 / 976 ms with 8, the same with 16)
    S->nworkers = S->cfg.workers ? S->cfg.workers : 8;
    S->budget = S->cfg.hbm_budget_bytes ? S->cfg.hbm_budget_bytes : dev_free_bytes() / 2;
    gbc_server_s* raw = S.get();
    int dev = 0;
    GBC_CUDA(cudaGetDevice(&dev));   // the workers run on the creating thread's device
    for (int32_t w = 0; w < S->nworkers; w++)
        S->workers.emplace_back([raw, dev] {
            cudaSetDevice(dev);
            raw->run();
        });
    *out = S.release();
    return GBC_OK;
}

gbc_status gbc_server_destroy(gbc_server s) {
    if (!s) { set_error("NULL server"); return GBC_ERR_ARG; }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& w : s->workers)
        if (w.joinable()) w.join();
    s->reqs.clear();
    s->graphs.clear();
    delete s;
    return GBC_OK;
}

gbc_status gbc_server_add_graph(gbc_server s, const int64_t* row, const int32_t* col, int32_t n, int32_t* gid) {
    if (!s || !gid) { set_error("NULL argument"); return GBC_ERR_ARG; }
    GBC_TRY(validate_csr(row, col, n));
    auto G = std::make_unique<SGraph>();
    G->g.n = n;
    G->g.m = row[n];
    GBC_CUDA(cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking));
    if (cudaMalloc(&G->g.row, sizeof(int64_t) * (n + 1)) != cudaSuccess ||
        cudaMalloc(&G->g.col, sizeof(int32_t) * std::max<int64_t>(row[n], 1)) != cudaSuccess) {
        cudaGetLastError();
        set_error("graph allocation");
        return GBC_ERR_NOMEM;
    }
    GBC_CUDA(cudaMemcpy(G->g.row, row, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    if (row[n]) GBC_CUDA(cudaMemcpy(G->g.col, col, sizeof(int32_t) * row[n], cudaMemcpyHostToDevice));
    GBC_TRY(relabel_graph(G->g, G->stream, &G->d_order, &G->d_inv));
    G->h_inv.resize(n);
    GBC_CUDA(cudaMemcpy(G->h_inv.data(), G->d_inv, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    int32_t depth = 0;
    GBC_TRY(level_profile_key(G->g, G->stream, G->key, depth));
    // 128-lane groups on small-world graphs; one lane per task on deep graphs of low degree, whose
    // sampled sources rarely share a level (as graph handles choose them); 32-lane groups otherwise
    int64_t maxdeg = 0;
    for (int32_t v = 0; v < n; v++) maxdeg = std::max<int64_t>(maxdeg, row[v + 1] - row[v]);
    if (depth > 0 && depth <= SMALL_WORLD_DEPTH && s->max_lanes % 128 == 0) G->group = 128;
    else if (depth > SMALL_WORLD_DEPTH && maxdeg <= ONE_LANE_MAX_DEGREE && n < ONE_LANE_MAX_N) G->group = 1;
    else G->group = 32;
    HostCSR h;
    h.n = n;
    h.row.assign(row, row + n + 1);
    h.col.assign(col, col + row[n]);
    std::vector<int64_t> sizes;
    const int32_t nc = components(h, G->g.comp, sizes);
    G->g.comp_edges.assign(nc, 0);
    for (int32_t v = 0; v < n; v++) G->g.comp_edges[G->g.comp[v]] += row[v + 1] - row[v];
    for (auto& e : G->g.comp_edges) e /= 2;
    G->all_sorted.resize(n);
    for (int32_t i = 0; i < n; i++) G->all_sorted[i] = i;
    {
        const SGraph* SG = G.get();
        std::stable_sort(G->all_sorted.begin(), G->all_sorted.end(), [SG](int32_t a, int32_t b) {
            const bool ia = SG->isolated(a), ib = SG->isolated(b);
            return ia != ib ? ib : SG->key[SG->h_inv[a]] < SG->key[SG->h_inv[b]];
        });
        G->n_with_edges = 0;
        while (G->n_with_edges < (size_t)n && !SG->isolated(G->all_sorted[G->n_with_edges])) G->n_with_edges++;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    *gid = (int32_t)s->graphs.size();
    s->graphs.push_back(std::move(G));
    return GBC_OK;
}

gbc_status gbc_server_submit(gbc_server s, int32_t gid, int32_t kind, int32_t k, uint64_t seed, const gbc_options* opt,
                             double deadline_ms, int64_t* req_id) {
    if (!s || !req_id) { set_error("NULL argument"); return GBC_ERR_ARG; }
    if (kind < GBC_Q_CC || kind > GBC_Q_BC_SAMPLED) { set_error("bad query kind"); return GBC_ERR_ARG; }
    auto r = std::make_unique<Req>();
    int32_t n = 0;
    const SGraph* SG = nullptr;   // graphs are never removed while the server lives
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (gid < 0 || gid >= (int32_t)s->graphs.size()) { set_error("unknown graph %d", gid); return GBC_ERR_NOT_FOUND; }
        SG = s->graphs[gid].get();
        n = SG->g.n;
    }
    gbc_options_default(&r->opt);
    if (opt) r->opt = *opt;
    if (r->opt.semantics != GBC_BC_BRANDES && r->opt.semantics != GBC_BC_REFERENCE) { set_error("bad semantics"); return GBC_ERR_ARG; }
    r->gid = gid;
    r->kind = kind;
    // sources in level-profile order (results are per vertex, so the order is free)
    if (kind == GBC_Q_BC_SAMPLED) {
        if (k < 1) { set_error("sampled BC needs k >= 1"); return GBC_ERR_ARG; }
        Rng rng(seed, 17);
        r->src.resize(k);
        for (int32_t i = 0; i < k; i++) r->src[i] = (int32_t)rng.below((uint64_t)n);
        std::stable_sort(r->src.begin(), r->src.end(), [&](int32_t a, int32_t b) {
            const bool ia = SG->isolated(a), ib = SG->isolated(b);
            return ia != ib ? ib : SG->key[SG->h_inv[a]] < SG->key[SG->h_inv[b]];
        });
        while (r->nlane < r->src.size() && !SG->isolated(r->src[r->nlane])) r->nlane++;
    } else {
        r->src = SG->all_sorted;
        r->nlane = SG->n_with_edges;
    }
    if (r->bc()) r->res_bytes = sizeof(double) * (size_t)n;
    else r->cc.assign(n, 0);
    r->t_submit = now_ms();
    r->deadline = deadline_ms > 0 ? r->t_submit + deadline_ms : 0;
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    *req_id = r->id;
    if (r->nlane == 0) {   // nothing to run: a zero result, done at once
        r->state = GBC_REQ_DONE;
        r->t_done = r->t_submit;
        s->completed++;
        s->reqs[r->id] = std::move(r);
        s->cv_done.notify_all();
        return GBC_OK;
    }
    s->fifo.push_back(r->id);
    s->reqs[r->id] = std::move(r);
    s->cv_work.notify_all();
    return GBC_OK;
}

gbc_status gbc_server_request_bytes(gbc_server s, int32_t gid, int32_t kind, size_t* result_bytes, size_t* engine_bytes) {
    if (!s) { set_error("NULL server"); return GBC_ERR_ARG; }
    if (kind < GBC_Q_CC || kind > GBC_Q_BC_SAMPLED) { set_error("bad query kind"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(s->mu);
    if (gid < 0 || gid >= (int32_t)s->graphs.size()) { set_error("unknown graph %d", gid); return GBC_ERR_NOT_FOUND; }
    const SGraph& G = *s->graphs[gid];
    if (result_bytes) *result_bytes = kind == GBC_Q_CC ? 0 : sizeof(double) * (size_t)G.g.n;
    if (engine_bytes) *engine_bytes = G.engine_floor();
    return GBC_OK;
}

gbc_status gbc_server_poll(gbc_server s, int64_t id, int32_t* state) {
    if (!s || !state) { set_error("NULL argument"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return GBC_ERR_NOT_FOUND; }
    *state = it->second->state;
    return GBC_OK;
}

gbc_status gbc_server_wait(gbc_server s, int64_t id, double timeout_ms, int32_t* state) {
    if (!s) { set_error("NULL server"); return GBC_ERR_ARG; }
    std::unique_lock<std::mutex> lk(s->mu);
    const double t_end = timeout_ms > 0 ? now_ms() + timeout_ms : 0;
    for (;;) {
        auto it = s->reqs.find(id);
        if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return GBC_ERR_NOT_FOUND; }
        const int32_t st = it->second->state;
        if (st == GBC_REQ_DONE || st == GBC_REQ_FAILED || st == GBC_REQ_CANCELLED) {
            if (state) *state = st;
            return GBC_OK;
        }
        if (t_end > 0 && now_ms() >= t_end) {
            if (state) *state = st;
            set_error("wait timed out");
            return GBC_ERR_TIMEOUT;
        }
        s->cv_done.wait_for(lk, std::chrono::milliseconds(20));
    }
}

gbc_status gbc_server_fetch(gbc_server s, int64_t id, double* bc, int64_t* cc, double* latency_ms) {
    if (!s) { set_error("NULL server"); return GBC_ERR_ARG; }
    std::unique_ptr<Req> r;
    int32_t n = 0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(id);
        if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return GBC_ERR_NOT_FOUND; }
        const int32_t st = it->second->state;
        if (it->second->inflight > 0 || st == GBC_REQ_QUEUED || st == GBC_REQ_RUNNING) {
            set_error("request not finished");
            return GBC_ERR_BUSY;
        }
        if (st == GBC_REQ_FAILED || st == GBC_REQ_CANCELLED) {
            const gbc_status e = st == GBC_REQ_FAILED ? it->second->err : GBC_ERR_ARG;
            set_error("request %s: %s", st == GBC_REQ_FAILED ? "failed" : "was cancelled", it->second->msg.c_str());
            s->reqs.erase(it);
            return e;
        }
        r = std::move(it->second);
        s->reqs.erase(it);
        n = s->graphs[r->gid]->g.n;
    }
    if (latency_ms) *latency_ms = r->t_done - r->t_submit;
    if (r->bc() && bc && !r->d_bc) {   // no source with edges: every value is 0
        std::memset(bc, 0, sizeof(double) * (size_t)n);
    } else if (r->bc() && bc) {
        // the result accumulated in internal ids: gather to the caller's, through a scratch vector
        double* tmp = nullptr;
        const size_t bytes = sizeof(double) * (size_t)n;
        if (dev_alloc((void**)&tmp, bytes) != cudaSuccess) { cudaGetLastError(); set_error("fetch buffer"); return GBC_ERR_NOMEM; }
        struct Tmp { double* p; size_t b; ~Tmp() { dev_release(p, b); } } ft{tmp, bytes};   // after the synchronous copy below
        const int32_t* d_inv = nullptr;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            d_inv = s->graphs[r->gid]->d_inv;
        }
        GBC_TRY(gather_to_caller<double>(r->d_bc, d_inv, n, 1, tmp, 0));
        GBC_CUDA(cudaMemcpy(bc, tmp, sizeof(double) * n, cudaMemcpyDeviceToHost));
    }
    if (!r->bc() && cc) std::memcpy(cc, r->cc.data(), sizeof(int64_t) * n);
    return GBC_OK;
}

gbc_status gbc_server_sources(gbc_server s, int64_t id, int32_t* out, int32_t cap, int32_t* k) {
    if (!s || !k) { set_error("NULL argument"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return GBC_ERR_NOT_FOUND; }
    const std::vector<int32_t>& src = it->second->src;
    *k = (int32_t)src.size();
    if (out) {
        if (cap < (int32_t)src.size()) { set_error("capacity %d < %zu sources", cap, src.size()); return GBC_ERR_ARG; }
        std::memcpy(out, src.data(), sizeof(int32_t) * src.size());
    }
    return GBC_OK;
}

gbc_status gbc_server_cancel(gbc_server s, int64_t id) {
    if (!s) { set_error("NULL server"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) { set_error("unknown request %lld", (long long)id); return GBC_ERR_NOT_FOUND; }
    Req* r = it->second.get();
    if (r->state == GBC_REQ_QUEUED || r->state == GBC_REQ_RUNNING) {
        r->state = GBC_REQ_CANCELLED;
        r->t_done = now_ms();
    }
    s->cv_done.notify_all();
    return GBC_OK;
}

gbc_status gbc_server_counters(gbc_server s, int64_t* completed, int64_t* batches, int64_t* shared, int64_t* edges,
                               double* busy_ms) {
    if (!s) { set_error("NULL server"); return GBC_ERR_ARG; }
    std::lock_guard<std::mutex> lk(s->mu);
    if (completed) *completed = s->completed;
    if (batches) *batches = s->batches;
    if (shared) *shared = s->shared_batches;
    if (edges) *edges = s->edges;
    if (busy_ms) *busy_ms = s->busy_ms + (s->active ? now_ms() - s->busy_t0 : 0.0);
    return GBC_OK;
}

}  // extern "C"
