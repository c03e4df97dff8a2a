// Engines behind the C ABI: the batched multi-source lane engine and the
// plain one-source-at-a-time engine.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "gbc_internal.h"

namespace gbc {

#define GBC_CUDA(call)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            gbc::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return GBC_ERR_CUDA;                                                               \
        }                                                                                      \
    } while (0)

#define GBC_TRY(expr)                         \
    do {                                      \
        gbc_status s_ = (expr);               \
        if (s_ != GBC_OK) return s_;          \
    } while (0)

// Device-buffer cache for lane state (devmem.cpp): dev_alloc takes a cached
// block of the same size (or at most 25% larger) or calls cudaMalloc;
// dev_release returns a block whose work has finished to the cache.
cudaError_t dev_alloc(void** p, size_t bytes);
void dev_release(void* p, size_t bytes);
size_t dev_cached_bytes();
// cudaMemGetInfo's free bytes plus the cached ones.
size_t dev_free_bytes();

// Edge list on the device -> symmetric, deduplicated CSR without self-loops,
// rows in ascending neighbour order (ingest.cu).  *d_row / *d_col are
// cudaMalloc'd; *M = directed entries.
gbc_status csr_from_edges_device(const int32_t* d_u, const int32_t* d_v, int64_t m, int32_t n, cudaStream_t s,
                                 int64_t** d_row, int32_t** d_col, int64_t* M);

// Connected-component label of every vertex of a device CSR (the smallest
// vertex id of its component), by union-find on the device (reduce_dev.cu).
gbc_status component_labels(const int64_t* d_row, const int32_t* d_col, int32_t n, cudaStream_t s, int32_t* d_lab);

struct DevGraph;
// Reassign vertex ids by descending degree and rewrite the rows (relabel.cu).
// g.row / g.col are replaced; *d_order[new] = old, *d_inv[old] = new.
gbc_status relabel_by_degree(DevGraph& g, cudaStream_t s, int32_t** d_order, int32_t** d_inv);
// The id order of graph handles and served graphs: Cuthill-McKee on deep graphs
// of low degree (fewer than LOCALITY_MAX_N vertices, maximum degree at most
// LOCALITY_MAX_DEGREE, a BFS deeper than LOCALITY_MIN_DEPTH levels),
// descending degree on all others (relabel.cu).
constexpr int32_t LOCALITY_MAX_N = 1 << 22, LOCALITY_MAX_DEGREE = 64, LOCALITY_MIN_DEPTH = 32;
gbc_status relabel_graph(DevGraph& g, cudaStream_t s, int32_t** d_order, int32_t** d_inv);
// out[r*n + v] = in[r*n + inv[v]], r < rows.
template <typename T>
gbc_status gather_to_caller(const T* d_in, const int32_t* d_inv, int32_t n, int64_t rows, T* d_out, cudaStream_t s);

// Device CSR (+ host-side component information for the GTEPS numerator).
struct DevGraph {
    int32_t n = 0;
    int64_t m = 0;             // directed entries
    int64_t* row = nullptr;    // device [n+1]
    int32_t* col = nullptr;    // device [m]
    const int32_t* w = nullptr;   // device per-vertex weights (reduced graphs), nullable
    const int64_t* ff = nullptr;  // device per-vertex folded distance sums, nullable
    std::vector<int32_t> comp;         // host, per vertex
    std::vector<int64_t> comp_edges;   // host, undirected edges per component
    int32_t max_degree = 0;
    // Level width new lane engines on this graph start with: 2 once some BFS on
    // it went deeper than 8-bit levels allow, so later engines skip that pass.
    mutable int level_bytes_hint = 1;
    // Bytes per exact path count that 128-lane engines on this graph start with:
    // 2, widened to 4 and then 8 once a batch's counts did not fit.
    mutable int sigma_bytes_hint = 2;
};

// Which computation a lane batch performs.
enum class LaneJob { CC, BC, SSSP };

struct LaneRequest {
    LaneJob job = LaneJob::CC;
    const int32_t* d_src = nullptr;  // device sources of this batch
    int32_t kb = 0;                  // sources in this batch (<= lanes)
    int sigma_wide = 0;              // 1: wide-exponent path counts
    int delta_f64 = 1;
    int semantics = GBC_BC_BRANDES;
    unsigned long long* d_cc = nullptr;  // [kb] per-lane distance sums (CC)
    double* d_bcg = nullptr;             // [lanes/32][n] per-32-lane BC partials (BC)
    int32_t* d_dist = nullptr;           // [kb][n] (SSSP) nullable
    uint64_t* d_sigma = nullptr;         // [kb][n] (SSSP) nullable
    bool abort_on_overflow = false;      // exact sigma: stop before the backward sweep if a lane overflowed
    uint32_t* d_profile_key = nullptr;   // [n] (CC job): level of lane 0 << 16 | min level of lanes 1..31
    bool top_down_only = false;          // CC job, 128-lane groups: no bottom-up levels
};

struct LaneResult {
    int64_t levels = 0;
    uint32_t ovf_bits[32] = {};    // per lane group: lanes whose exact sigma overflowed (last batch)
    int32_t overflow_count = 0;    // overflowed lanes, summed over batches
    int64_t frontier_entries = 0;
    int64_t kernel_launches = 0;
    int64_t graph_launches = 0;
    double fwd_ms = 0, bwd_ms = 0;      // device time inside the level-loop graphs
    int64_t fwd_kernels = 0, bwd_kernels = 0;
    int64_t bottom_up_levels = 0;       // closeness levels discovered bottom-up
    int32_t sigma_bytes = 8;            // bytes per exact path count of the last batch
    int64_t neighbour_visits = 0;       // top-down forward tasks' neighbour visits (degrees summed over entries)
    // last batch only: frontier entries per BFS level (regular + hub queue) and
    // device time per forward / dependency-sweep graph launch (levels_per_graph
    // levels each)
    std::vector<int64_t> level_entries;
    std::vector<float> fwd_launch_ms, bwd_launch_ms;
};

class LaneEngine {
public:
    LaneEngine() = default;
    ~LaneEngine();
    LaneEngine(const LaneEngine&) = delete;
    LaneEngine& operator=(const LaneEngine&) = delete;
    // Allocate lane state for `lanes` (multiple of 32, <= 1024) on graph g.
    // group_lanes: sources per lane group (32: one per warp thread; 128: four per thread;
    // 1: one lane per task, lane-major state, for deep graphs whose lanes rarely share a level).
    gbc_status init(const DevGraph* g, int32_t lanes, bool need_bc, int sparse_lanes, int levels_per_graph,
                    cudaStream_t stream, int group_lanes = 32);
    // Expansion tuning (negative = default: 2 / 16 / 16 / 256 threads / 16;
    // levels_per_graph 0 and block_threads 0 = default too).  block_threads: threads per CTA of the level kernels (128, 256 or
    // 512); bu_share: closeness levels on 128-lane groups go bottom-up once
    // past the frontier peak while frontier edges x bu_share exceed all edges x
    // groups (0: never).  A change drops the captured level-loop graphs, which
    // hold the old values.
    void set_tuning(int sparse_lanes, int light_steps, int levels_per_graph, int block_threads = -1, int bu_share = -1);
    int block_threads() const { return block_; }
    int bu_share() const { return bu_share_; }
    // One batch of rq.kb <= lanes sources (forward, then backward for BC).
    gbc_status run(const LaneRequest& rq, LaneResult& res);
    // BC accumulation across batches: zero the per-group partials / reduce them into d_bc[n].
    gbc_status bc_begin();
    gbc_status bc_finish(double* d_bc);
    // d_dst: device table of ng device pointers (or null): dst[g][v] += partial of group g.
    gbc_status bc_scatter(double* const* d_dst);
    // Per-lane distance sums of the last CC batch (lanes entries) to the host.
    gbc_status cc_read(unsigned long long* h_cc, int32_t count);
    int32_t lanes() const { return lanes_; }
    int32_t group_lanes() const { return 1 << gs_; }
    int level_bytes() const { return lvl_bytes_; }
    bool has_bc() const { return need_bc_; }
    const DevGraph* graph() const { return g_; }
    cudaStream_t stream() const { return stream_; }
    size_t device_bytes() const { return bytes_; }
    static size_t bytes_needed(int32_t n, int32_t lanes, bool need_bc, int32_t group = 32);

private:
    friend struct LaneAccess;
    // the captured level loop of `count` level kernels for a kernel key
    gbc_status get_graph(int key, int count, cudaGraphExec_t* out);
    gbc_status alloc_queue(unsigned long long cap, unsigned long long hcap);
    gbc_status ensure_events(size_t count);
    void release();

    const DevGraph* g_ = nullptr;
    int32_t lanes_ = 0, ng_ = 0;
    int gs_ = 5;          // lanes per group = 1 << gs_
    bool need_bc_ = false;
    int sparse_ = 2;
    int light_ = 16;
    int lpg_ = 16;
    int block_ = 256;     // threads per CTA of the level kernels
    int bu_share_ = 16;   // direction-switch threshold of closeness levels (0: top-down only)
    int lvl_bytes_ = 1;   // 1 while every BFS stays under 254 levels, else 2
    int sig_bytes_ = 8;   // bytes per exact path count (128-lane groups: 2 or 4 while the counts fit)
    int width_index() const;
    int hub_lim_ = -1;    // ids below this are the hubs (ids in descending degree order), -1: unknown
    size_t lvl_sz_ = 0, vmark_sz_ = 0, sig_sz_ = 0, rho_sz_ = 0, bcg_sz_ = 0;   // bytes of the cached buffers
    cudaStream_t stream_ = nullptr;
    size_t bytes_ = 0;
    uint16_t* lvl_ = nullptr;
    uint64_t* sig_ = nullptr;
    void* rho_ = nullptr;
    int32_t* vmark_ = nullptr;
    uint32_t* fq_ = nullptr;
    unsigned long long fcap_ = 0;
    unsigned long long* foff_ = nullptr;
    uint32_t* hq_ = nullptr;              // hub frontier entries
    unsigned long long hcap_ = 0;
    unsigned long long* hoff_ = nullptr;
    int64_t n_hubs_ = 0;
    void* ctl_ = nullptr;
    void* ctl_host_ = nullptr;
    uint32_t* ovf_ = nullptr;
    double* bcg_ = nullptr;
    unsigned long long* ccbuf_ = nullptr;
    int32_t* srcw_ = nullptr;             // per-lane source weights of the running batch
    int4* ell_ = nullptr;                 // one lane per task, degree <= 8: padded neighbour table
    int ell_q_ = 0;                       // int4 slots per vertex of ell_ (0: no table)
    size_t ell_sz_ = 0;                   // bytes of ell_
    // bottom-up closeness levels (128-lane groups), set up on the first closeness batch
    int32_t* vcomp_ = nullptr;            // component label of every vertex
    int32_t* lcomp_ = nullptr;            // component label of every lane's source
    uint32_t* done_ = nullptr;            // [ng][ceil(n/32)] bits: (vertex, group) has nothing left to reach
    size_t done_sz_ = 0;
    struct Captured { int key = -1; cudaGraphExec_t exec = nullptr; };
    std::vector<Captured> graphs_;
    int depth_hint_ = 0;                  // levels of the engine's last batch: the first forward graph's length
    int sm_count_ = 0;
    std::vector<cudaEvent_t> ev_;       // timing events, two per graph launch
};

// Level-profile key of every vertex of a degree-relabelled device graph: one
// 32-lane closeness batch from its 32 highest-degree vertices; key = (level
// from the top vertex) << 16 | (nearest of the others); depth = that batch's
// levels (api.cu).  Sources sorted by key share lane groups with sources
// whose BFS levels move together; graphs whose depth stays within
// SMALL_WORLD_DEPTH run on 128-lane groups.
gbc_status level_profile_key(const DevGraph& g, cudaStream_t stream, std::vector<uint32_t>& key, int32_t& depth);
constexpr int32_t SMALL_WORLD_DEPTH = 32;
// Graphs deeper than SMALL_WORLD_DEPTH with at most this degree and fewer vertices run one lane per
// task by default (the entry packing v << 10 | lane needs n < 2^22).
constexpr int32_t ONE_LANE_MAX_DEGREE = 64, ONE_LANE_MAX_N = 1 << 22;

// Plain engine: one source at a time, int32 distances, uint64 sigma, the
// level loop driven from the host with one device->host read per level.
gbc_status plain_bc(const DevGraph* g, const int32_t* h_src, int32_t k, int semantics, int delta_f64,
                    double* d_bc, cudaStream_t st, LaneResult& res);
gbc_status plain_cc(const DevGraph* g, const int32_t* h_src, int32_t k, int64_t* h_cc, cudaStream_t st,
                    LaneResult& res);

}  // namespace gbc
