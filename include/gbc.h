/*
 * gbc.h -- native C ABI of libgbc, a GB300 (sm_103a) implementation of the
 * XPPGX/BC centrality path: Brandes betweenness centrality and closeness
 * (distance-sum) centrality on undirected, unweighted graphs, with the
 * degree-1 folding and articulation-point reductions.
 *
 * Plain pointers and sizes only.  Every call returns a gbc_status; on error
 * gbc_last_error() gives a message for the calling thread.  Host-buffer
 * entry points copy inputs to the device and results back; *_device entry
 * points take device pointers and a cudaStream_t (passed as void*).
 *
 * Reference interfaces replaced (paths within the XPPGX/BC project):
 *   gbc_bc          <- void computeBC(struct CSR*, float*)       Seq_Brandes/Brandes.c:224
 *   gbc_cc          <- int* computeCC(struct CSR*, int*)         Seq_CC/CC.cpp:37
 *   gbc_cc_reduced  <- void compute_D1_AP_CC_shareBased_DegreeOrder(struct CSR*, int*)
 *                                                                Seq_CC/CC.cpp:1728
 *   gbc_reduce_*    <- D1Folding (Lib/D1Process/D1Process.c:5), AP_detection /
 *                      AP_Copy_And_Split / rebuildGraph (Lib/AP_Process/AP_Process.c:6,468,1141)
 *   gbc_bc_plain / gbc_cc_plain (one source at a time) <- the reference's GPU
 *                      programs' per-source level loop (GPU_FAN/gpu_fan.cu:59,
 *                      parallel_CC/para_CC.cu:61)
 * The struct-CSR drop-in names themselves are declared in gbc_compat.h.
 */
#ifndef GBC_H
#define GBC_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GBC_OK = 0,
    GBC_ERR_ARG = 1,        /* invalid argument (size, index, pointer, option) */
    GBC_ERR_CUDA = 2,       /* CUDA runtime error */
    GBC_ERR_NOMEM = 3,      /* device or host allocation failed / over budget */
    GBC_ERR_OVERFLOW = 4,   /* exact uint64 path counts overflowed (GBC_SIGMA_EXACT) */
    GBC_ERR_LIMIT = 5,      /* a device-side cap was hit (levels, queue capacity) */
    GBC_ERR_NOT_FOUND = 6,  /* unknown handle / graph id */
    GBC_ERR_BUSY = 7,       /* admission refused: no room for the request now */
    GBC_ERR_TIMEOUT = 8,    /* request deadline passed */
    GBC_ERR_NO_DEVICE = 9   /* no usable CUDA device */
} gbc_status;

/* Betweenness semantics. */
enum {
    GBC_BC_BRANDES = 0,     /* textbook: delta_s(w) added once per source */
    GBC_BC_REFERENCE = 1    /* XPPGX/BC: delta_s(w) added once per shortest-path
                               predecessor of w (Seq_Brandes/Brandes.c:319-326) */
};
/* Precision of the dependency (delta) sweep; BC sums across sources are FP64. */
enum { GBC_DELTA_F32 = 0, GBC_DELTA_F64 = 1 };
/* Path-count (sigma) representation. */
enum {
    GBC_SIGMA_AUTO = 0,     /* exact uint64; on overflow re-run the batch in WIDE form */
    GBC_SIGMA_EXACT = 1,    /* exact uint64; overflow is an error (GBC_ERR_OVERFLOW) */
    GBC_SIGMA_WIDE = 2      /* 44-bit mantissa, 20-bit exponent: up to 2^524287, ~6e-14 relative */
};
/* Engine. */
enum {
    GBC_ENGINE_AUTO = 0,
    GBC_ENGINE_PLAIN = 1,   /* one source at a time, host-driven level loop */
    GBC_ENGINE_LANES = 2    /* batched multi-source lanes, graph-captured level loop */
};

typedef struct {
    int32_t semantics;        /* GBC_BC_* (default GBC_BC_BRANDES) */
    int32_t delta_precision;  /* GBC_DELTA_* (default GBC_DELTA_F64) */
    int32_t sigma_mode;       /* GBC_SIGMA_* (default AUTO) */
    int32_t engine;           /* GBC_ENGINE_* (default AUTO = LANES) */
    int32_t lanes;            /* sources per batch, multiple of 32 in [32,1024]; 0 = autotune */
    int32_t sparse_lanes;     /* a frontier task with <= this many active lanes expands
                                 edge-parallel, otherwise lane-parallel; -1 = autotune */
    int32_t levels_per_graph; /* level kernels per captured CUDA graph; 0 = default (16, or 64 on
                                 graphs deeper than 8-bit levels allow); a batch's first forward graph
                                 and its sweep's last graph may be shorter, sized to the depth */
    int32_t source_order;     /* 0: group sources with similar BFS level profiles into the same
                                 lane group (results do not depend on it); 1: lanes in the order given */
    int32_t light_steps;      /* a frontier task with (active lanes x degree) <= this is expanded by a
                                 single thread, 32 tasks per warp; 0 = never; -1 = autotune */
    int32_t group_lanes;      /* sources per lane group: 32 (one per warp thread) or 128 (four per
                                 thread; lanes must then be a multiple of 128), or 1 (one lane per
                                 task, lane-major state: deep graphs whose lanes rarely share a
                                 level; fewer than 2^22 vertices); 0 = automatic */
    int32_t direction;        /* closeness with 128-lane groups: 0 = switch between top-down and
                                 bottom-up levels by frontier size (default); 1 = top-down only */
    int32_t block_threads;    /* threads per CTA of the level kernels: 128, 256 or 512; 0 = the
                                 autotuned value, else 256 */
    int32_t bu_share;         /* closeness with 128-lane groups: a level goes bottom-up once the
                                 frontier is past its peak while its edges x bu_share exceed all
                                 edges x lane groups; 0 = the autotuned value, else 16 */
    int32_t reserved[3];
} gbc_options;

typedef struct {
    int64_t sources;          /* sources processed by the last call */
    int64_t batches;          /* lane batches */
    int64_t levels;           /* BFS levels summed over batches (forward) */
    int64_t kernel_launches;  /* kernels launched by the library in the last call */
    int64_t graph_launches;   /* CUDA graph launches in the last call */
    int64_t edges_traversed;  /* sum over sources of undirected edges in the source's component */
    int64_t frontier_entries; /* (vertex, lane-group) frontier entries over all levels */
    int64_t sigma_overflow_lanes; /* lanes whose exact sigma overflowed (before any wide re-run) */
    double  kernel_ms;        /* device time of the traversal kernels (CUDA events) */
    double  total_ms;         /* wall time of the call */
    int32_t lanes;            /* lanes per batch actually used */
    int32_t sigma_mode_used;  /* GBC_SIGMA_EXACT or GBC_SIGMA_WIDE */
    double  fwd_ms;           /* device time of the forward (BFS / path count) level kernels */
    double  bwd_ms;           /* device time of the dependency-sweep level kernels */
    int64_t fwd_kernels;      /* forward level kernels launched (incl. no-op tail launches) */
    int64_t bwd_kernels;      /* dependency-sweep level kernels launched */
    int32_t group_lanes;      /* lanes per group of the engine that ran (1, 32 or 128; the plain
                                 engine reports 1 with lanes = 1) */
    int32_t bottom_up_levels; /* closeness levels discovered bottom-up, summed over batches */
    int32_t sigma_bytes;      /* bytes per exact path count in the last batch: 128-lane groups store
                                 them in 2 or 4 bytes while they fit, else 8 */
    int64_t neighbour_visits; /* adjacency entries scanned by top-down forward tasks (each frontier
                                 entry's degree), summed over batches; the sweep scans the same */
} gbc_run_stats;

typedef struct gbc_graph_s* gbc_graph;

void gbc_options_default(gbc_options* opt);
const char* gbc_last_error(void);
const char* gbc_version(void);
/* Number of CUDA devices visible (0 when none; never fails). */
int gbc_device_count(void);
/* Make `device` the calling thread's device for the library's own CUDA
 * runtime (it is linked statically, so a device chosen through another
 * runtime, e.g. a framework's, need not reach it).  Graphs, engines and
 * servers live on the device that was current when they were created; a
 * server's worker threads use its device. */
gbc_status gbc_set_device(int device);

/* ---- device-resident graphs ------------------------------------------- */
/* Upload an undirected CSR (both directions of every edge present):
 * row[n+1] int64 offsets, col[row[n]] int32 neighbour ids in [0,n).
 * No self-loops are expected; duplicates count as parallel edges. */
gbc_status gbc_graph_create(const int64_t* row, const int32_t* col, int32_t n, gbc_graph* out);
/* Same, from device pointers (copied; the caller keeps ownership). */
gbc_status gbc_graph_create_device(const int64_t* d_row, const int32_t* d_col, int32_t n,
                                   int64_t m_directed, gbc_graph* out);
gbc_status gbc_graph_destroy(gbc_graph g);
/* Vertex weights for the reduced-graph forms of the reference's algorithms
 * (the reach "representNode" and folded distance sums "ff" that D1Folding
 * leaves, Lib/D1Process/D1Process.c:43-46; used by compute_D1_CC,
 * Seq_CC/CC.cpp:418).  w[n] >= 0 and ff[n] >= 0 are host arrays in the
 * caller's ids; either may be NULL (w = 1, ff = 0); both NULL clears them.
 * With weights set, gbc_cc returns sum over reached v of (ff[v] + d(s,v)*w[v])
 * (v = s included), and gbc_bc (GBC_BC_BRANDES only) returns
 * sum_s w[s] sum_t w[t] sigma_st(v)/sigma_st.  The plain engine refuses
 * weighted graphs. */
gbc_status gbc_graph_set_weights(gbc_graph g, const int32_t* w, const int64_t* ff);
/* Device-side ingest: edge list (u[i], v[i]), i < m, ids in [0, n) -> the
 * symmetric CSR without self-loops or repeated edges, rows in ascending
 * neighbour order, built on the GPU (radix sort of both directions, unique,
 * row offsets).  Replaces buildGraph + createCSR (Lib/AdjList/AdjList.c:13,
 * Lib/CSR/CSR.c:9) for callers that hold an edge list.  _device takes device
 * arrays; the host variant copies them first. */
gbc_status gbc_graph_from_edges(const int32_t* u, const int32_t* v, int64_t m, int32_t n, gbc_graph* out);
gbc_status gbc_graph_from_edges_device(const int32_t* d_u, const int32_t* d_v, int64_t m, int32_t n, gbc_graph* out);
/* The graph's CSR copied to malloc'd host arrays (free with gbc_free). */
gbc_status gbc_graph_export(gbc_graph g, int64_t** row, int32_t** col, int32_t* n);
gbc_status gbc_graph_info(gbc_graph g, int32_t* n, int64_t* m_directed, size_t* device_bytes);
/* Statistics of the last compute call on this graph. */
gbc_status gbc_graph_last_stats(gbc_graph g, gbc_run_stats* st);
/* Level profile of the last lane batch of the last compute call on this
 * graph: *levels = BFS levels, entries[d] (up to entries_cap) = frontier
 * (vertex, lane-group) entries of level d; fwd_ms / bwd_ms (up to launch_cap)
 * = device time of each forward / dependency-sweep graph launch, which runs
 * levels_per_graph level kernels (set levels_per_graph = 1 for per-level
 * times).  Output arrays may be NULL. */
gbc_status gbc_graph_last_levels(gbc_graph g, int64_t* entries, int32_t entries_cap, float* fwd_ms, float* bwd_ms,
                                 int32_t launch_cap, int32_t* levels, int32_t* fwd_launches, int32_t* bwd_launches);

/* ---- betweenness --------------------------------------------------------
 * bc[n] (host) receives sum over the k sources of the per-source
 * dependencies, under opt->semantics; k = 0 with sources = NULL means all
 * n vertices.  Unnormalised: ordered source/target pairs, as the reference. */
gbc_status gbc_bc(gbc_graph g, const int32_t* sources, int32_t k, const gbc_options* opt, double* bc);
gbc_status gbc_bc_device(gbc_graph g, const int32_t* d_sources, int32_t k, const gbc_options* opt,
                         double* d_bc, void* stream);

/* Autotuner: time one betweenness batch of the given sources (k = 0: all
 * vertices) per candidate expansion setting -- lane-group width (32/128, and
 * 1 on deep graphs of degree <= 64),
 * one-thread task threshold (light_steps 0/8/16/32), edge-parallel threshold
 * (sparse_lanes 1/2/4), level kernels per captured graph (16/64, deep graphs),
 * threads per CTA of the level kernels (block_threads 128/256/512) and batch
 * width (halved from the widest while the time per source drops, down to 32
 * lanes), one at a time -- and keep the fastest on the graph.  On 128-lane
 * groups it then times one closeness batch per direction-switch share
 * (bu_share 4/8/16/32/64, or top-down only).  Later calls whose
 * options leave a setting to autotuning (-1 / 0) use the tuned value; values
 * set in the options are not tuned.  *chosen (nullable) receives the options
 * with the chosen settings filled in.  Results do not depend on the settings
 * beyond FP64 summation order. */
gbc_status gbc_autotune(gbc_graph g, const int32_t* sources, int32_t k, const gbc_options* opt, gbc_options* chosen);

/* ---- closeness (distance sums) -----------------------------------------
 * cc[i] = sum of hop distances from sources[i] to every vertex it reaches
 * (Seq_CC/CC.cpp:76-100); k = 0 with sources = NULL means all n vertices. */
gbc_status gbc_cc(gbc_graph g, const int32_t* sources, int32_t k, const gbc_options* opt, int64_t* cc);
gbc_status gbc_cc_device(gbc_graph g, const int32_t* d_sources, int32_t k, const gbc_options* opt,
                         int64_t* d_cc, void* stream);

/* ---- per-source distances and exact path counts (parity surface) -------
 * dist[k*n] int32 (-1 unreachable), sigma[k*n] uint64 exact, ovf[k] = 1
 * when that source's counts overflowed uint64 (its sigma row is then
 * invalid).  Any pointer may be NULL. */
gbc_status gbc_sssp(gbc_graph g, const int32_t* sources, int32_t k, const gbc_options* opt,
                    int32_t* dist, uint64_t* sigma, uint8_t* ovf);

/* ---- closeness without allocation ----------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory at call time -- a process that reserved all of HBM for its own pool
 * up front (any cudaMalloc would fail or fragment it), or a latency-critical
 * path that must not risk the device synchronisation cudaMalloc/cudaFree can
 * bring.  Device CSR (row[n+1] int64, col int32), device sources[k]; writes
 * cc[i] (device int64) = sum of hop distances from sources[i], like gbc_cc.
 * The BFS state lives in one fixed file-scope device array (16 MB on every
 * GPU that loads the library, kept until exit), so n is limited to
 * GBC_NOALLOC_MAX_VERTICES; larger graphs get GBC_ERR_ARG.  Nothing is
 * allocated on the host or the device.  Every call shares that array and
 * re-initialises it; calls that overlap on the GPU race and must be
 * serialised by the caller.  The first call on a device looks up the array's
 * device address; make that first call before any stream capture.  Every
 * call first checks the CSR on the device (row[0] == 0, rows non-decreasing,
 * col entries in [0,n)) and refuses a bad one with GBC_ERR_ARG before the BFS
 * touches the array.  Runs on `stream` (a cudaStream_t): it waits for
 * `stream` after the CSR check and after every BFS level, whose frontier size
 * it reads back, and returns when the results are written. */
#define GBC_NOALLOC_MAX_VERTICES (1 << 21)
gbc_status gbc_cc_noalloc(const int64_t* d_row, const int32_t* d_col, int32_t n, const int32_t* d_sources,
                          int32_t k, int64_t* d_cc, void* stream);

/* ---- D1 folding + articulation-point (block) reduction ---------------- */
typedef struct gbc_reduced_s* gbc_reduced;
typedef struct {
    int32_t n;                 /* vertex slots of the input */
    int32_t d1_folded;         /* degree-1 vertices folded (D1Process.c:71) */
    int32_t d1_hubs;           /* unfolded vertices that absorbed a folded vertex */
    int32_t alive;             /* vertices left after folding */
    int32_t articulation_points;
    int32_t blocks;            /* biconnected blocks (incl. bridges) of the folded graph */
    int32_t max_block;         /* vertices in the largest block */
    int32_t block_slots;       /* vertex slots of the block graph (APs counted once per block) */
    int64_t block_edges;       /* directed CSR entries of the block graph */
    int32_t components;        /* connected components of the input (isolated slots included) */
    int32_t on_device;         /* 1: folded and split on the device (gbc_reduce) */
    int32_t fold_rounds;       /* device path: peeling rounds of the folding */
    int32_t forest_levels;     /* device path: levels of the BFS spanning forest of the folded graph */
    int32_t reserved[4];
} gbc_reduced_info;

/* Fold and split a host CSR (vertex slots [start, n) are real vertices;
 * start = 1 marks the reference's phantom slot 0 of 1-based inputs).
 * Replaces D1Folding + AP_detection + AP_Copy_And_Split + rebuildGraph
 * (Lib/D1Process/D1Process.c:5, Lib/AP_Process/AP_Process.c:6,468,1141).
 * gbc_reduce runs the folding (peeling rounds) and the block split
 * (Tarjan-Vishkin over a BFS spanning forest) on the device;
 * gbc_reduce_host runs the same reduction on the host (O(n + m) folding and a
 * Hopcroft-Tarjan DFS), where the reference runs it.  Both give the same
 * folded vertices, articulation points, blocks and results. */
gbc_status gbc_reduce(const int64_t* row, const int32_t* col, int32_t n, int32_t start, gbc_reduced* out);
gbc_status gbc_reduce_host(const int64_t* row, const int32_t* col, int32_t n, int32_t start, gbc_reduced* out);
/* gbc_reduce on a CSR already in device memory (d_row[n+1], d_col[d_row[n]]
 * on the current device, complete before the call, not modified); its
 * entries are checked on the device as gbc_reduce checks them. */
gbc_status gbc_reduce_device(const int64_t* d_row, const int32_t* d_col, int32_t n, int32_t start, gbc_reduced* out);
gbc_status gbc_reduced_info_get(gbc_reduced r, gbc_reduced_info* info);
/* Closeness of every vertex slot through the reduction: cc[n] (host).
 * Equal to gbc_cc over all vertices of the unreduced graph. */
gbc_status gbc_cc_reduced(gbc_reduced r, const gbc_options* opt, int64_t* cc);
/* Betweenness (GBC_BC_BRANDES) of every vertex slot through D1 folding and
 * the block split: reach-weighted Brandes inside every block with the clone
 * weights w' on the device (every slot a source), plus the pairs each
 * articulation point separates and the exact pair counts of the folded
 * pendant trees.  Equal to gbc_bc over all vertices of the unreduced graph. */
gbc_status gbc_bc_reduced(gbc_reduced r, const gbc_options* opt, double* bc);
gbc_status gbc_reduced_destroy(gbc_reduced r);
/* The block graph the reduction hands to the device: slot CSR (malloc'd,
 * free with gbc_free) and per-slot clone weights w'. */
gbc_status gbc_reduced_block_graph(gbc_reduced r, int64_t** row, int32_t** col, int32_t** weight, int32_t* n_slots);
/* Host assembly step: given D[s] = sum_u d(s,u) * w'(u) for every slot s of
 * the block graph, write the closeness of every vertex slot to cc[n]. */
gbc_status gbc_reduced_assemble_cc(gbc_reduced r, const int64_t* D, int64_t* cc);
/* The folded ("core") graph betweenness runs on: CSR over the unfolded
 * vertices (malloc'd, free with gbc_free), their reach weights and the
 * vertex slot of each core id. */
gbc_status gbc_reduced_core_graph(gbc_reduced r, int64_t** row, int32_t** col, int32_t** weight, int32_t** vertex,
                                  int32_t* n_core);
/* Host assembly step for betweenness: core_bc[i] = reach-weighted Brandes
 * betweenness of core id i; adds the folding contributions, writes bc[n]. */
gbc_status gbc_reduced_assemble_bc(gbc_reduced r, const double* core_bc, double* bc);

/* ---- synthetic graphs (host CSR, malloc'd; free with gbc_free) --------
 * All generators are deterministic for a seed on any host. */
gbc_status gbc_gen_ba(int32_t n, int32_t m, uint64_t seed, int64_t** row, int32_t** col);
gbc_status gbc_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                        int32_t permute, int64_t** row, int32_t** col, int32_t* n);
gbc_status gbc_gen_grid(int32_t rows, int32_t cols, double remove_frac, uint64_t seed, int32_t largest_only,
                        int64_t** row, int32_t** col, int32_t* n);
gbc_status gbc_gen_er(int32_t n, double avg_degree, uint64_t seed, int64_t** row, int32_t** col);
/* Attach `trees` pendant paths of length 1..max_depth (uniform) to uniformly
 * chosen vertices of a CSR; returns a new CSR. */
gbc_status gbc_add_pendants(const int64_t* row, const int32_t* col, int32_t n, int32_t trees, int32_t max_depth,
                            uint64_t seed, int64_t** row_out, int32_t** col_out, int32_t* n_out);
/* Attach `cycles` cycles of min_len..max_len vertices (uniform, min_len >= 3)
 * to uniformly chosen vertices of a CSR (each through its chosen vertex and
 * len - 1 new ones): articulation points with small blocks behind them;
 * returns a new CSR. */
gbc_status gbc_add_cycles(const int64_t* row, const int32_t* col, int32_t n, int32_t cycles, int32_t min_len,
                          int32_t max_len, uint64_t seed, int64_t** row_out, int32_t** col_out, int32_t* n_out);
/* Edge-list text file (header "n m", then "u v" lines; 0- or 1-based as in
 * Lib/AdjList/AdjList.c:13) -> CSR over n (0-based) or n+1 (1-based) slots;
 * *start = 0 or 1.  Neighbours ordered by neighbour degree ascending. */
gbc_status gbc_read_edgelist(const char* path, int64_t** row, int32_t** col, int32_t* n, int32_t* start);
/* Score file in the reference's BC_Score.txt layout (Seq_Brandes/Brandes.c:2318-2321):
 * a "start end" line, then values[v] for v = start..end, one "%f" per line,
 * each rounded to FP32 first as the reference's float arrays are.  append != 0
 * appends as the reference's "a" mode does. */
gbc_status gbc_write_scores(const char* path, const double* values, int32_t start, int32_t end, int32_t append);
void gbc_free(void* p);

/* Lane-state buffers of destroyed graphs and engines are kept for reuse by
 * later engines of the same size (creating and destroying graphs in a loop
 * then costs no cudaMalloc/cudaFree).  This returns the cached buffers of the
 * current device to the driver.  Cached bytes count as free when the library
 * sizes its own engines. */
gbc_status gbc_release_cached_memory(void);

/* ---- serving: continuous batching over device-resident graphs ---------
 * A server owns a set of registered graphs and worker threads.  Requests
 * (exact CC, exact BC, or k-source sampled BC) are admitted in arrival order
 * while their device bytes fit the HBM budget: the result vectors of the
 * admitted requests not yet fetched (n FP64 values per BC request) plus, per
 * graph with admitted work, its lane engine or the narrowest engine it could
 * run with.  A request that does not fit waits, and later ones wait behind
 * it; one that could never fit fails with GBC_ERR_NOMEM.  Sources of
 * concurrent requests on the same graph share lane batches.  Results are
 * identical (FP64 tolerance) alone and mixed. */
typedef struct gbc_server_s* gbc_server;
enum { GBC_Q_CC = 0, GBC_Q_BC = 1, GBC_Q_BC_SAMPLED = 2 };
enum { GBC_REQ_QUEUED = 0, GBC_REQ_RUNNING = 1, GBC_REQ_DONE = 2, GBC_REQ_FAILED = 3, GBC_REQ_CANCELLED = 4 };

typedef struct {
    size_t  hbm_budget_bytes;   /* engines + result vectors; 0 = 50% of free device memory */
    int32_t max_lanes;          /* lanes per shared batch (multiple of 32), 0 = 1024 */
    int32_t max_inflight;       /* requests admitted at once, 0 = 64 */
    int32_t workers;            /* lane batches in flight at once, on different graphs; 0 = 8 */
    int32_t reserved[7];
} gbc_server_config;

gbc_status gbc_server_create(const gbc_server_config* cfg, gbc_server* out);
gbc_status gbc_server_destroy(gbc_server s);
/* Register a host CSR; the server keeps it resident.  *graph_id out. */
gbc_status gbc_server_add_graph(gbc_server s, const int64_t* row, const int32_t* col, int32_t n, int32_t* graph_id);
/* Submit a query.  kind GBC_Q_*; for GBC_Q_BC_SAMPLED, k sources drawn
 * uniformly with the seed.  deadline_ms <= 0 means none.  *req_id out. */
gbc_status gbc_server_submit(gbc_server s, int32_t graph_id, int32_t kind, int32_t k, uint64_t seed,
                             const gbc_options* opt, double deadline_ms, int64_t* req_id);
/* Device bytes a request of this kind on this graph is charged at
 * admission: its result vector (until fetched) and the narrowest lane engine
 * of the graph (charged once per graph with admitted work). */
gbc_status gbc_server_request_bytes(gbc_server s, int32_t graph_id, int32_t kind, size_t* result_bytes,
                                    size_t* engine_bytes);
/* Poll: *state = GBC_REQ_*; when DONE, result buffers may be fetched. */
gbc_status gbc_server_poll(gbc_server s, int64_t req_id, int32_t* state);
/* Block until the request finishes (timeout_ms <= 0: no timeout). */
gbc_status gbc_server_wait(gbc_server s, int64_t req_id, double timeout_ms, int32_t* state);
/* Copy the result: BC kinds fill bc[n]; CC fills cc[n]. Latency in ms
 * from submit to completion goes to *latency_ms. Frees the request. */
gbc_status gbc_server_fetch(gbc_server s, int64_t req_id, double* bc, int64_t* cc, double* latency_ms);
gbc_status gbc_server_cancel(gbc_server s, int64_t req_id);
/* The source vertices of a request (the drawn sample for GBC_Q_BC_SAMPLED):
 * *k = count; out (may be NULL) receives them if cap >= count, in the order
 * the server runs them (grouped by BFS level profile, not the draw order),
 * then the sources without edges: those reach nothing, add nothing to
 * betweenness, have closeness sum 0, and take no lane.  Valid until the
 * request is fetched. */
gbc_status gbc_server_sources(gbc_server s, int64_t req_id, int32_t* out, int32_t cap, int32_t* k);
/* Aggregate counters: completed requests, lane batches, shared batches
 * (batches that carried sources of more than one request), edges traversed. */
gbc_status gbc_server_counters(gbc_server s, int64_t* completed, int64_t* batches, int64_t* shared_batches,
                               int64_t* edges_traversed, double* busy_ms);

#ifdef __cplusplus
}
#endif
#endif
