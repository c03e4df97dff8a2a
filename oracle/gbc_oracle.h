/*
 * gbc_oracle.h -- CPU restatement of the XPPGX/BC centrality path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; it is the checker that tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg use.  Arithmetic is widened relative to the
 * reference (uint64 sigma with overflow tracking, FP64 delta and BC, int64
 * distance sums); each function names the reference file:line it restates.
 *
 * Vertex-ID convention (same as the reference's struct CSR): N vertex slots
 * [0, N).  For a 1-based edge list, slot 0 is a phantom vertex with no edges
 * (the reference sets csrV[0] = -1 and starts traversal at startNodeID = 1,
 * Lib/CSR/CSR.c:20-26,93).  row[N+1] are int64 offsets into col[].
 */
#ifndef GBC_ORACLE_H
#define GBC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BC_BRANDES = 0, ORC_BC_REFERENCE = 1 };

/* Edge-list text reader + CSR builder (Lib/AdjList/AdjList.c:13-150,
 * Lib/CSR/CSR.c:9-108).  Neighbour lists are ordered by neighbour degree
 * ascending, ties in file order.  Arrays are malloc'd; free with orc_free. */
int orc_load_edgelist(const char* path, int32_t* N, int64_t* M, int32_t* start,
                      int64_t** row, int32_t** col);
void orc_free(void* p);

/* Single-source forward BFS (Seq_Brandes/Brandes.c:274-298): hop distances
 * (-1 unreachable), exact uint64 shortest-path counts with a per-vertex
 * overflow flag, and the number of BFS-DAG predecessors of each vertex. */
int orc_sssp(int32_t N, const int64_t* row, const int32_t* col, int32_t s,
             int32_t* dist, uint64_t* sigma, uint8_t* sigma_ovf, int32_t* npred);

/* Brandes BC over the given sources (Seq_Brandes/Brandes.c:224-372) in FP64.
 * semantics ORC_BC_REFERENCE adds delta_s(w) once per predecessor of w
 * (Brandes.c:319-326); ORC_BC_BRANDES adds it once.  scaled != 0 computes
 * delta from level-normalised FP64 path counts (valid where sigma exceeds
 * uint64); otherwise from exact uint64 sigma.  n_ovf receives the number of
 * (source, vertex) pairs whose exact sigma overflowed uint64.  bc[N] is
 * accumulated into (caller zeroes it). nthreads > 1 splits the sources over
 * pthreads and sums per-thread partials in thread order. */
int orc_bc(int32_t N, const int64_t* row, const int32_t* col,
           const int32_t* src, int32_t k, int semantics, int scaled,
           int nthreads, double* bc, int64_t* n_ovf);

/* Closeness distance sums (Seq_CC/CC.cpp:37-117): cc[i] = sum of hop
 * distances from src[i] to every vertex it reaches.  With w/ff non-NULL the
 * D1-folded weighted form of Seq_CC/CC.cpp:1838-1842 is used instead:
 * cc[i] = ff[s] + sum_{v != s reached} (ff[v] + d(s,v) * w[v]). */
int orc_cc(int32_t N, const int64_t* row, const int32_t* col,
           const int32_t* src, int32_t k, const int64_t* w, const int64_t* ff,
           int nthreads, int64_t* cc);

/* Shared-BFS closeness (Seq_CC/CC.cpp:1845-2022, with its float twin
 * Seq_Brandes/Brandes.c:1744-2016): sources in the order given; each BFS
 * from an undone source also derives the sums of up to 32 undone neighbours
 * from the SI / relation bitmasks.  Unweighted; cc[N] (all vertices of the
 * sources' components receive their sum).  Returns the number of BFS runs. */
int64_t orc_cc_shared(int32_t N, const int64_t* row, const int32_t* col,
                      const int32_t* order, int32_t norder, int64_t* cc);

/* Degree-1 folding (Lib/D1Process/D1Process.c:5-154).  Works on a private
 * copy of the adjacency.  Outputs, per vertex slot: represent (reach, 1 for
 * unfolded vertices), ff (folded distance sum), parent (-1 if not folded),
 * and live_lo[v] = first live adjacency index after folding (the
 * reference's advanced csrV[v]; live neighbours of v are
 * col_out[live_lo[v] .. row[v+1]) ).  fold_order[] lists folded vertices in
 * folding order.  Unlike the reference, a vertex whose last neighbour was
 * folded into it (the root of a tree component) is not folded again. */
int orc_d1_fold(int32_t N, const int64_t* row, const int32_t* col,
                int32_t start, int64_t* represent, int64_t* ff, int32_t* parent,
                int64_t* live_lo, int32_t* col_out, int32_t* fold_order,
                int32_t* n_folded, int32_t* n_hub);

/* Closeness via D1 folding (Seq_CC/CC.cpp:418-499): weighted BFS on the
 * folded graph, then recovery CC[d1] = CC[parent] + N' - 2 represent[d1]
 * in reverse fold order (CC.cpp:2037-2049).  fix_components != 0 uses N' =
 * size of d1's connected component; 0 uses the reference's global vertex
 * count (wrong on disconnected graphs). cc[N] out. */
int orc_d1_cc(int32_t N, const int64_t* row, const int32_t* col, int32_t start,
              int fix_components, int64_t* cc);

/* Articulation points of the D1-folded graph (Lib/AP_Process/AP_Process.c:
 * 6-225), by iterative Tarjan.  is_ap[N] out; returns the count. */
int32_t orc_articulation_points(int32_t N, const int64_t* row, const int32_t* col,
                                int32_t start, uint8_t* is_ap);

/* Per-AP part information (Lib/AP_Process/AP_Process.c:383-466, getPartsInfo)
 * on the D1-folded graph: for each AP a, CC[a] = ff[a] + sum over parts of
 * sum_{v in part} (ff[v] + d(a,v) represent[v])  (AP_Process.c:741).
 * cc_ap[N] receives it for APs (others untouched). Returns the AP count. */
int32_t orc_ap_cc(int32_t N, const int64_t* row, const int32_t* col,
                  int32_t start, int64_t* cc_ap);

/* Connected components: comp[N] (component index, by increasing smallest
 * vertex), returns the count.  size_out[N] (nullable) = size of each
 * vertex's component. */
int32_t orc_components(int32_t N, const int64_t* row, const int32_t* col,
                       int32_t* comp, int32_t* size_out);

/* Seeded R-MAT graph (scale, edge factor, quadrant probabilities a, b, c),
 * symmetrised, without self-loops or repeated edges, rows ascending; with
 * permute, vertex ids are relabelled by a seeded shuffle.  Gives the same
 * arrays as libgbc's gbc_gen_rmat for the same arguments.  *row_out /
 * *col_out are malloc'd (orc_free). */
int orc_gen_rmat(int32_t scale, int32_t ef, double a, double b, double c, uint64_t seed, int permute, int nthreads,
                 int32_t* n_out, int64_t** row_out, int32_t** col_out);

#ifdef __cplusplus
}
#endif
#endif
