/*
 * gbc_compat.h -- drop-in replacement for the XPPGX/BC C host API over
 * struct CSR, backed by libgbc's CUDA engines.
 *
 * The structs below have the same field order and types as the reference's
 * (Lib/CSR/CSR.h:34-95, Lib/AdjList/AdjList.h:37-50, Lib/qQueue/qQueue.h,
 * Lib/vVector/vVector.h, Lib/AP_Process/AP_Process.h:36-39), so a reference
 * driver compiled against this header and linked with -lgbc (instead of the
 * reference's Lib/, Seq_Brandes/ and Seq_CC/ objects) runs unchanged.
 *
 * Differences from the reference, all deliberate:
 *   - computeBC starts at csr->startNodeID (the reference starts at a global
 *     nextBFS = 0, which reads csrE[-1] for 1-based graphs; Brandes.c:24,249).
 *   - Betweenness is computed in FP64 and added to the caller's float array;
 *     path counts are exact (uint64, or a wide-exponent float when they overflow) instead
 *     of FP32 (Brandes.c:226).
 *   - computeCC returns the CCs pointer (the reference returns a freed
 *     buffer, CC.cpp:113-116).
 *   - The D1+AP closeness recovers folded vertices with the size of their
 *     connected component, so it is also right on disconnected graphs (the
 *     reference uses csr->totalNodeNumber, CC.cpp:2044).
 *   - Sums are computed in int64 and stored into the reference's int arrays.
 */
#ifndef GBC_COMPAT_H
#define GBC_COMPAT_H

#ifdef __cplusplus
extern "C" {
#endif

#define Ordinary  0x00000001U
#define D1        0x00000002U
#define D1Hub     0x00000004U
#define OriginAP  0x00000008U
#define ClonedAP  0x00000010U

struct vVector {     /* Lib/vVector/vVector.h */
    int* dataArr;
    int tail;
    int size;
};

struct qQueue {      /* Lib/qQueue/qQueue.h */
    int* dataArr;
    int front;
    int rear;
    int size;
};

struct adjList {     /* Lib/AdjList/AdjList.h:33-35 */
    struct vVector* neighbors;
};

struct Edge {        /* Lib/AdjList/AdjList.h:47-50 */
    int node1;
    int node2;
};

struct Graph {       /* Lib/AdjList/AdjList.h:37-45 */
    int nodeNum;
    int edgeNum;
    int startAtZero;
    int* nodeDegrees;
    struct adjList* vertices;
    struct qQueue* degreeOneQueue;
    struct Edge* edges;
};

struct newID_info {  /* Lib/AP_Process/AP_Process.h:36-39 */
    int ff;
    int w;
};

struct CSR {         /* Lib/CSR/CSR.h:34-95, same order and types */
    int* csrV;
    int* csrE;
    int csrVSize;
    int csrESize;
    int* csrNodesDegree;

    int* oriCsrV;
    int* oriCsrNodesDegree;

    unsigned int* nodesType;

    int* representNode;
    int* ff;

    struct qQueue* degreeOneNodesQ;
    int* notD1Node;
    int* D1Parent;
    int foldedDegreeOneCount;
    int hubNodeCount;
    int ordinaryNodeCount;

    int startAtZero;
    int maxDegree;

    int startNodeID;
    int endNodeID;
    int totalNodeNumber;

    int* low;
    int* depth_level;
    int* Dfs_sequence;
    int ap_count;
    int* AP_List;
    int* AP_component_number;
    int* compID;
    int* apCloneTrackOriAp_ID;
    int apCloneCount;
    int compNum;
    int maxCompSize_afterSplit;

    int* aliveNode;
    int aliveNodeCount;
    int* aliveNodeFlags;

    int* comp_NodesID_CsrData;
    int* comp_CsrOffset;
    int* nodesCompID;

    int* mapNodeID_New_to_Old;
    int* mapNodeID_Old_to_new;
    int* orderedCsrV;
    int* orderedCsrE;
    int newEndID;
    int* comp_newNodesID_CsrData;
    int* comp_newCsrOffset;
    int* newNodesCompID;
    int compEndID;

    float* BCs;
    int* CCs;
};

/* Ingest (Lib/AdjList/AdjList.c:13 buildGraph, Lib/CSR/CSR.c:9 createCSR).
 * Same text format, ID conventions and array layouts; neighbour lists are
 * ordered by neighbour degree ascending (ties in file order).  Exits with a
 * message on an unreadable file, as the reference does. */
struct Graph* buildGraph(char* datasetPath);
struct CSR* createCSR(struct Graph* adjlist);

/* Brandes betweenness of every source in [startNodeID, endNodeID]
 * (Seq_Brandes/Brandes.c:224), reference semantics: delta_s(w) added once per
 * shortest-path predecessor of w.  Adds into BCs[csrVSize].  Adjacency of v
 * is csrE[csrV[v] .. csrV[v+1]) as in the reference. */
void computeBC(struct CSR* csr, float* BCs);

/* Shared-traversal betweenness (Seq_Brandes/Brandes.c:374
 * computeBC_shareBased): same sums as computeBC.  The sources are scheduled
 * as the reference pairs them (each source followed by its first not-done
 * neighbour of degree != 1), and the device's lane batches, which run many
 * sources over one traversal of each row, stand in for its two-source
 * derivation. */
void computeBC_shareBased(struct CSR* csr, float* BCs);

/* Closeness distance sums of every source in [startNodeID, endNodeID]
 * (Seq_CC/CC.cpp:37): CCs[s] += sum of distances.  Adjacency of v is
 * csrE[csrV[v] .. oriCsrV[v+1]) as in the reference. Returns CCs. */
int* computeCC(struct CSR* csr, int* CCs);

/* Shared-BFS closeness (Seq_CC/CC.cpp:122): same sums as computeCC; the
 * batched lanes of the device engine stand in for the 32-neighbour sharing. */
void computeCC_shareBased(struct CSR* csr, int* CCs);

/* D1-folded closeness (Seq_CC/CC.cpp:418 compute_D1_CC): runs D1Folding on
 * the struct first, as the reference does, then adds to CCs[s] of every
 * unfolded vertex s the weighted distance sum ff[s] + sum over the other
 * reached unfolded v of (ff[v] + d(s,v) * representNode[v]) over the live
 * ranges, on the device; then sets the folded vertices in reverse folding
 * order: CCs[d1] = CCs[parent] + N - 2 * representNode[d1].  N is the vertex
 * count of d1's connected component; the reference uses totalNodeNumber,
 * which is wrong on disconnected graphs. */
void compute_D1_CC(struct CSR* csr, int* CCs);

/* Release path (Seq_CC/CC.cpp:1728): D1 folding + articulation-point
 * splitting, then closeness of every vertex into CCs.  Also sets the
 * structural fields foldedDegreeOneCount, hubNodeCount, ordinaryNodeCount,
 * ap_count, compNum (blocks) and maxCompSize_afterSplit (largest block). */
void compute_D1_AP_CC_shareBased_DegreeOrder(struct CSR* csr, int* CCs);

/* Reductions on the struct (Lib/D1Process/D1Process.c:5,
 * Lib/AP_Process/AP_Process.c:6): D1Folding fills representNode, ff,
 * D1Parent, nodesType, notD1Node and the counts, moves each folded vertex
 * to the front of its parent's live range and advances csrV[parent].
 * AP_detection fills AP_List, ap_count and OriginAP bits of nodesType (and
 * low / depth_level / Dfs_sequence of its own DFS). */
void D1Folding(struct CSR* csr);
void AP_detection(struct CSR* csr);

/* The reference's GPU programs' entry points (GPU_FAN/gpu_fan.cu:59,
 * GPU_VP/gpu_vp.cu:111, parallel_CC/para_CC.cu:61): closeness of every
 * vertex into csr->CCs by the plain engine, the lane engine, and the
 * D1+block reduction respectively. */
void gpu_fan(struct Graph* graph, struct CSR* csr);
void gpu_vb(struct CSR* csr);
void preprocess_then_parallel_sharedBased_DegreeOrder(struct CSR* csr);

#ifdef __cplusplus
}
#endif
#endif
