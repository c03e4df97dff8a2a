// Drop-in implementation of the XPPGX/BC C host API over struct CSR
// (include/gbc_compat.h) on top of the native C ABI (include/gbc.h).
// Fatal conditions print a message and exit(1), the reference's only error
// convention (Lib/AdjList/AdjList.c:17-20), since these entry points return
// void.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/gbc.h"
#include "../../include/gbc_compat.h"
#include "gbc_internal.h"

namespace {

[[noreturn]] void die(const char* where, gbc_status st) {
    fprintf(stderr, "[gbc] %s failed: status %d: %s\n", where, (int)st, gbc_last_error());
    exit(1);
}

void ok(gbc_status st, const char* where) {
    if (st != GBC_OK) die(where, st);
}

// Adjacency of slot v is csrE[csrV[v] .. hi(v)), hi = oriCsrV[v+1] (live
// range after folding) or csrV[v+1]; slots below startNodeID are empty.
void to_native(const struct CSR* c, bool live, std::vector<int64_t>& row, std::vector<int32_t>& col) {
    const int32_t N = c->csrVSize - 1;
    row.assign(N + 1, 0);
    col.clear();
    col.reserve(c->csrESize > 0 ? c->csrESize : 0);
    for (int32_t v = 0; v < N; v++) {
        if (v >= c->startNodeID && v <= c->endNodeID) {
            const int lo = c->csrV[v];
            const int hi = (live && c->oriCsrV) ? c->oriCsrV[v + 1] : c->csrV[v + 1];
            if (lo < 0 || hi < lo) {
                fprintf(stderr, "[gbc] malformed struct CSR at vertex %d\n", v);
                exit(1);
            }
            for (int e = lo; e < hi; e++) col.push_back(c->csrE[e]);
        }
        row[v + 1] = (int64_t)col.size();
    }
}

std::vector<int32_t> source_range(const struct CSR* c) {
    std::vector<int32_t> s;
    for (int v = c->startNodeID; v <= c->endNodeID; v++) s.push_back(v);
    return s;
}

void closeness_into(const struct CSR* c, bool live, int engine, int* CCs, bool add) {
    std::vector<int64_t> row;
    std::vector<int32_t> col;
    to_native(c, live, row, col);
    gbc_graph g = nullptr;
    ok(gbc_graph_create(row.data(), col.data(), c->csrVSize - 1, &g), "gbc_graph_create");
    std::vector<int32_t> src = source_range(c);
    std::vector<int64_t> cc(src.size());
    gbc_options o;
    gbc_options_default(&o);
    o.engine = engine;
    if (!src.empty()) ok(gbc_cc(g, src.data(), (int32_t)src.size(), &o, cc.data()), "gbc_cc");
    gbc_graph_destroy(g);
    for (size_t i = 0; i < src.size(); i++) {
        if (add) CCs[src[i]] += (int)cc[i];
        else CCs[src[i]] = (int)cc[i];
    }
}

void reduced_closeness_into(struct CSR* c, int* CCs) {
    std::vector<int64_t> row;
    std::vector<int32_t> col;
    to_native(c, true, row, col);
    gbc_reduced r = nullptr;
    ok(gbc_reduce(row.data(), col.data(), c->csrVSize - 1, c->startNodeID, &r), "gbc_reduce");
    std::vector<int64_t> cc(c->csrVSize - 1);
    ok(gbc_cc_reduced(r, nullptr, cc.data()), "gbc_cc_reduced");
    gbc_reduced_info info;
    gbc_reduced_info_get(r, &info);
    gbc_reduced_destroy(r);
    for (int v = c->startNodeID; v <= c->endNodeID; v++) CCs[v] = (int)cc[v];
    c->foldedDegreeOneCount = info.d1_folded;
    c->hubNodeCount = info.d1_hubs;
    c->ordinaryNodeCount = info.alive;
    c->ap_count = info.articulation_points;
    c->compNum = info.blocks;
    c->maxCompSize_afterSplit = info.max_block;
}

struct vVector* new_vec(int cap) {
    struct vVector* v = (struct vVector*)malloc(sizeof(struct vVector));
    v->size = cap < 5 ? 5 : cap;
    v->dataArr = (int*)malloc(sizeof(int) * v->size);
    v->tail = -1;
    return v;
}

// Reference-semantics betweenness of the sources in `src`, added into BCs.
void betweenness_into(struct CSR* c, const std::vector<int32_t>& src, float* BCs) {
    std::vector<int64_t> row;
    std::vector<int32_t> col;
    to_native(c, false, row, col);
    gbc_graph g = nullptr;
    ok(gbc_graph_create(row.data(), col.data(), c->csrVSize - 1, &g), "gbc_graph_create");
    std::vector<double> bc(c->csrVSize - 1, 0.0);
    gbc_options o;
    gbc_options_default(&o);
    o.semantics = GBC_BC_REFERENCE;
    o.delta_precision = GBC_DELTA_F64;
    if (!src.empty()) ok(gbc_bc(g, src.data(), (int32_t)src.size(), &o, bc.data()), "gbc_bc");
    gbc_graph_destroy(g);
    for (int v = 0; v < c->csrVSize - 1; v++) BCs[v] += (float)bc[v];
}

// The source schedule of Seq_Brandes/Brandes.c:417-475 (computeBC_shareBased):
// sources in id order, each not-yet-done source s followed by its first
// not-done neighbour of degree != 1 in csrE[csrV[s] .. csrV[s+1]), which the
// reference derives from s's traversal.  Every vertex of the range appears
// once, so the sums equal computeBC's.
std::vector<int32_t> shared_pair_order(const struct CSR* c) {
    std::vector<int32_t> order;
    std::vector<char> done(c->csrVSize, 0);
    for (int s = c->startNodeID; s <= c->endNodeID; s++) {
        if (done[s]) continue;
        done[s] = 1;
        order.push_back(s);
        for (int e = c->csrV[s]; e < c->csrV[s + 1]; e++) {
            const int t = c->csrE[e];
            if (t < c->startNodeID || t > c->endNodeID || done[t]) continue;
            const int deg = c->csrNodesDegree ? c->csrNodesDegree[t] : c->csrV[t + 1] - c->csrV[t];
            if (deg != 1) {
                done[t] = 1;
                order.push_back(t);
                break;
            }
        }
    }
    return order;
}

}  // namespace

extern "C" {

struct Graph* buildGraph(char* path) {
    FILE* f = fopen(path, "r");
    if (!f) {
        printf("Error: Open file\n");
        exit(1);
    }
    char line[2000];
    long n = 0, m = 0;
    if (!fgets(line, sizeof line, f) || sscanf(line, "%ld %ld", &n, &m) != 2 || n <= 0 || m < 0) {
        printf("Error: bad header in %s\n", path);
        exit(1);
    }
    struct Graph* g = (struct Graph*)calloc(1, sizeof(struct Graph));
    g->nodeNum = (int)n;
    g->edgeNum = (int)m;
    g->edges = (struct Edge*)malloc(sizeof(struct Edge) * (m ? m : 1));
    bool zero = false;
    long got = 0;
    while (got < m && fgets(line, sizeof line, f)) {
        int a, b;
        if (sscanf(line, "%d %d", &a, &b) != 2) continue;
        g->edges[got].node1 = a;
        g->edges[got].node2 = b;
        zero |= (a == 0 || b == 0);
        got++;
    }
    fclose(f);
    if (got != m) {
        printf("Error: %s has %ld of %ld edges\n", path, got, m);
        exit(1);
    }
    g->startAtZero = zero ? 1 : 0;
    const int slots = zero ? (int)n : (int)n + 1;
    g->nodeDegrees = (int*)calloc(slots, sizeof(int));
    for (long i = 0; i < m; i++) {
        const int a = g->edges[i].node1, b = g->edges[i].node2;
        if (a < 0 || a >= slots || b < 0 || b >= slots) {
            printf("Error: vertex id out of range in %s\n", path);
            exit(1);
        }
        g->nodeDegrees[a]++;
        g->nodeDegrees[b]++;
    }
    g->vertices = (struct adjList*)malloc(sizeof(struct adjList) * slots);
    for (int v = 0; v < slots; v++) g->vertices[v].neighbors = new_vec(g->nodeDegrees[v]);
    for (long i = 0; i < m; i++) {
        const int a = g->edges[i].node1, b = g->edges[i].node2;
        struct vVector* va = g->vertices[a].neighbors;
        va->dataArr[++va->tail] = b;
        struct vVector* vb = g->vertices[b].neighbors;
        vb->dataArr[++vb->tail] = a;
    }
    g->degreeOneQueue = (struct qQueue*)malloc(sizeof(struct qQueue));
    g->degreeOneQueue->size = (int)n;
    g->degreeOneQueue->dataArr = (int*)malloc(sizeof(int) * (n ? n : 1));
    g->degreeOneQueue->front = 0;
    g->degreeOneQueue->rear = -1;
    const int* deg = g->nodeDegrees;
    for (int v = zero ? 0 : 1; v < slots; v++) {
        struct vVector* nb = g->vertices[v].neighbors;
        if (deg[v] == 1) {
            g->degreeOneQueue->dataArr[++g->degreeOneQueue->rear] = v;
        } else {
            std::stable_sort(nb->dataArr, nb->dataArr + nb->tail + 1, [deg](int x, int y) { return deg[x] < deg[y]; });
        }
    }
    return g;
}

struct CSR* createCSR(struct Graph* g) {
    const int zero = g->startAtZero;
    const int temp = zero ? g->nodeNum + 1 : g->nodeNum + 2;   // CSR.c:16-27
    struct CSR* c = (struct CSR*)calloc(1, sizeof(struct CSR));
    c->csrV = (int*)malloc(sizeof(int) * 2 * temp);
    c->csrE = (int*)malloc(sizeof(int) * (g->edgeNum ? 4 * (size_t)g->edgeNum : 1));
    int v = zero ? 0 : 1;
    if (!zero) c->csrV[0] = -1;
    int idx = 0, maxdeg = 0;
    for (; v < temp - 1; v++) {
        c->csrV[v] = idx;
        struct vVector* nb = g->vertices[v].neighbors;
        for (int i = 0; i <= nb->tail; i++) c->csrE[idx++] = nb->dataArr[i];
        maxdeg = std::max(maxdeg, nb->tail + 1);
    }
    c->csrV[v] = 2 * g->edgeNum;
    c->csrVSize = temp;
    c->csrESize = 2 * g->edgeNum;
    c->csrNodesDegree = g->nodeDegrees;
    c->maxDegree = maxdeg;
    c->oriCsrNodesDegree = (int*)malloc(sizeof(int) * temp);
    std::memcpy(c->oriCsrNodesDegree, c->csrNodesDegree, sizeof(int) * (temp - (zero ? 1 : 1)));
    c->oriCsrNodesDegree[temp - 1] = 0;
    c->oriCsrV = (int*)malloc(sizeof(int) * 2 * temp);
    std::memcpy(c->oriCsrV, c->csrV, sizeof(int) * temp);
    c->nodesType = (unsigned int*)calloc(2 * (size_t)temp, sizeof(unsigned int));
    c->CCs = (int*)calloc(2 * (size_t)temp, sizeof(int));
    c->startAtZero = zero;
    c->totalNodeNumber = zero ? temp - 1 : temp - 2;
    c->startNodeID = !zero;
    c->endNodeID = c->totalNodeNumber - zero;
    c->degreeOneNodesQ = g->degreeOneQueue;
    c->foldedDegreeOneCount = 0;
    return c;
}

void computeBC(struct CSR* c, float* BCs) { betweenness_into(c, source_range(c), BCs); }

void computeBC_shareBased(struct CSR* c, float* BCs) { betweenness_into(c, shared_pair_order(c), BCs); }

int* computeCC(struct CSR* c, int* CCs) {
    closeness_into(c, true, GBC_ENGINE_LANES, CCs, true);
    return CCs;
}

void computeCC_shareBased(struct CSR* c, int* CCs) { closeness_into(c, true, GBC_ENGINE_LANES, CCs, true); }

void compute_D1_CC(struct CSR* c, int* CCs) {
    D1Folding(c);
    const int32_t N = c->csrVSize - 1;
    // live ranges of the unfolded vertices (folded neighbours sit before csrV[v]); folded vertices get empty rows
    std::vector<int64_t> row(N + 1, 0);
    std::vector<int32_t> col;
    std::vector<int32_t> w(N, 1);
    std::vector<int64_t> ff(N, 0);
    col.reserve(c->csrESize > 0 ? c->csrESize : 0);
    for (int32_t v = 0; v < N; v++) {
        if (v >= c->startNodeID && v <= c->endNodeID && c->nodesType[v] != D1) {
            for (int e = c->csrV[v]; e < c->oriCsrV[v + 1]; e++) col.push_back(c->csrE[e]);
            w[v] = c->representNode[v];
            ff[v] = c->ff[v];
        }
        row[v + 1] = (int64_t)col.size();
    }
    std::vector<int32_t> src(c->notD1Node, c->notD1Node + c->ordinaryNodeCount);
    gbc_graph g = nullptr;
    ok(gbc_graph_create(row.data(), col.data(), N, &g), "gbc_graph_create");
    ok(gbc_graph_set_weights(g, w.data(), ff.data()), "gbc_graph_set_weights");
    std::vector<int64_t> cc(src.size());
    gbc_options o;
    gbc_options_default(&o);
    if (!src.empty()) ok(gbc_cc(g, src.data(), (int32_t)src.size(), &o, cc.data()), "gbc_cc");
    gbc_graph_destroy(g);
    for (size_t i = 0; i < src.size(); i++) CCs[src[i]] += (int)cc[i];
    // vertex count of every connected component, over the original rows
    std::vector<int32_t> parent(N);
    for (int32_t v = 0; v < N; v++) parent[v] = v;
    auto find = [&](int32_t x) {
        while (parent[x] != x) x = parent[x] = parent[parent[x]];
        return x;
    };
    for (int32_t v = c->startNodeID; v <= c->endNodeID; v++)
        for (int e = c->oriCsrV[v]; e < c->oriCsrV[v + 1]; e++) {
            const int32_t a = find(v), b = find(c->csrE[e]);
            if (a != b) parent[std::max(a, b)] = std::min(a, b);
        }
    std::vector<int32_t> size(N, 0);
    for (int32_t v = c->startNodeID; v <= c->endNodeID; v++) size[find(v)]++;
    const struct qQueue* q = c->degreeOneNodesQ;
    for (int i = q->rear; i >= 0; i--) {
        const int d1 = q->dataArr[i];
        CCs[d1] = CCs[c->D1Parent[d1]] + size[find(d1)] - 2 * c->representNode[d1];
    }
}

void compute_D1_AP_CC_shareBased_DegreeOrder(struct CSR* c, int* CCs) { reduced_closeness_into(c, CCs); }

void gpu_fan(struct Graph* g, struct CSR* c) {
    (void)g;
    closeness_into(c, false, GBC_ENGINE_PLAIN, c->CCs, false);
}

void gpu_vb(struct CSR* c) { closeness_into(c, false, GBC_ENGINE_LANES, c->CCs, false); }

void preprocess_then_parallel_sharedBased_DegreeOrder(struct CSR* c) { reduced_closeness_into(c, c->CCs); }

// Degree-1 folding on the struct (Lib/D1Process/D1Process.c:5-154).
void D1Folding(struct CSR* c) {
    const int vs = c->csrVSize;
    c->hubNodeCount = 0;
    c->ordinaryNodeCount = 0;
    c->foldedDegreeOneCount = 0;
    c->representNode = (int*)malloc(sizeof(int) * 2 * (size_t)vs);
    for (int i = 0; i < 2 * vs; i++) c->representNode[i] = 1;
    c->ff = (int*)calloc(2 * (size_t)vs, sizeof(int));
    c->D1Parent = (int*)malloc(sizeof(int) * vs);
    for (int i = 0; i < vs; i++) c->D1Parent[i] = -1;
    if (!c->oriCsrV) {
        c->oriCsrV = (int*)malloc(sizeof(int) * 2 * (size_t)vs);
        std::memcpy(c->oriCsrV, c->csrV, sizeof(int) * vs);
    }
    std::vector<int> deg(vs, 0);
    for (int v = c->startNodeID; v <= c->endNodeID; v++) deg[v] = c->oriCsrV[v + 1] - c->csrV[v];
    struct qQueue* q = c->degreeOneNodesQ;
    if (!q) {
        q = (struct qQueue*)malloc(sizeof(struct qQueue));
        q->size = vs;
        q->dataArr = (int*)malloc(sizeof(int) * vs);
        q->front = 0;
        q->rear = -1;
        for (int v = c->startNodeID; v <= c->endNodeID; v++) if (deg[v] == 1) q->dataArr[++q->rear] = v;
        c->degreeOneNodesQ = q;
    }
    // queue storage sized for every vertex (a folded parent can be pushed)
    if (q->size < vs) {
        int* d = (int*)malloc(sizeof(int) * vs);
        std::memcpy(d, q->dataArr, sizeof(int) * (q->rear + 1));
        free(q->dataArr);
        q->dataArr = d;
        q->size = vs;
    }
    while (q->front <= q->rear) {
        const int d1 = q->dataArr[q->front++];
        if (deg[d1] != 1) continue;   // root of a tree component: not folded
        c->nodesType[d1] = D1;
        const int p = c->csrE[c->csrV[d1]];
        c->D1Parent[d1] = p;
        c->nodesType[p] = D1Hub;
        c->representNode[p] += c->representNode[d1];
        c->ff[p] += c->representNode[d1] + c->ff[d1];
        for (int e = c->csrV[p]; e < c->oriCsrV[p + 1]; e++)
            if (c->csrE[e] == d1) { std::swap(c->csrE[e], c->csrE[c->csrV[p]]); break; }
        c->csrV[p]++;
        if (c->csrNodesDegree) c->csrNodesDegree[p]--;
        deg[d1] = 0;
        if (--deg[p] == 1) q->dataArr[++q->rear] = p;
        c->foldedDegreeOneCount++;
    }
    // keep the queue's full history readable for recovery in reverse order
    std::vector<int> order;
    order.reserve(q->rear + 1);
    for (int i = 0; i <= q->rear; i++) {
        const int v = q->dataArr[i];
        if (c->nodesType[v] == D1) order.push_back(v);
    }
    // each folded vertex appears once (popped when its degree was 1)
    std::vector<char> seen(vs, 0);
    int k = 0;
    for (int v : order) if (!seen[v]) { seen[v] = 1; q->dataArr[k++] = v; }
    q->front = 0;
    q->rear = k - 1;
    c->notD1Node = (int*)malloc(sizeof(int) * (c->endNodeID - c->startNodeID + 1 - c->foldedDegreeOneCount + 1));
    int idx = 0;
    for (int v = c->startNodeID; v <= c->endNodeID; v++) {
        if (c->nodesType[v] == D1) continue;
        if (c->nodesType[v] == D1Hub) c->hubNodeCount++;
        else c->nodesType[v] = Ordinary;
        c->notD1Node[idx++] = v;
        c->ordinaryNodeCount++;
    }
}

// Articulation points on the live ranges, D1 vertices skipped
// (Lib/AP_Process/AP_Process.c:6-225), by iterative Tarjan.
void AP_detection(struct CSR* c) {
    const int vs = c->csrVSize;
    c->AP_List = (int*)malloc(sizeof(int) * vs);
    c->AP_component_number = (int*)calloc(vs, sizeof(int));
    c->depth_level = (int*)calloc(vs, sizeof(int));
    c->low = (int*)calloc(vs, sizeof(int));
    c->Dfs_sequence = (int*)malloc(sizeof(int) * (vs + 1));
    for (int i = 0; i < vs; i++) c->AP_List[i] = -1;
    for (int i = 0; i <= vs; i++) c->Dfs_sequence[i] = -1;
    const int* hi = c->oriCsrV ? c->oriCsrV : c->csrV;
    std::vector<int> par(vs, -1), it(vs), nchild(vs, 0), stk;
    int timer = 0, count = 0;
    for (int r = c->startNodeID; r <= c->endNodeID; r++) {
        if ((c->nodesType[r] & D1) || c->depth_level[r]) continue;
        stk.assign(1, r);
        c->depth_level[r] = c->low[r] = ++timer;
        c->Dfs_sequence[timer] = r;
        it[r] = c->csrV[r];
        while (!stk.empty()) {
            const int v = stk.back();
            if (it[v] < hi[v + 1]) {
                const int u = c->csrE[it[v]++];
                if (!c->depth_level[u]) {
                    par[u] = v;
                    c->depth_level[u] = c->low[u] = ++timer;
                    c->Dfs_sequence[timer] = u;
                    it[u] = c->csrV[u];
                    nchild[v]++;
                    stk.push_back(u);
                } else if (u != par[v]) {
                    c->low[v] = std::min(c->low[v], c->depth_level[u]);
                }
            } else {
                stk.pop_back();
                const int p = par[v];
                if (p >= 0) {
                    c->low[p] = std::min(c->low[p], c->low[v]);
                    if (par[p] >= 0 && c->low[v] >= c->depth_level[p] && !(c->nodesType[p] & OriginAP)) {
                        c->nodesType[p] |= OriginAP;
                        c->AP_List[count++] = p;
                    }
                }
            }
        }
        if (nchild[r] > 1 && !(c->nodesType[r] & OriginAP)) {
            c->nodesType[r] |= OriginAP;
            c->AP_List[count++] = r;
        }
    }
    c->ap_count = count;
}

}  // extern "C"
