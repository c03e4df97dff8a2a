/*
 * dropin_driver.c -- a C caller of the struct-CSR drop-in API, built with
 * gcc against include/gbc_compat.h and linked with -lgbc, the way a reference
 * driver switches over (Lib/AdjList/AdjList.c:13 buildGraph, Lib/CSR/CSR.c:9
 * createCSR, Seq_Brandes/Brandes.c:224 computeBC, Seq_CC/CC.cpp:37 computeCC,
 * Seq_CC/CC.cpp:1728 compute_D1_AP_CC_shareBased_DegreeOrder).
 *
 * usage: dropin_driver <edge list> <out prefix>
 * writes <prefix>_bc.txt (a "start end" header, then one value per vertex, as
 * the reference's BC score files), <prefix>_cc.txt and <prefix>_d1ap.txt
 * (one closeness sum per vertex), and prints the reduction's counts.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbc_compat.h"

static int write_ints(const char* path, const int* v, int start, int end) {
    FILE* f = fopen(path, "w");
    if (!f) return 1;
    for (int i = start; i <= end; i++) fprintf(f, "%d\n", v[i]);
    fclose(f);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <edge list> <out prefix>\n", argv[0]);
        return 2;
    }
    char path[4096];
    struct Graph* g = buildGraph(argv[1]);
    struct CSR* csr = createCSR(g);
    const int vs = csr->csrVSize;

    float* bc = (float*)calloc((size_t)vs, sizeof(float));
    computeBC(csr, bc);
    snprintf(path, sizeof path, "%s_bc.txt", argv[2]);
    FILE* f = fopen(path, "w");
    if (!f) return 1;
    fprintf(f, "%d %d\n", csr->startNodeID, csr->endNodeID);
    for (int v = csr->startNodeID; v <= csr->endNodeID; v++) fprintf(f, "%f\n", bc[v]);
    fclose(f);

    int* cc = (int*)calloc((size_t)vs, sizeof(int));
    computeCC(csr, cc);
    snprintf(path, sizeof path, "%s_cc.txt", argv[2]);
    if (write_ints(path, cc, csr->startNodeID, csr->endNodeID)) return 1;

    /* the release path on a fresh struct: it folds and splits the graph */
    struct CSR* csr2 = createCSR(buildGraph(argv[1]));
    int* d1ap = (int*)calloc(2 * (size_t)vs, sizeof(int));
    compute_D1_AP_CC_shareBased_DegreeOrder(csr2, d1ap);
    snprintf(path, sizeof path, "%s_d1ap.txt", argv[2]);
    if (write_ints(path, d1ap, csr2->startNodeID, csr2->endNodeID)) return 1;
    printf("folded %d hubs %d aps %d\n", csr2->foldedDegreeOneCount, csr2->hubNodeCount, csr2->ap_count);
    free(bc);
    free(cc);
    free(d1ap);
    return 0;
}
