/*
 * ref_bc_harness.c -- builds the reference's own sequential Brandes
 * (Seq_Brandes/Brandes.c, compiled in place from the reference tree via -I;
 * nothing is copied) into oracle/_ref/libref_bc.so for tests and CPU timing.
 * TEST INFRASTRUCTURE ONLY.
 *
 * ref_bc_file() applies the harness fix the reference needs: computeBC
 * starts at the global nextBFS (Seq_Brandes/Brandes.c:24,249), which must be
 * set to csr->startNodeID for 1-based graphs.
 */
#define main ref_brandes_main
#include "Seq_Brandes/Brandes.c"
#undef main

int ref_bc_file(const char* path, int s_begin, int s_end_inclusive, float* out,
                int out_len, int* vsize) {
    struct Graph* g = buildGraph((char*)path);
    struct CSR* csr = createCSR(g);
    *vsize = csr->csrVSize;
    if (out_len < csr->csrVSize) return -1;
    nextBFS = s_begin < 0 ? csr->startNodeID : s_begin;
    int saved_end = csr->endNodeID;
    if (s_end_inclusive >= 0) csr->endNodeID = s_end_inclusive;
    computeBC(csr, out);
    csr->endNodeID = saved_end;
    return 0;
}

/* The reference's shared-traversal variant (Seq_Brandes/Brandes.c:374
 * computeBC_shareBased): one forward BFS from a source s also yields the BFS
 * DAG of s's first not-done, non-leaf neighbour.  It loops from startNodeID
 * on its own (no nextBFS global). */
int ref_bc_shared_file(const char* path, float* out, int out_len, int* vsize) {
    struct Graph* g = buildGraph((char*)path);
    struct CSR* csr = createCSR(g);
    *vsize = csr->csrVSize;
    if (out_len < csr->csrVSize) return -1;
    computeBC_shareBased(csr, out);
    return 0;
}
