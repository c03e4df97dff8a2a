/*
 * ref_cc_harness.cpp -- builds the reference's own sequential closeness code
 * (Seq_CC/CC.cpp with the Lib_cpps objects, compiled in place from the
 * reference tree via -I; nothing is copied) into oracle/_ref/libref_cc.so.
 * TEST INFRASTRUCTURE ONLY.
 */
#define main ref_cc_main
#include "Seq_CC/CC.cpp"
#undef main

extern "C" int ref_cc_file(const char* path, int* out, int out_len, int* vsize) {
    struct Graph* g = buildGraph((char*)path);
    struct CSR* csr = createCSR(g);
    *vsize = csr->csrVSize;
    if (out_len < csr->csrVSize) return -1;
    memset(out, 0, sizeof(int) * csr->csrVSize);
    computeCC(csr, out);
    return 0;
}

/* stats[0..6] = D1 count, hub count, ordinary count, AP count, component
 * count, max component size, endNodeID after AP cloning. */
extern "C" int ref_d1ap_cc_file(const char* path, int* out, int out_len, int* vsize, int* stats) {
    struct Graph* g = buildGraph((char*)path);
    struct CSR* csr = createCSR(g);
    *vsize = csr->csrVSize;
    if (out_len < csr->csrVSize) return -1;
    compute_D1_AP_CC_shareBased_DegreeOrder(csr, csr->CCs);
    memcpy(out, csr->CCs, sizeof(int) * csr->csrVSize);
    stats[0] = csr->foldedDegreeOneCount;
    stats[1] = csr->hubNodeCount;
    stats[2] = csr->ordinaryNodeCount;
    stats[3] = csr->ap_count;
    stats[4] = csr->compNum;
    stats[5] = csr->maxCompSize_afterSplit;
    stats[6] = csr->endNodeID;
    return 0;
}
