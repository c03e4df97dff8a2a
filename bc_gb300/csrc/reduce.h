// The D1 folding + block split as the device computes it (reduce_dev.cu),
// handed to the host-side assembly of reduce.cu.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "gbc_internal.h"

namespace gbc {

struct FoldSplit {
    // folding (Lib/D1Process/D1Process.c:32-73), per vertex slot
    std::vector<int32_t> parent;      // vertex a folded vertex was folded into, -1
    std::vector<int32_t> fround;      // peeling round a vertex was folded in, -1 if it stays
    std::vector<int64_t> r, ff;       // reach and folded distance sums
    // the folded graph: alive vertices in id order ("core ids")
    std::vector<int32_t> core_v;      // core id -> vertex
    HostCSR core;                     // live adjacency in core ids
    std::vector<int32_t> core_comp;   // connected component, numbered by smallest member
    int32_t n_comp = 0;
    // biconnected blocks of the folded graph
    std::vector<uint8_t> core_ap;     // articulation points
    std::vector<int64_t> bvoff;       // block -> first slot
    std::vector<int32_t> slot_core;   // slot -> core id, ascending within a block
    std::vector<int32_t> core_vslot;  // core id -> its first slot
    HostCSR bg;                       // block graph over slots, rows ascending
    int32_t rounds = 0, levels = 0;   // peeling rounds, spanning-forest depth + 1
    // the folded graph and the block graph stay on the device (cudaMalloc'd,
    // owned by the receiver); core and bg above carry only their n
    int64_t* d_core_row = nullptr;
    int32_t* d_core_col = nullptr;
    int64_t core_m = 0;
    int64_t* d_bg_row = nullptr;
    int32_t* d_bg_col = nullptr;
    int64_t bg_m = 0;
};

// The per-entry checks of the reduction's input on the device copy: row
// offsets monotone, ids in [0, n), no self-loops (same messages as the host
// checks).  host_col, when given, supplies the offending value for a message.
gbc_status check_csr_device(const int64_t* d_row, const int32_t* d_col, int32_t n, int64_t M, const int32_t* host_col,
                            cudaStream_t s);

// Fold and split a device CSR (vertex slots [start, n) are real vertices).
// Everything proportional to n or to the edge count runs on the device; the
// result is copied to `out`.
gbc_status fold_split_device(const int64_t* d_row, const int32_t* d_col, int32_t n, int64_t M, int32_t start,
                             cudaStream_t s, FoldSplit& out);

}  // namespace gbc
