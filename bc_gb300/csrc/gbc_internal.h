// Internal declarations shared by the libgbc translation units.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/gbc.h"

namespace gbc {

// Thread-local error message behind gbc_last_error().
void set_error(const char* fmt, ...);
const char* last_error();

// Host CSR: row[n+1] int64, col[row[n]] int32.
struct HostCSR {
    int32_t n = 0;
    std::vector<int64_t> row;
    std::vector<int32_t> col;
    int64_t m() const { return row.empty() ? 0 : row.back(); }
};

// Validate a caller-provided CSR (offsets monotone, ids in range).
gbc_status validate_csr(const int64_t* row, const int32_t* col, int32_t n);

// The O(1) part of validate_csr: arguments, row[0] == 0 and 0 <= row[n] < 2^31
// (for a row[n] outside that range it runs the full check, so the message is
// the one validate_csr gives).  The per-entry checks then run on the device.
gbc_status validate_csr_header(const int64_t* row, const int32_t* col, int32_t n);

// Build a symmetric, deduplicated CSR without self-loops from an edge list
// (u[i], v[i]) over n vertices; rows sorted by neighbour id. Multi-threaded.
void csr_from_edges(int32_t n, const std::vector<int32_t>& u, const std::vector<int32_t>& v, HostCSR& out);

// Connected components of a host CSR: comp[v] in [0, count), sizes[c].
int32_t components(const HostCSR& g, std::vector<int32_t>& comp, std::vector<int64_t>& sizes);

// Undirected edge count (row[n]/2) of every vertex's component, summed per
// source -- the GTEPS numerator.
int64_t edges_of_sources(const HostCSR& g, const std::vector<int32_t>& comp, const std::vector<int64_t>& comp_edges,
                         const int32_t* src, int32_t k);

// malloc'd copies for the C ABI.
gbc_status export_csr(const HostCSR& g, int64_t** row, int32_t** col);

// Deterministic RNG (splitmix64 seeding, xoshiro256** stream).
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed, uint64_t stream = 0);
    uint64_t next();
    double uniform();                     // [0,1)
    uint64_t below(uint64_t bound);       // [0,bound)
};

}  // namespace gbc
