// Device-side graph ingest: an edge list (u[i], v[i]) over n vertices becomes
// the symmetric, deduplicated CSR without self-loops that the engines use,
// built on the GPU.  It replaces the reference's host ingest
// (Lib/AdjList/AdjList.c:13-150 per-vertex vector appends, then
// Lib/CSR/CSR.c:9-108), whose cost grows with the text parse and per-vertex
// reallocations.
//
// Every edge becomes two 64-bit keys u<<32|v and v<<32|u (a self-loop becomes
// n<<32, past every real key).  One radix sort over the bits the ids need puts
// each row's neighbours in ascending order; a unique pass drops repeats; the
// row offsets are written by one thread per kept key, each filling the offsets
// of the rows between the previous key's row and its own.  Rows come out in
// ascending neighbour order, as the host builder (csr_from_edges) makes them.
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include "engine.h"

namespace gbc {

namespace {

// ids in [0, n): else record the smallest bad edge index
__global__ void ingest_keys_kernel(const int32_t* __restrict__ u, const int32_t* __restrict__ v, int64_t m, int32_t n,
                                   uint64_t* __restrict__ keys, unsigned long long* __restrict__ bad) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = u[i], b = v[i];
        if ((uint32_t)a >= (uint32_t)n || (uint32_t)b >= (uint32_t)n) {
            atomicMin(bad, (unsigned long long)i);
            keys[2 * i] = keys[2 * i + 1] = (uint64_t)n << 32;
            continue;
        }
        if (a == b) {
            keys[2 * i] = keys[2 * i + 1] = (uint64_t)n << 32;
        } else {
            keys[2 * i] = ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
            keys[2 * i + 1] = ((uint64_t)(uint32_t)b << 32) | (uint32_t)a;
        }
    }
}

// col[i] = low half of key i; row[w] = first key index of row w (row[n] = M).
__global__ void ingest_csr_kernel(const uint64_t* __restrict__ uk, int64_t M, int32_t n, int64_t* __restrict__ row,
                                  int32_t* __restrict__ col) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= M; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ui = i < M ? (int64_t)(uk[i] >> 32) : (int64_t)n;
        const int64_t up = i > 0 ? (int64_t)(uk[i - 1] >> 32) : -1;
        for (int64_t w = up + 1; w <= ui; w++) row[w] = i;
        if (i < M) col[i] = (int32_t)(uint32_t)uk[i];
    }
}

}  // namespace

gbc_status csr_from_edges_device(const int32_t* d_u, const int32_t* d_v, int64_t m, int32_t n, cudaStream_t s,
                                 int64_t** d_row_out, int32_t** d_col_out, int64_t* M_out) {
    *d_row_out = nullptr;
    *d_col_out = nullptr;
    *M_out = 0;
    const int64_t K = 2 * m;
    uint64_t *k0 = nullptr, *k1 = nullptr;
    unsigned long long* d_bad = nullptr;
    int64_t* d_nsel = nullptr;
    void* tmp = nullptr;
    int64_t* d_row = nullptr;
    int32_t* d_col = nullptr;
    auto cleanup = [&]() {
        cudaFree(k0); cudaFree(k1); cudaFree(d_bad); cudaFree(d_nsel); cudaFree(tmp);
    };
    auto fail = [&](gbc_status st) {
        cleanup();
        cudaFree(d_row);
        cudaFree(d_col);
        return st;
    };
    if (cudaMalloc(&k0, sizeof(uint64_t) * std::max<int64_t>(K, 1)) != cudaSuccess ||
        cudaMalloc(&k1, sizeof(uint64_t) * std::max<int64_t>(K, 1)) != cudaSuccess ||
        cudaMalloc(&d_bad, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&d_nsel, sizeof(int64_t)) != cudaSuccess) {
        cudaGetLastError();
        set_error("ingest buffers for %lld edges", (long long)m);
        return fail(GBC_ERR_NOMEM);
    }
    const unsigned long long none = ~0ULL;
    if (cudaMemcpyAsync(d_bad, &none, sizeof none, cudaMemcpyHostToDevice, s) != cudaSuccess) return fail(GBC_ERR_CUDA);
    int dev = 0, sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    if (m > 0) ingest_keys_kernel<<<sm * 8, 256, 0, s>>>(d_u, d_v, m, n, k0, d_bad);
    // sort on the bits the keys use: row ids up to n (self-loops) above 32 bits
    int bits = 1;
    while (bits < 31 && ((int64_t)1 << bits) <= (int64_t)n) bits++;
    const int end_bit = 32 + bits;
    size_t tb_sort = 0, tb_uniq = 0;
    cub::DoubleBuffer<uint64_t> db(k0, k1);
    if (cub::DeviceRadixSort::SortKeys(nullptr, tb_sort, db, (int64_t)K, 0, end_bit, s) != cudaSuccess ||
        cub::DeviceSelect::Unique(nullptr, tb_uniq, k0, k1, d_nsel, (int64_t)K, s) != cudaSuccess) {
        cudaGetLastError();
        set_error("ingest: sort setup failed");
        return fail(GBC_ERR_CUDA);
    }
    if (cudaMalloc(&tmp, std::max(tb_sort, tb_uniq) + 16) != cudaSuccess) {
        cudaGetLastError();
        set_error("ingest sort workspace");
        return fail(GBC_ERR_NOMEM);
    }
    if (K > 0 && cub::DeviceRadixSort::SortKeys(tmp, tb_sort, db, (int64_t)K, 0, end_bit, s) != cudaSuccess) {
        cudaGetLastError();
        set_error("ingest: radix sort failed");
        return fail(GBC_ERR_CUDA);
    }
    uint64_t* sorted = db.Current();
    uint64_t* uniq = db.Alternate();
    int64_t nsel = 0;
    if (K > 0) {
        if (cub::DeviceSelect::Unique(tmp, tb_uniq, sorted, uniq, d_nsel, (int64_t)K, s) != cudaSuccess) {
            cudaGetLastError();
            set_error("ingest: unique failed");
            return fail(GBC_ERR_CUDA);
        }
        if (cudaMemcpyAsync(&nsel, d_nsel, sizeof nsel, cudaMemcpyDeviceToHost, s) != cudaSuccess) return fail(GBC_ERR_CUDA);
    }
    unsigned long long bad = none;
    if (cudaMemcpyAsync(&bad, d_bad, sizeof bad, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        set_error("ingest: device error");
        return fail(GBC_ERR_CUDA);
    }
    if (bad != none) {
        set_error("edge %llu has a vertex id outside [0,%d)", bad, n);
        return fail(GBC_ERR_ARG);
    }
    // the self-loop key, if any, is the last unique key
    int64_t M = nsel;
    if (M > 0) {
        uint64_t last = 0;
        if (cudaMemcpy(&last, uniq + (M - 1), sizeof last, cudaMemcpyDeviceToHost) != cudaSuccess) return fail(GBC_ERR_CUDA);
        if ((int64_t)(last >> 32) == (int64_t)n) M--;
    }
    if (M >= ((int64_t)1 << 31)) {
        set_error("more than 2^31-1 directed edges after symmetrisation (%lld)", (long long)M);
        return fail(GBC_ERR_ARG);
    }
    if (cudaMalloc(&d_row, sizeof(int64_t) * ((size_t)n + 1)) != cudaSuccess ||
        cudaMalloc(&d_col, sizeof(int32_t) * std::max<int64_t>(M, 1)) != cudaSuccess) {
        cudaGetLastError();
        set_error("CSR allocation");
        return fail(GBC_ERR_NOMEM);
    }
    ingest_csr_kernel<<<sm * 8, 256, 0, s>>>(uniq, M, n, d_row, d_col);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        set_error("ingest: CSR kernel failed");
        return fail(GBC_ERR_CUDA);
    }
    cleanup();
    *d_row_out = d_row;
    *d_col_out = d_col;
    *M_out = M;
    return GBC_OK;
}

}  // namespace gbc
