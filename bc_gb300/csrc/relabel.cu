// Degree relabelling of a device CSR: vertex ids are reassigned in order of
// descending degree -- ties broken by the degree rank of the vertex's
// highest-degree neighbour, so that the low-degree vertices hanging off one
// hub get consecutive ids, then by original id -- and every row is rewritten
// in the new ids, ascending.  The lane state is laid out by vertex id, so the
// rows of the high-degree vertices -- which most neighbour visits of a
// power-law graph land on -- become one dense region that stays in L2 instead
// of being scattered over gigabytes.  On R-MAT scale 22 this took batched BC
// from 78.9 to 98.8 GTEPS and closeness from 187 to 251 GTEPS with the same
// frontier work (the neighbour tie-break adds about 3%).  The caller keeps
// original ids: the library maps sources in and per-vertex results out
// (order[] / inv[]).
//
// Deep graphs of low degree (meshes, grids, road-like graphs: maximum degree
// at most 64, a BFS deeper than 32 levels) have no hubs to gather; there the
// ids follow a Cuthill-McKee order instead (relabel_graph): per component a
// BFS from a far vertex, so that a vertex's neighbours sit in the BFS levels
// next to its own and a BFS wavefront of one source walks along consecutive
// ids.  A lane's level / path-count row then shares its cache lines between
// neighbouring frontier entries: on the 1024^2 grid with 1024 one-lane tasks
// a batch took 181 + 149 ms (forward + sweep) against 207 + 192 ms in degree
// order, and the cache-line footprint of a level fits L2 better.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include <cub/cub.cuh>

#include "engine.h"

namespace gbc {

namespace {

__global__ void deg_iota_kernel(const int64_t* __restrict__ row, int32_t n, int32_t* __restrict__ deg,
                                int32_t* __restrict__ ids) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        deg[v] = (int32_t)(row[v + 1] - row[v]);
        ids[v] = v;
    }
}

// rank[order[i]] = i
__global__ void rank_kernel(const int32_t* __restrict__ order, int32_t n, int32_t* __restrict__ rank) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) rank[order[i]] = i;
}

// key[v] = (max degree - degree) << 32 | smallest degree rank among v's neighbours (n if none); one warp per vertex
__global__ void tie_key_kernel(const int64_t* __restrict__ row, const int32_t* __restrict__ col,
                               const int32_t* __restrict__ rank, const int32_t* __restrict__ deg, int32_t n,
                               uint64_t* __restrict__ key) {
    const int t = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = w0; v < n; v += nw) {
        int32_t best = n;
        for (int64_t j = row[v] + t; j < row[v + 1]; j += 32) best = min(best, rank[col[j]]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xFFFFFFFFu, best, o));
        if (t == 0) key[v] = ((uint64_t)(uint32_t)(0x7FFFFFFF - deg[v]) << 32) | (uint32_t)best;
    }
}

// inv[order[i]] = i; ndeg[i] = degree of new vertex i
__global__ void inverse_kernel(const int32_t* __restrict__ order, const int32_t* __restrict__ deg, int32_t n,
                               int32_t* __restrict__ inv, int32_t* __restrict__ ndeg) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t o = order[i];
        inv[o] = i;
        ndeg[i] = deg[o];
    }
}

__global__ void widen_kernel(const int32_t* __restrict__ off32, int32_t n, int64_t M, int64_t* __restrict__ row) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x)
        row[i] = i < n ? (int64_t)off32[i] : M;
}

// one warp per new vertex: its old row's neighbours in new ids
__global__ void fill_kernel(const int64_t* __restrict__ row, const int32_t* __restrict__ col,
                            const int32_t* __restrict__ order, const int32_t* __restrict__ inv,
                            const int64_t* __restrict__ nrow, int32_t n, int32_t* __restrict__ ncol) {
    const int t = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < n; i += nw) {
        const int32_t o = order[i];
        const int64_t r0 = row[o], len = row[o + 1] - r0, d0 = nrow[i];
        for (int64_t j = t; j < len; j += 32) ncol[d0 + j] = inv[col[r0 + j]];
    }
}

}  // namespace

gbc_status relabel_by_degree(DevGraph& g, cudaStream_t s, int32_t** d_order_out, int32_t** d_inv_out) {
    const int32_t n = g.n;
    const int64_t M = g.m;
    int32_t *deg = nullptr, *ids = nullptr, *skeys = nullptr, *order = nullptr, *inv = nullptr, *ndeg = nullptr,
            *off32 = nullptr, *ncol = nullptr, *ncol2 = nullptr;
    int64_t* nrow = nullptr;
    uint64_t *key = nullptr, *skey = nullptr;
    void* tmp = nullptr;
    // all buffers through the lane-state cache: graphs created in a loop reuse them
    const size_t sn = sizeof(int32_t) * (size_t)n, sm8 = sizeof(uint64_t) * (size_t)n,
                 srow = sizeof(int64_t) * ((size_t)n + 1), scol = sizeof(int32_t) * std::max<int64_t>(M, 1);
    size_t stmp = 0;
    auto cleanup = [&](bool keep) {
        cudaStreamSynchronize(s);   // nothing in flight may still use a buffer handed back
        dev_release(deg, sn); dev_release(ids, sn); dev_release(skeys, sn); dev_release(ndeg, sn);
        dev_release(off32, sn); dev_release(tmp, stmp); dev_release(key, sm8); dev_release(skey, sm8);
        if (!keep) {
            dev_release(order, sn); dev_release(inv, sn); dev_release(nrow, srow);
            dev_release(ncol, scol); dev_release(ncol2, scol);
        }
    };
    bool ok = true;
    ok &= dev_alloc((void**)&deg, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&ids, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&skeys, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&order, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&inv, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&ndeg, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&off32, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&nrow, srow) == cudaSuccess;
    ok &= dev_alloc((void**)&ncol, scol) == cudaSuccess;
    ok &= dev_alloc((void**)&ncol2, scol) == cudaSuccess;
    ok &= dev_alloc((void**)&key, sm8) == cudaSuccess;
    ok &= dev_alloc((void**)&skey, sm8) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cleanup(false);
        set_error("relabel buffers (n=%d, m=%lld)", n, (long long)M);
        return GBC_ERR_NOMEM;
    }
    int dev = 0, sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    size_t tb1 = 0, tb2 = 0, tb3 = 0, tb4 = 0;
    cudaError_t e = cub::DeviceRadixSort::SortPairsDescending(nullptr, tb1, deg, skeys, ids, order, n, 0, 32, s);
    if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(nullptr, tb2, ndeg, off32, n, s);
    if (e == cudaSuccess)
        e = cub::DeviceSegmentedSort::SortKeys(nullptr, tb3, ncol, ncol2, M, n, nrow, nrow + 1, s);
    if (e == cudaSuccess) e = cub::DeviceRadixSort::SortPairs(nullptr, tb4, key, skey, ids, order, n, 0, 64, s);
    stmp = std::max(std::max(tb1, tb4), std::max(tb2, tb3)) + 16;
    if (e == cudaSuccess) e = dev_alloc(&tmp, stmp);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cleanup(false);
        set_error("relabel workspace: %s", cudaGetErrorString(e));
        return GBC_ERR_NOMEM;
    }
    const int grid = sm * 8;
    deg_iota_kernel<<<grid, 256, 0, s>>>(g.row, n, deg, ids);
    // degree ranks first, then the final order by (degree, rank of the top neighbour, id)
    e = cub::DeviceRadixSort::SortPairsDescending(tmp, tb1, deg, skeys, ids, order, n, 0, 32, s);
    if (e == cudaSuccess) {
        rank_kernel<<<grid, 256, 0, s>>>(order, n, inv);
        tie_key_kernel<<<grid, 256, 0, s>>>(g.row, g.col, inv, deg, n, key);
        e = cub::DeviceRadixSort::SortPairs(tmp, tb4, key, skey, ids, order, n, 0, 64, s);
    }
    if (e == cudaSuccess) {
        inverse_kernel<<<grid, 256, 0, s>>>(order, deg, n, inv, ndeg);
        e = cub::DeviceScan::ExclusiveSum(tmp, tb2, ndeg, off32, n, s);
    }
    if (e == cudaSuccess) {
        widen_kernel<<<grid, 256, 0, s>>>(off32, n, M, nrow);
        fill_kernel<<<grid, 256, 0, s>>>(g.row, g.col, order, inv, nrow, n, ncol);
        if (M > 0) e = cub::DeviceSegmentedSort::SortKeys(tmp, tb3, ncol, ncol2, M, n, nrow, nrow + 1, s);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cleanup(false);
        set_error("relabel failed: %s", cudaGetErrorString(e));
        return GBC_ERR_CUDA;
    }
    dev_release(g.row, srow);
    dev_release(g.col, scol);
    dev_release(ncol, scol);
    ncol = nullptr;
    g.row = nrow;
    g.col = ncol2;
    *d_order_out = order;
    *d_inv_out = inv;
    cleanup(true);
    return GBC_OK;
}

namespace {

// inv[order[i]] = i; ndeg[i] = degree of new vertex i (from the old rows)
__global__ void inverse_row_kernel(const int64_t* __restrict__ row, const int32_t* __restrict__ order, int32_t n,
                                   int32_t* __restrict__ inv, int32_t* __restrict__ ndeg) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int32_t o = order[i];
        inv[o] = i;
        ndeg[i] = (int32_t)(row[o + 1] - row[o]);
    }
}

// Cuthill-McKee order of a host CSR: components in order of their smallest
// vertex; in each, a BFS from the vertex a BFS from that smallest vertex
// reached last (a far, pseudo-peripheral vertex), neighbours in row order.
// order[new] = old.  Returns the most levels any of these BFS had.
int32_t cuthill_mckee(const std::vector<int64_t>& row, const std::vector<int32_t>& col, int32_t n,
                      std::vector<int32_t>& order) {
    std::vector<int32_t> lev(n, -1), probe(n, -1), q(n);
    order.clear();
    order.reserve(n);
    int32_t depth = 0;
    for (int32_t s0 = 0; s0 < n; s0++) {
        if (lev[s0] >= 0) continue;
        // probe BFS from s0: its last vertex is the start
        int32_t head = 0, tail = 0;
        q[tail++] = s0;
        probe[s0] = s0;
        while (head < tail) {
            const int32_t v = q[head++];
            for (int64_t j = row[v]; j < row[v + 1]; j++) {
                const int32_t x = col[j];
                if (probe[x] != s0) { probe[x] = s0; q[tail++] = x; }
            }
        }
        const int32_t a = q[tail - 1];
        head = 0;
        tail = 0;
        q[tail++] = a;
        lev[a] = 0;
        while (head < tail) {
            const int32_t v = q[head++];
            order.push_back(v);
            depth = std::max(depth, lev[v] + 1);
            for (int64_t j = row[v]; j < row[v + 1]; j++) {
                const int32_t x = col[j];
                if (lev[x] < 0) { lev[x] = lev[v] + 1; q[tail++] = x; }
            }
        }
    }
    return depth;
}

}  // namespace

// Rewrite g's rows in the ids of `order` (device, order[new] = old; the
// function takes it over and hands it back as *d_order_out).
static gbc_status apply_order(DevGraph& g, cudaStream_t s, int32_t* order, int32_t** d_order_out, int32_t** d_inv_out) {
    const int32_t n = g.n;
    const int64_t M = g.m;
    int32_t *inv = nullptr, *ndeg = nullptr, *off32 = nullptr, *ncol = nullptr, *ncol2 = nullptr;
    int64_t* nrow = nullptr;
    void* tmp = nullptr;
    const size_t sn = sizeof(int32_t) * (size_t)n, srow = sizeof(int64_t) * ((size_t)n + 1),
                 scol = sizeof(int32_t) * std::max<int64_t>(M, 1);
    size_t stmp = 0;
    auto cleanup = [&](bool keep) {
        cudaStreamSynchronize(s);
        dev_release(ndeg, sn); dev_release(off32, sn); dev_release(tmp, stmp);
        if (!keep) {
            dev_release(order, sn); dev_release(inv, sn); dev_release(nrow, srow);
            dev_release(ncol, scol); dev_release(ncol2, scol);
        }
    };
    bool ok = true;
    ok &= dev_alloc((void**)&inv, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&ndeg, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&off32, sn) == cudaSuccess;
    ok &= dev_alloc((void**)&nrow, srow) == cudaSuccess;
    ok &= dev_alloc((void**)&ncol, scol) == cudaSuccess;
    ok &= dev_alloc((void**)&ncol2, scol) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cleanup(false);
        set_error("relabel buffers (n=%d, m=%lld)", n, (long long)M);
        return GBC_ERR_NOMEM;
    }
    int dev = 0, sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    size_t tb2 = 0, tb3 = 0;
    cudaError_t e = cub::DeviceScan::ExclusiveSum(nullptr, tb2, ndeg, off32, n, s);
    if (e == cudaSuccess) e = cub::DeviceSegmentedSort::SortKeys(nullptr, tb3, ncol, ncol2, M, n, nrow, nrow + 1, s);
    stmp = std::max(tb2, tb3) + 16;
    if (e == cudaSuccess) e = dev_alloc(&tmp, stmp);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cleanup(false);
        set_error("relabel workspace: %s", cudaGetErrorString(e));
        return GBC_ERR_NOMEM;
    }
    const int grid = sm * 8;
    inverse_row_kernel<<<grid, 256, 0, s>>>(g.row, order, n, inv, ndeg);
    e = cub::DeviceScan::ExclusiveSum(tmp, tb2, ndeg, off32, n, s);
    if (e == cudaSuccess) {
        widen_kernel<<<grid, 256, 0, s>>>(off32, n, M, nrow);
        fill_kernel<<<grid, 256, 0, s>>>(g.row, g.col, order, inv, nrow, n, ncol);
        if (M > 0) e = cub::DeviceSegmentedSort::SortKeys(tmp, tb3, ncol, ncol2, M, n, nrow, nrow + 1, s);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cleanup(false);
        set_error("relabel failed: %s", cudaGetErrorString(e));
        return GBC_ERR_CUDA;
    }
    dev_release(g.row, srow);
    dev_release(g.col, scol);
    dev_release(ncol, scol);
    ncol = nullptr;
    g.row = nrow;
    g.col = ncol2;
    *d_order_out = order;
    *d_inv_out = inv;
    cleanup(true);
    return GBC_OK;
}

gbc_status relabel_graph(DevGraph& g, cudaStream_t s, int32_t** d_order_out, int32_t** d_inv_out) {
    const int32_t n = g.n;
    if (n >= LOCALITY_MAX_N || g.m == 0) return relabel_by_degree(g, s, d_order_out, d_inv_out);
    std::vector<int64_t> row((size_t)n + 1);
    GBC_CUDA(cudaMemcpyAsync(row.data(), g.row, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    int64_t md = 0;
    for (int32_t v = 0; v < n; v++) md = std::max<int64_t>(md, row[v + 1] - row[v]);
    g.max_degree = (int32_t)md;
    if (md > LOCALITY_MAX_DEGREE) return relabel_by_degree(g, s, d_order_out, d_inv_out);
    std::vector<int32_t> col((size_t)g.m), order;
    GBC_CUDA(cudaMemcpyAsync(col.data(), g.col, sizeof(int32_t) * (size_t)g.m, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    if (cuthill_mckee(row, col, n, order) <= LOCALITY_MIN_DEPTH) return relabel_by_degree(g, s, d_order_out, d_inv_out);
    int32_t* d_order = nullptr;
    if (dev_alloc((void**)&d_order, sizeof(int32_t) * (size_t)n) != cudaSuccess) {
        cudaGetLastError();
        set_error("relabel order buffer");
        return GBC_ERR_NOMEM;
    }
    if (cudaMemcpyAsync(d_order, order.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        dev_release(d_order, sizeof(int32_t) * (size_t)n);
        set_error("relabel order upload failed");
        return GBC_ERR_CUDA;
    }
    return apply_order(g, s, d_order, d_order_out, d_inv_out);
}

// out[r*n + v] = in[r*n + inv[v]] for r < rows: per-vertex results back to the
// caller's ids.
template <typename T>
__global__ void gather_kernel(const T* __restrict__ in, const int32_t* __restrict__ inv, int32_t n, int64_t rows,
                              T* __restrict__ out) {
    const int64_t total = rows * (int64_t)n;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k / n;
        const int32_t v = (int32_t)(k - r * n);
        out[k] = in[r * n + inv[v]];
    }
}

template <typename T>
gbc_status gather_to_caller(const T* d_in, const int32_t* d_inv, int32_t n, int64_t rows, T* d_out, cudaStream_t s) {
    int dev = 0, sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    gather_kernel<T><<<sm * 8, 256, 0, s>>>(d_in, d_inv, n, rows, d_out);
    GBC_CUDA(cudaGetLastError());
    return GBC_OK;
}

template gbc_status gather_to_caller<double>(const double*, const int32_t*, int32_t, int64_t, double*, cudaStream_t);
template gbc_status gather_to_caller<int32_t>(const int32_t*, const int32_t*, int32_t, int64_t, int32_t*, cudaStream_t);
template gbc_status gather_to_caller<uint64_t>(const uint64_t*, const int32_t*, int32_t, int64_t, uint64_t*,
                                                cudaStream_t);

}  // namespace gbc
