// Closeness distance sums with no allocation: gbc_cc_noalloc.
//
// Some callers cannot allocate device memory at call time.
// - A serving process may reserve all of HBM for its own pool up front, so
//   any further cudaMalloc fails or fragments that pool.
// - A latency-critical caller cannot accept the implicit device
//   synchronisation cudaMalloc/cudaFree may bring.
// - A host runtime may only hand out pre-registered buffers.
// Such callers pass their own device inputs (CSR, sources) and output (one
// int64 per source). The BFS state these kernels need lives in one
// file-scope device array of fixed size. It holds one distance and one
// queue slot per vertex, which limits the graph to GBC_NOALLOC_MAX_VERTICES
// vertices.
//
// The array is shared by every call in the process and keeps the previous
// call's contents. Each call re-initialises what it reads: distances, queue
// head and tail. Two calls that overlap on the GPU (different streams or
// host threads) race on the array; callers must serialise them. The array
// occupies its 16 MB on every GPU that loads the library, until the process
// exits.
//
// The first call on each device looks up the array's device address with
// cudaGetSymbolAddress (the array's name in host code is not a device
// address) and keeps it for later calls; make that first call on a device
// before any stream capture.
//
// Before any BFS indexes the array with the caller's CSR, a check kernel
// reads the whole CSR on the device: row[0] == 0, rows non-decreasing, every
// col entry in [0, n). It records the first offending row and the first
// offending entry in two 64-bit status words of the array's header, and a
// bad CSR is refused with GBC_ERR_ARG before anything is written past the
// header.
//
// The kernels are launched on the caller's stream. The host reads each new
// frontier size and the two status words back with copies into local
// variables, and writes each source's sum with a 64-bit copy from a local
// variable. Nothing is allocated on either side.
#include <cuda_runtime.h>

#include <mutex>

#include "engine.h"

namespace {

constexpr int32_t NOALLOC_MAX_N = 1 << 21;   // GBC_NOALLOC_MAX_VERTICES
constexpr int32_t HDR = 64;                  // int32 slots before the distance array (counters)
constexpr unsigned FULL = 0xFFFFFFFFu;

// [0,64): counters (queue tail at slots 0-1, first bad row at 2-3, first bad
// col entry at 4-5, each 64 bits), then dist[MAX_N], queue[MAX_N]
static __device__ __align__(256) int32_t g_noalloc_scratch[HDR + 2 * NOALLOC_MAX_N];

// Device address of g_noalloc_scratch, looked up once per device.
int32_t* g_scratch_ptr[64] = {};
std::mutex g_scratch_mu;

gbc_status scratch_for_current_device(int32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        gbc::set_error("gbc_cc_noalloc: no usable current device (%s)", cudaGetErrorString(e));
        return GBC_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            gbc::set_error("gbc_cc_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return GBC_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<int32_t*>(p);
    }
    *out = g_scratch_ptr[dev];
    return GBC_OK;
}

// CSR entry check: the smallest v with row[v] > row[v+1] and the smallest j
// with col[j] outside [0, n), into the status words (all ones: none).  The
// host has checked row[0] == 0 and 0 <= row[n] < 2^31 already.
__global__ void na_check(const int64_t* __restrict__ row, const int32_t* __restrict__ col, int32_t n, long long m,
                         int32_t* scratch) {
    unsigned long long* bad = reinterpret_cast<unsigned long long*>(scratch) + 1;
    const long long span = m > (long long)n ? m : (long long)n;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < span; i += (long long)gridDim.x * blockDim.x) {
        if (i < n && row[i] > row[i + 1]) atomicMin(&bad[0], (unsigned long long)i);
        if (i < m) {
            const int32_t x = col[i];
            if (x < 0 || x >= n) atomicMin(&bad[1], (unsigned long long)i);
        }
    }
}

// dist[0..n) = -1 (every call starts from a cleared distance array).
__global__ void na_init(int32_t* scratch, int32_t n) {
    int32_t* dist = scratch + HDR;
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) dist[v] = -1;
}
// Source s at distance 0 as the only queue entry; tail = 1.
__global__ void na_seed(int32_t* scratch, int32_t s) {
    int32_t* dist = scratch + HDR;
    int32_t* queue = scratch + HDR + NOALLOC_MAX_N;
    dist[s] = 0;
    queue[0] = s;
    *reinterpret_cast<unsigned long long*>(scratch) = 1ULL;
}

// One BFS level: warp per frontier vertex, threads over its neighbours.
__global__ void na_expand(const int64_t* __restrict__ row, const int32_t* __restrict__ col, int32_t* scratch,
                          unsigned long long lo, unsigned long long hi, int32_t d) {
    int32_t* dist = scratch + HDR;
    int32_t* queue = scratch + HDR + NOALLOC_MAX_N;
    unsigned long long* tail = reinterpret_cast<unsigned long long*>(scratch);
    const int t = threadIdx.x & 31;
    const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long i = lo + wid; i < hi; i += nw) {
        const int32_t v = queue[i];
        const long long r0 = row[v], r1 = row[v + 1];
        for (long long jb = r0; jb < r1; jb += 32) {
            const long long j = jb + t;
            bool fresh = false;
            int32_t x = 0;
            if (j < r1) {
                x = col[j];
                fresh = (dist[x] < 0) && (atomicCAS(&dist[x], -1, d + 1) == -1);
            }
            const unsigned m = __ballot_sync(FULL, fresh);
            if (m) {
                const int leader = __ffs(m) - 1;
                unsigned long long base = 0;
                if (t == leader) base = atomicAdd(tail, (unsigned long long)__popc(m));
                base = __shfl_sync(FULL, base, leader);
                if (fresh) queue[base + __popc(m & ((1u << t) - 1u))] = x;
            }
        }
    }
}

}  // namespace

extern "C" gbc_status gbc_cc_noalloc(const int64_t* d_row, const int32_t* d_col, int32_t n, const int32_t* d_sources,
                                     int32_t k, int64_t* d_cc, void* stream) {
    using gbc::set_error;
    if (!d_row || !d_col || !d_sources || !d_cc || k < 0) {
        set_error("gbc_cc_noalloc: NULL pointer or negative k");
        return GBC_ERR_ARG;
    }
    if (n <= 0 || n > NOALLOC_MAX_N) {
        set_error("gbc_cc_noalloc: n = %d is outside [1, %d], the size of its fixed scratch array", n, NOALLOC_MAX_N);
        return GBC_ERR_ARG;
    }
    int32_t* scratch = nullptr;
    gbc_status st = scratch_for_current_device(&scratch);
    if (st != GBC_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0, sm = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    GBC_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
    unsigned long long* d_tail = reinterpret_cast<unsigned long long*>(scratch);
    // the CSR's two end offsets, then every row and entry on the device
    int64_t ends[2] = {-1, -1};
    GBC_CUDA(cudaMemcpyAsync(&ends[0], d_row, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaMemcpyAsync(&ends[1], d_row + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    if (ends[0] != 0) {
        set_error("gbc_cc_noalloc: row[0] must be 0 (got %lld)", (long long)ends[0]);
        return GBC_ERR_ARG;
    }
    if (ends[1] < 0 || ends[1] >= ((int64_t)1 << 31)) {
        set_error("gbc_cc_noalloc: row[n]=%lld out of range", (long long)ends[1]);
        return GBC_ERR_ARG;
    }
    unsigned long long bad[2] = {0, 0};
    GBC_CUDA(cudaMemsetAsync(d_tail + 1, 0xFF, sizeof(bad), s));
    na_check<<<sm * 4, 256, 0, s>>>(d_row, d_col, n, (long long)ends[1], scratch);
    GBC_CUDA(cudaGetLastError());
    GBC_CUDA(cudaMemcpyAsync(bad, d_tail + 1, sizeof(bad), cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    if (bad[0] != ~0ULL) {
        set_error("gbc_cc_noalloc: row offsets decrease at vertex %llu", bad[0]);
        return GBC_ERR_ARG;
    }
    if (bad[1] != ~0ULL) {
        set_error("gbc_cc_noalloc: col[%llu] is outside [0,%d)", bad[1], n);
        return GBC_ERR_ARG;
    }
    for (int32_t i = 0; i < k; i++) {
        int32_t src = -1;
        GBC_CUDA(cudaMemcpyAsync(&src, d_sources + i, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaStreamSynchronize(s));
        if (src < 0 || src >= n) {
            set_error("gbc_cc_noalloc: source %d (index %d) out of range [0,%d)", src, i, n);
            return GBC_ERR_ARG;
        }
        na_init<<<sm * 4, 256, 0, s>>>(scratch, n);
        na_seed<<<1, 1, 0, s>>>(scratch, src);
        GBC_CUDA(cudaGetLastError());
        unsigned long long lo = 0, hi = 1;
        int64_t sum = 0;
        for (int32_t d = 0; d < n; d++) {
            na_expand<<<sm * 8, 256, 0, s>>>(d_row, d_col, scratch, lo, hi, d);
            GBC_CUDA(cudaGetLastError());
            unsigned long long tail = 0;
            GBC_CUDA(cudaMemcpyAsync(&tail, d_tail, sizeof(tail), cudaMemcpyDeviceToHost, s));
            GBC_CUDA(cudaStreamSynchronize(s));
            if (tail == hi) break;
            sum += (int64_t)(d + 1) * (int64_t)(tail - hi);
            lo = hi;
            hi = tail;
        }
        GBC_CUDA(cudaMemcpyAsync(d_cc + i, &sum, sizeof(sum), cudaMemcpyHostToDevice, s));
        GBC_CUDA(cudaStreamSynchronize(s));
    }
    return GBC_OK;
}
