// Device-buffer cache for lane state.
//
// A lane engine holds tens of GB (R-MAT scale 22 at 1024 lanes: ~78 GB), and
// cudaFree of that much takes ~50 ms and synchronises the device.  Callers
// that create and destroy graph handles in a loop (the drop-in path builds a
// CSR per call) would pay it every time.  Freed engine buffers therefore go to
// a per-device cache and are handed to the next engine that asks for the same
// size (or at most 25% less).  At most 40% of the device's memory is kept
// cached; past that, freed buffers go straight back.  gbc_release_cached_memory()
// returns them to the driver; a failed cudaMalloc also does, then retries.
// Cached bytes count as free when engines are sized (dev_free_bytes).
#include <cuda_runtime.h>

#include <map>
#include <mutex>

#include "gbc_internal.h"

namespace gbc {

namespace {

struct Cache {
    std::mutex mu;
    std::multimap<size_t, void*> blocks[64];   // per device: size -> block
    size_t bytes[64] = {};
    size_t limit[64] = {};
};

Cache& cache() {
    static Cache* c = new Cache();   // never destroyed: buffers may be returned during exit
    return *c;
}

int current_device() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) { cudaGetLastError(); return 0; }
    return (d >= 0 && d < 64) ? d : 0;
}

void trim_device(Cache& c, int d) {
    for (auto& kv : c.blocks[d]) cudaFree(kv.second);
    c.blocks[d].clear();
    c.bytes[d] = 0;
}

}  // namespace

cudaError_t dev_alloc(void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 1;
    Cache& c = cache();
    const int d = current_device();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        auto it = c.blocks[d].lower_bound(bytes);
        if (it != c.blocks[d].end() && it->first - bytes <= it->first / 4) {
            *p = it->second;
            c.bytes[d] -= it->first;
            c.blocks[d].erase(it);
            return cudaSuccess;
        }
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        {
            std::lock_guard<std::mutex> lk(c.mu);
            trim_device(c, d);
        }
        e = cudaMalloc(p, bytes);
    }
    return e;
}

void dev_release(void* p, size_t bytes) {
    if (!p) return;
    if (bytes == 0) bytes = 1;
    Cache& c = cache();
    const int d = current_device();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        if (c.limit[d] == 0) {
            size_t fr = 0, tot = 0;
            if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); tot = (size_t)16 << 30; }
            c.limit[d] = tot / 5 * 2;   // at most 40% of the device stays cached
        }
        if (c.bytes[d] + bytes <= c.limit[d]) {
            c.blocks[d].emplace(bytes, p);
            c.bytes[d] += bytes;
            return;
        }
    }
    cudaFree(p);
}

size_t dev_cached_bytes() {
    Cache& c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    return c.bytes[current_device()];
}

size_t dev_free_bytes() {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); fr = (size_t)8 << 30; }
    return fr + dev_cached_bytes();
}

}  // namespace gbc

extern "C" gbc_status gbc_release_cached_memory(void) {
    gbc::Cache& c = gbc::cache();
    std::lock_guard<std::mutex> lk(c.mu);
    gbc::trim_device(c, gbc::current_device());
    return GBC_OK;
}
