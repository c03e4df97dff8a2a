// Plain engine: one source at a time.  Per level, one kernel expands the
// frontier (warp per frontier vertex, threads over its neighbours; distances
// claimed with atomicCAS, path counts added with 64-bit atomics) and the host
// reads the new frontier size back before launching the next level -- the
// per-source, per-level host loop of the reference's GPU programs
// (GPU_FAN/gpu_fan.cu:101-121, parallel_CC/para_CC.cu:237-254), with sigma
// and the dependency sweep added.  It is the one-source-at-a-time baseline
// that the batched lane engine is measured against.
#include <cuda_runtime.h>

#include <vector>

#include "engine.h"

namespace gbc {
namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;

__global__ void plain_init(int32_t* dist, int n, int s, uint64_t* sig, int32_t* q, unsigned long long* tail,
                           uint32_t* ovf) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) dist[v] = -1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *tail = 1;
        q[0] = s;
        *ovf = 0;
    }
}
__global__ void plain_seed(int32_t* dist, uint64_t* sig, int s) {
    dist[s] = 0;
    if (sig) sig[s] = 1ULL;
}

__global__ void plain_expand(const int64_t* __restrict__ row, const int32_t* __restrict__ col, int32_t* dist,
                             uint64_t* sig, int32_t* q, unsigned long long lo, unsigned long long hi,
                             unsigned long long* tail, int d, uint32_t* ovf) {
    const int t = threadIdx.x & 31;
    const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long i = lo + wid; i < hi; i += nw) {
        const int v = q[i];
        const uint64_t sv = sig ? sig[v] : 0ULL;
        const long long r0 = row[v], r1 = row[v + 1];
        for (long long jb = r0; jb < r1; jb += 32) {
            const long long j = jb + t;
            bool fresh = false;
            int x = 0;
            if (j < r1) {
                x = col[j];
                int dx = dist[x];
                if (dx < 0) {
                    const int old = atomicCAS(&dist[x], -1, d + 1);
                    fresh = (old == -1);
                    dx = fresh ? d + 1 : old;
                }
                if (sig && dx == d + 1) {
                    const unsigned long long old = atomicAdd((unsigned long long*)&sig[x], (unsigned long long)sv);
                    if (old + sv < old) atomicOr(ovf, 1u);
                }
            }
            const unsigned m = __ballot_sync(FULL, fresh);
            if (m) {
                const int leader = __ffs(m) - 1;
                unsigned long long base = 0;
                if (t == leader) base = atomicAdd(tail, (unsigned long long)__popc(m));
                base = __shfl_sync(FULL, base, leader);
                if (fresh) q[base + __popc(m & ((1u << t) - 1u))] = x;
            }
        }
    }
}

template <typename T>
__global__ void plain_backward(const int64_t* __restrict__ row, const int32_t* __restrict__ col,
                               const int32_t* dist, const uint64_t* sig, T* rho, const int32_t* q,
                               unsigned long long lo, unsigned long long hi, int d, int refsem, double* bc) {
    const int t = threadIdx.x & 31;
    const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long i = lo + wid; i < hi; i += nw) {
        const int v = q[i];
        T acc = T(0);
        int pc = 0;
        for (long long j = row[v] + t; j < row[v + 1]; j += 32) {
            const int x = col[j];
            const int dx = dist[x];
            if (dx == d + 1) acc += rho[x];
            else if (dx == d - 1) pc++;
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc += __shfl_xor_sync(FULL, acc, o);
            pc += __shfl_xor_sync(FULL, pc, o);
        }
        if (t == 0) {
            const T sv = (T)sig[v];
            const T delta = sv * acc;
            rho[v] = (T(1) + delta) / sv;
            bc[v] += (double)delta * (refsem ? (double)pc : 1.0);
        }
    }
}

struct PlainState {
    int32_t* dist = nullptr;
    uint64_t* sig = nullptr;
    void* rho = nullptr;
    int32_t* q = nullptr;
    unsigned long long* tail = nullptr;
    uint32_t* ovf = nullptr;
    unsigned long long* h_tail = nullptr;
    ~PlainState() {
        cudaFree(dist); cudaFree(sig); cudaFree(rho); cudaFree(q); cudaFree(tail); cudaFree(ovf);
        if (h_tail) cudaFreeHost(h_tail);
    }
};

gbc_status plain_alloc(PlainState& S, int n, bool bc) {
    bool ok = cudaMalloc(&S.dist, sizeof(int32_t) * n) == cudaSuccess;
    ok &= cudaMalloc(&S.q, sizeof(int32_t) * n) == cudaSuccess;
    ok &= cudaMalloc(&S.tail, sizeof(unsigned long long)) == cudaSuccess;
    ok &= cudaMalloc(&S.ovf, sizeof(uint32_t)) == cudaSuccess;
    ok &= cudaMallocHost(&S.h_tail, sizeof(unsigned long long) * 2) == cudaSuccess;
    if (bc) {
        ok &= cudaMalloc(&S.sig, sizeof(uint64_t) * n) == cudaSuccess;
        ok &= cudaMalloc(&S.rho, sizeof(double) * n) == cudaSuccess;
    }
    if (!ok) { cudaGetLastError(); set_error("plain engine allocation failed"); return GBC_ERR_NOMEM; }
    return GBC_OK;
}

int grid_for(int sm) { return sm * 8; }

// Forward BFS of one source with per-level host reads; fills level offsets.
gbc_status plain_forward(const DevGraph* g, PlainState& S, int s, bool bc, cudaStream_t st, int sm,
                         std::vector<unsigned long long>& off, LaneResult& res) {
    plain_init<<<sm * 4, 256, 0, st>>>(S.dist, g->n, s, S.sig, S.q, S.tail, S.ovf);
    plain_seed<<<1, 1, 0, st>>>(S.dist, bc ? S.sig : nullptr, s);
    res.kernel_launches += 2;
    off.assign(1, 0ULL);
    off.push_back(1ULL);
    int d = 0;
    for (;;) {
        const unsigned long long lo = off[d], hi = off[d + 1];
        plain_expand<<<grid_for(sm), 256, 0, st>>>(g->row, g->col, S.dist, bc ? S.sig : nullptr, S.q, lo, hi, S.tail,
                                                   d, S.ovf);
        res.kernel_launches++;
        GBC_CUDA(cudaMemcpyAsync(S.h_tail, S.tail, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        GBC_CUDA(cudaStreamSynchronize(st));
        const unsigned long long nt = S.h_tail[0];
        if (nt == hi) break;
        off.push_back(nt);
        d++;
    }
    res.levels += (int64_t)off.size() - 1;
    return GBC_OK;
}

}  // namespace

gbc_status plain_cc(const DevGraph* g, const int32_t* h_src, int32_t k, int64_t* h_cc, cudaStream_t st,
                    LaneResult& res) {
    PlainState S;
    GBC_TRY(plain_alloc(S, g->n, false));
    int dev = 0, sm = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    GBC_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
    std::vector<unsigned long long> off;
    for (int32_t i = 0; i < k; i++) {
        GBC_TRY(plain_forward(g, S, h_src[i], false, st, sm, off, res));
        int64_t sum = 0;
        // level d holds queue entries off[d] .. off[d+1]
        for (size_t d = 1; d + 1 < off.size(); d++) sum += (int64_t)d * (int64_t)(off[d + 1] - off[d]);
        h_cc[i] = sum;
    }
    GBC_CUDA(cudaStreamSynchronize(st));
    return GBC_OK;
}

gbc_status plain_bc(const DevGraph* g, const int32_t* h_src, int32_t k, int semantics, int delta_f64, double* d_bc,
                    cudaStream_t st, LaneResult& res) {
    PlainState S;
    GBC_TRY(plain_alloc(S, g->n, true));
    int dev = 0, sm = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    GBC_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
    std::vector<unsigned long long> off;
    uint32_t h_ovf = 0;
    for (int32_t i = 0; i < k; i++) {
        GBC_CUDA(cudaMemsetAsync(S.sig, 0, sizeof(uint64_t) * g->n, st));
        GBC_TRY(plain_forward(g, S, h_src[i], true, st, sm, off, res));
        const int levels = (int)off.size() - 1;   // levels 0 .. levels-1
        for (int d = levels - 1; d >= 1; d--) {
            if (delta_f64)
                plain_backward<double><<<grid_for(sm), 256, 0, st>>>(g->row, g->col, S.dist, S.sig, (double*)S.rho, S.q,
                                                                     off[d], off[d + 1], d,
                                                                     semantics == GBC_BC_REFERENCE, d_bc);
            else
                plain_backward<float><<<grid_for(sm), 256, 0, st>>>(g->row, g->col, S.dist, S.sig, (float*)S.rho, S.q,
                                                                    off[d], off[d + 1], d,
                                                                    semantics == GBC_BC_REFERENCE, d_bc);
            res.kernel_launches++;
        }
        GBC_CUDA(cudaGetLastError());
        GBC_CUDA(cudaMemcpyAsync(&h_ovf, S.ovf, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        GBC_CUDA(cudaStreamSynchronize(st));
        if (h_ovf) res.overflow_count++;
    }
    return GBC_OK;
}

}  // namespace gbc
