// Batched multi-source lane engine for sm_103a.
//
// B sources ("lanes") of one batch run level-synchronous BFS together.  Lane
// state is lane-interleaved: for lane group g (32 lanes, one per warp thread)
// and vertex v the 32 entries lvl/sigma/rho[g][v][0..31] are contiguous, so a
// warp that visits a neighbour x touches one 64-byte (lvl) or 256-byte
// (sigma, rho) segment for all 32 lanes of its group.  The frontier of level
// d is a list of (vertex, group) entries; the lists of all levels are kept
// (fq + foff) and replayed in reverse by the dependency sweep.
//
// Forward, one kernel per level (expand): for every entry (v,g) of F_d and
// every lane with lvl == d, pull sigma(v) from the level-(d-1) neighbours
// (no atomics, deterministic) and discover level d+1 among the neighbours
// (plain store of d+1, enqueue once per (x,g) via vmark).  A task whose active
// lanes are few expands edge-parallel (threads over neighbours, lanes in
// turn), otherwise lane-parallel (threads over lanes, neighbours in turn).
// Backward, one kernel per level (pull): delta(v) = sigma(v) * sum over
// successors w of rho(w), rho(v) = (1 + delta(v)) / sigma(v); per-group FP64
// partials of BC accumulate without atomics.  Levels are read from a device
// control block and advanced by the last CTA of each launch, so a fixed run
// of level launches is captured once as a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "engine.h"

namespace gbc {

namespace {

constexpr uint16_t INF16 = 0xFFFFu;
constexpr int MAX_LEVEL = 65000;   // lvl is uint16; deeper BFS is reported as GBC_ERR_LIMIT
constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr int BLOCK = 256;

struct Ctl {
    int level;
    int maxlevel;
    int done;
    int err;            // bit0: frontier queue overflow, bit1: level cap
    unsigned blocks;    // finished-CTA counter of the running launch
    int pad;
    unsigned long long tail;
};

struct KArgs {
    const int64_t* __restrict__ row;
    const int32_t* __restrict__ col;
    int n;
    int ng;
    const int32_t* w;      // nullable vertex weights
    const int64_t* ff;     // nullable folded distance sums
    uint16_t* lvl;
    uint64_t* sig;
    void* rho;
    int32_t* vmark;
    uint32_t* fq;
    unsigned long long fcap;
    unsigned long long* foff;
    Ctl* ctl;
    uint32_t* ovf;
    unsigned long long* cc;
    double* bcg;
    int sparse;
    int semantics;
};

__device__ __forceinline__ size_t sidx(int g, int n, int v, int t) {
    return ((((size_t)g * (size_t)n) + (size_t)v) << 5) + (size_t)t;
}

// Enqueue (x, g) for level lev unless already enqueued at lev.
__device__ __forceinline__ void enqueue_once(const KArgs& A, int x, int g, int lev) {
    if (atomicExch(&A.vmark[(size_t)g * A.n + x], lev) != lev) {
        unsigned long long pos = atomicAdd(&A.ctl->tail, 1ULL);
        if (pos < A.fcap) A.fq[pos] = ((uint32_t)x << 5) | (uint32_t)g;
    }
}

// Warp-aggregated append of the entries of threads with has == true.
__device__ __forceinline__ void warp_append(const KArgs& A, bool has, uint32_t ent) {
    const unsigned m = __ballot_sync(FULL, has);
    if (!m) return;
    const int t = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if (t == leader) base = atomicAdd(&A.ctl->tail, (unsigned long long)__popc(m));
    base = __shfl_sync(FULL, base, leader);
    if (has) {
        unsigned long long pos = base + __popc(m & ((1u << t) - 1u));
        if (pos < A.fcap) A.fq[pos] = ent;
    }
}

__device__ __forceinline__ void lse_add(double& m, double& s, double y) {
    if (y > m) { s = s * exp2(m - y) + 1.0; m = y; }
    else s += exp2(y - m);
}
__device__ __forceinline__ void lse_merge(double& m, double& s, double m2, double s2) {
    const double M = fmax(m, m2);
    if (M == -INFINITY) { m = M; s = 0.0; return; }
    s = s * exp2(m - M) + s2 * exp2(m2 - M);
    m = M;
}

// Last CTA of a forward launch publishes the next level's frontier bounds.
__device__ __forceinline__ void fwd_last_block(const KArgs& A, int d, int done) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&A.ctl->blocks, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            A.ctl->blocks = 0;
            if (!done) {
                unsigned long long tail = atomicAdd(&A.ctl->tail, 0ULL);
                if (tail > A.fcap) {
                    A.ctl->err |= 1;
                    A.ctl->done = 1;
                    A.ctl->maxlevel = d;
                } else {
                    A.foff[d + 2] = tail;
                    if (tail == A.foff[d + 1]) { A.ctl->done = 1; A.ctl->maxlevel = d; }
                    else if (d + 1 >= MAX_LEVEL) { A.ctl->err |= 2; A.ctl->done = 1; A.ctl->maxlevel = d; }
                    else A.ctl->level = d + 1;
                }
            }
        }
    }
}

// MODE 0: distances only (closeness sums per lane); 1: exact uint64 sigma;
// 2: log2-domain sigma (FP64).
template <int MODE>
__global__ void __launch_bounds__(BLOCK) expand_kernel(KArgs A) {
    __shared__ unsigned long long cc_sh[MODE == 0 ? 32 * 32 : 1];
    if (MODE == 0) {
        for (int i = threadIdx.x; i < A.ng * 32; i += blockDim.x) cc_sh[i] = 0ULL;
        __syncthreads();
    }
    const int done = *(volatile int*)&A.ctl->done;
    const int d = *(volatile int*)&A.ctl->level;
    if (!done) {
        const unsigned long long b = A.foff[d], e = A.foff[d + 1];
        const int t = threadIdx.x & 31;
        const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
        double* sigd = reinterpret_cast<double*>(A.sig);
        for (unsigned long long i = b + wid; i < e; i += nw) {
            const uint32_t ent = A.fq[i];
            const int v = (int)(ent >> 5), g = (int)(ent & 31u);
            const size_t gbase = (size_t)g * (size_t)A.n;
            uint16_t* lv = A.lvl + (gbase << 5);
            const uint16_t L = lv[((size_t)v << 5) + t];
            const bool act = (L == (uint16_t)d);
            const unsigned am = __ballot_sync(FULL, act);
            if (am == 0u) continue;
            if (MODE == 0 && act) {
                const long long c = (A.w ? (long long)d * (long long)A.w[v] : (long long)d) + (A.ff ? A.ff[v] : 0LL);
                atomicAdd(&cc_sh[g * 32 + t], (unsigned long long)c);
            }
            const long long r0 = A.row[v], r1 = A.row[v + 1];
            uint64_t acc = 0;
            bool of = false;
            double lm = -INFINITY, ls = 0.0;
            if (__popc(am) > A.sparse) {
                // lane-parallel: thread t owns lane t, neighbours in turn
                for (long long jb = r0; jb < r1; jb += 32) {
                    const int cnt = (int)min(32LL, r1 - jb);
                    const int xm = (t < cnt) ? A.col[jb + t] : 0;
#pragma unroll 4
                    for (int q = 0; q < cnt; q++) {
                        const int x = __shfl_sync(FULL, xm, q);
                        uint16_t* px = lv + ((size_t)x << 5) + t;
                        const uint16_t Lx = *px;
                        bool disc = false;
                        if (act) {
                            if (MODE != 0 && d > 0 && Lx == (uint16_t)(d - 1)) {
                                const size_t xi = ((gbase + (size_t)x) << 5) + t;
                                if (MODE == 1) {
                                    const uint64_t s = A.sig[xi];
                                    const uint64_t na = acc + s;
                                    of |= (na < acc);
                                    acc = na;
                                } else {
                                    lse_add(lm, ls, sigd[xi]);
                                }
                            }
                            if (Lx > (uint16_t)d) {
                                disc = true;
                                if (Lx == INF16) *px = (uint16_t)(d + 1);
                            }
                        }
                        const unsigned dm = __ballot_sync(FULL, disc);
                        if (dm && t == 0) enqueue_once(A, x, g, d + 1);
                    }
                }
            } else {
                // edge-parallel: threads over neighbours, active lanes in turn
                unsigned rem = am;
                while (rem) {
                    const int a = __ffs(rem) - 1;
                    rem &= rem - 1u;
                    uint64_t pacc = 0;
                    bool pof = false;
                    double pm = -INFINITY, ps = 0.0;
                    for (long long jb = r0; jb < r1; jb += 32) {
                        const long long j = jb + t;
                        bool has = false;
                        int x = 0;
                        if (j < r1) {
                            x = A.col[j];
                            uint16_t* px = lv + ((size_t)x << 5) + a;
                            const uint16_t Lx = *px;
                            if (MODE != 0 && d > 0 && Lx == (uint16_t)(d - 1)) {
                                const size_t xi = ((gbase + (size_t)x) << 5) + a;
                                if (MODE == 1) {
                                    const uint64_t s = A.sig[xi];
                                    const uint64_t na = pacc + s;
                                    pof |= (na < pacc);
                                    pacc = na;
                                } else {
                                    lse_add(pm, ps, sigd[xi]);
                                }
                            }
                            if (Lx > (uint16_t)d) {
                                if (Lx == INF16) *px = (uint16_t)(d + 1);
                                has = (atomicExch(&A.vmark[gbase + x], d + 1) != d + 1);
                            }
                        }
                        warp_append(A, has, ((uint32_t)x << 5) | (uint32_t)g);
                    }
                    if (MODE == 1) {
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) {
                            const uint64_t p2 = __shfl_xor_sync(FULL, pacc, o);
                            const int f2 = __shfl_xor_sync(FULL, (int)pof, o);
                            const uint64_t na = pacc + p2;
                            pof = pof || f2 || (na < pacc);
                            pacc = na;
                        }
                        if (t == a) { acc = pacc; of = pof; }
                    } else if (MODE == 2) {
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) {
                            const double m2 = __shfl_xor_sync(FULL, pm, o);
                            const double s2 = __shfl_xor_sync(FULL, ps, o);
                            lse_merge(pm, ps, m2, s2);
                        }
                        if (t == a) { lm = pm; ls = ps; }
                    }
                }
            }
            if (MODE != 0 && act && d > 0) {
                const size_t vi = ((gbase + (size_t)v) << 5) + t;
                if (MODE == 1) {
                    A.sig[vi] = acc;
                    if (of) atomicOr(&A.ovf[g], 1u << t);
                } else {
                    sigd[vi] = lm + log2(ls);
                }
            }
        }
    }
    if (MODE == 0) {
        __syncthreads();
        for (int i = threadIdx.x; i < A.ng * 32; i += blockDim.x)
            if (cc_sh[i]) atomicAdd(&A.cc[i], cc_sh[i]);
    }
    fwd_last_block(A, d, done);
}

// Dependency sweep for one level d >= 1 (descending).  LOG: sigma held as
// log2 and rho as a(w) = log2(1 + delta(w)) - log2 sigma(w), so that
// sigma(v)/sigma(w) * (1 + delta(w)) = exp2(log2 sigma(v) + a(w)).
template <bool LOG, typename T>
__global__ void __launch_bounds__(BLOCK) backward_kernel(KArgs A) {
    const int d = *(volatile int*)&A.ctl->level;
    if (d >= 1) {
        const unsigned long long b = A.foff[d], e = A.foff[d + 1];
        const int t = threadIdx.x & 31;
        const unsigned long long wid = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
        const double* sigd = reinterpret_cast<const double*>(A.sig);
        T* rho = reinterpret_cast<T*>(A.rho);
        double* rhod = reinterpret_cast<double*>(A.rho);
        const bool refsem = (A.semantics == GBC_BC_REFERENCE);
        for (unsigned long long i = b + wid; i < e; i += nw) {
            const uint32_t ent = A.fq[i];
            const int v = (int)(ent >> 5), g = (int)(ent & 31u);
            const size_t gbase = (size_t)g * (size_t)A.n;
            const uint16_t* lv = A.lvl + (gbase << 5);
            const size_t vi = ((gbase + (size_t)v) << 5) + t;
            const bool act = (lv[((size_t)v << 5) + t] == (uint16_t)d);
            const unsigned am = __ballot_sync(FULL, act);
            if (am == 0u) continue;
            double lsv = 0.0;
            if (LOG) lsv = act ? sigd[vi] : 0.0;
            T acc = T(0);
            int pc = 0;
            const long long r0 = A.row[v], r1 = A.row[v + 1];
            if (__popc(am) > A.sparse) {
                for (long long jb = r0; jb < r1; jb += 32) {
                    const int cnt = (int)min(32LL, r1 - jb);
                    const int xm = (t < cnt) ? A.col[jb + t] : 0;
#pragma unroll 4
                    for (int q = 0; q < cnt; q++) {
                        const int x = __shfl_sync(FULL, xm, q);
                        const uint16_t Lx = lv[((size_t)x << 5) + t];
                        if (act) {
                            if (Lx == (uint16_t)(d + 1)) {
                                const size_t xi = ((gbase + (size_t)x) << 5) + t;
                                if (LOG) acc += (T)exp2(lsv + rhod[xi]);
                                else acc += rho[xi];
                            } else if (Lx == (uint16_t)(d - 1)) {
                                pc++;
                            }
                        }
                    }
                }
            } else {
                unsigned rem = am;
                while (rem) {
                    const int a = __ffs(rem) - 1;
                    rem &= rem - 1u;
                    const double lsa = LOG ? __shfl_sync(FULL, lsv, a) : 0.0;
                    T pacc = T(0);
                    int ppc = 0;
                    for (long long jb = r0; jb < r1; jb += 32) {
                        const long long j = jb + t;
                        if (j < r1) {
                            const int x = A.col[j];
                            const uint16_t Lx = lv[((size_t)x << 5) + a];
                            if (Lx == (uint16_t)(d + 1)) {
                                const size_t xi = ((gbase + (size_t)x) << 5) + a;
                                if (LOG) pacc += (T)exp2(lsa + rhod[xi]);
                                else pacc += rho[xi];
                            } else if (Lx == (uint16_t)(d - 1)) {
                                ppc++;
                            }
                        }
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        pacc += __shfl_xor_sync(FULL, pacc, o);
                        ppc += __shfl_xor_sync(FULL, ppc, o);
                    }
                    if (t == a) { acc = pacc; pc = ppc; }
                }
            }
            double contrib = 0.0;
            if (act) {
                T delta;
                if (LOG) {
                    delta = acc;
                    rhod[vi] = log2(1.0 + (double)delta) - lsv;
                } else {
                    const T sv = (T)A.sig[vi];
                    delta = sv * acc;
                    rho[vi] = (T(1) + delta) / sv;
                }
                contrib = (double)delta * (refsem ? (double)pc : 1.0);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(FULL, contrib, o);
            if (t == 0) A.bcg[gbase + v] += contrib;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&A.ctl->blocks, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            A.ctl->blocks = 0;
            if (d >= 1) A.ctl->level = d - 1;
        }
    }
}

// One CTA: place each lane's source at level 0 and build F_0.
__global__ void seed_kernel(KArgs A, const int32_t* __restrict__ src, int kb, int mode) {
    const int l = threadIdx.x;
    if (l < kb) {
        const int g = l >> 5, t = l & 31;
        const int s = src[l];
        if (s >= 0 && s < A.n) {
            const size_t i = sidx(g, A.n, s, t);
            A.lvl[i] = 0;
            if (mode == 1) A.sig[i] = 1ULL;
            else if (mode == 2) reinterpret_cast<double*>(A.sig)[i] = 0.0;
            if (atomicExch(&A.vmark[(size_t)g * A.n + s], 0) != 0) {
                const unsigned long long pos = atomicAdd(&A.ctl->tail, 1ULL);
                A.fq[pos] = ((uint32_t)s << 5) | (uint32_t)g;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned long long tail = atomicAdd(&A.ctl->tail, 0ULL);
        A.foff[0] = 0;
        A.foff[1] = tail;
        A.ctl->level = 0;
        A.ctl->maxlevel = 0;
        A.ctl->done = (tail == 0);
        A.ctl->err = 0;
        A.ctl->blocks = 0;
    }
}

__global__ void bw_begin_kernel(KArgs A) { A.ctl->level = A.ctl->maxlevel; A.ctl->blocks = 0; }

// Reset the lane state touched by the batch (every (v,g) of every level).
__global__ void cleanup_kernel(KArgs A, unsigned long long count) {
    const unsigned long long tid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long k = tid; k < count * 32ULL; k += stride) {
        const unsigned long long i = k >> 5;
        const int t = (int)(k & 31ULL);
        const uint32_t ent = A.fq[i];
        const int v = (int)(ent >> 5), g = (int)(ent & 31u);
        A.lvl[sidx(g, A.n, v, t)] = INF16;
        if (t == 0) A.vmark[(size_t)g * A.n + v] = -1;
    }
}

// Distances and exact counts of lanes [0,kb) into dense [kb][n] arrays.
__global__ void sssp_out_kernel(KArgs A, int kb, int32_t* dist, uint64_t* sigma) {
    const size_t total = (size_t)kb * A.n;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(k / A.n), v = (int)(k % A.n);
        const size_t i = sidx(l >> 5, A.n, v, l & 31);
        const uint16_t L = A.lvl[i];
        if (dist) dist[k] = (L == INF16) ? -1 : (int32_t)L;
        if (sigma) sigma[k] = (L == INF16) ? 0ULL : A.sig[i];
    }
}

// bc[v] = sum over lane groups of the per-group partials (fixed order).
__global__ void bc_reduce_kernel(const double* __restrict__ bcg, int ng, int n, double* __restrict__ bc) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int g = 0; g < ng; g++) s += bcg[(size_t)g * n + v];
        bc[v] = s;
    }
}

}  // namespace

// ------------------------------------------------------------------------
struct LaneAccess {
    static KArgs args(const LaneEngine& e, int semantics) {
        KArgs A;
        A.row = e.g_->row; A.col = e.g_->col; A.n = e.g_->n; A.ng = e.ng_;
        A.w = e.g_->w; A.ff = e.g_->ff;
        A.lvl = e.lvl_; A.sig = e.sig_; A.rho = e.rho_; A.vmark = e.vmark_;
        A.fq = e.fq_; A.fcap = e.fcap_; A.foff = e.foff_; A.ctl = (Ctl*)e.ctl_; A.ovf = e.ovf_;
        A.cc = e.ccbuf_; A.bcg = e.bcg_; A.sparse = e.sparse_; A.semantics = semantics;
        return A;
    }
};

size_t LaneEngine::bytes_needed(int32_t n, int32_t lanes, bool need_bc) {
    const size_t ng = (size_t)lanes / 32;
    size_t b = (size_t)lanes * n * 2 + ng * n * 4 + ng * n * 8 * 4 /*initial queue*/ + (size_t)(MAX_LEVEL + 2) * 8;
    if (need_bc) b += (size_t)lanes * n * 16 + ng * n * 8;
    return b + lanes * 8 + (1 << 20);
}

void LaneEngine::release() {
    for (auto& c : graphs_) if (c.exec) cudaGraphExecDestroy(c.exec);
    graphs_.clear();
    cudaFree(lvl_); cudaFree(sig_); cudaFree(rho_); cudaFree(vmark_); cudaFree(fq_); cudaFree(foff_);
    cudaFree(ctl_); cudaFree(ovf_);
    if (ctl_host_) cudaFreeHost(ctl_host_);
    cudaFree(bcg_);
    cudaFree(ccbuf_);
    lvl_ = nullptr; sig_ = nullptr; rho_ = nullptr; vmark_ = nullptr; fq_ = nullptr; foff_ = nullptr;
    ctl_ = nullptr; ovf_ = nullptr; ctl_host_ = nullptr; bcg_ = nullptr; ccbuf_ = nullptr;
}

LaneEngine::~LaneEngine() { release(); }

gbc_status LaneEngine::alloc_queue(unsigned long long cap) {
    if (fq_) cudaFree(fq_);
    fq_ = nullptr;
    if (cudaMalloc(&fq_, cap * sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        set_error("frontier queue allocation of %llu entries failed", cap);
        return GBC_ERR_NOMEM;
    }
    fcap_ = cap;
    for (auto& c : graphs_) if (c.exec) cudaGraphExecDestroy(c.exec);
    graphs_.clear();
    return GBC_OK;
}

gbc_status LaneEngine::init(const DevGraph* g, int32_t lanes, bool need_bc, int sparse_lanes, int levels_per_graph,
                            cudaStream_t stream) {
    release();
    if (lanes < 32 || lanes > 1024 || lanes % 32) { set_error("lanes must be a multiple of 32 in [32,1024]"); return GBC_ERR_ARG; }
    if (g->n >= (1 << 27)) { set_error("lane engine supports fewer than 2^27 vertices"); return GBC_ERR_ARG; }
    g_ = g;
    lanes_ = lanes;
    ng_ = lanes / 32;
    need_bc_ = need_bc;
    sparse_ = sparse_lanes < 0 ? 2 : sparse_lanes;
    lpg_ = levels_per_graph > 0 ? levels_per_graph : 16;
    stream_ = stream;
    int dev = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    GBC_CUDA(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, dev));
    const size_t n = (size_t)g->n;
    const size_t cells = (size_t)lanes * n;
    bool ok = true;
    ok &= cudaMalloc(&lvl_, cells * sizeof(uint16_t)) == cudaSuccess;
    ok &= cudaMalloc(&vmark_, (size_t)ng_ * n * sizeof(int32_t)) == cudaSuccess;
    ok &= cudaMalloc(&foff_, (MAX_LEVEL + 2) * sizeof(unsigned long long)) == cudaSuccess;
    ok &= cudaMalloc(&ctl_, sizeof(Ctl)) == cudaSuccess;
    ok &= cudaMalloc(&ovf_, 32 * sizeof(uint32_t)) == cudaSuccess;
    ok &= cudaMalloc(&ccbuf_, 1024 * sizeof(unsigned long long)) == cudaSuccess;
    ok &= cudaMallocHost(&ctl_host_, sizeof(Ctl)) == cudaSuccess;
    if (need_bc) {
        ok &= cudaMalloc(&sig_, cells * sizeof(uint64_t)) == cudaSuccess;
        ok &= cudaMalloc(&rho_, cells * sizeof(double)) == cudaSuccess;
        ok &= cudaMalloc(&bcg_, (size_t)ng_ * n * sizeof(double)) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        release();
        set_error("lane state allocation failed (n=%zu lanes=%d)", n, lanes);
        return GBC_ERR_NOMEM;
    }
    GBC_TRY(alloc_queue((unsigned long long)ng_ * n * 8ULL + (1ULL << 16)));
    GBC_CUDA(cudaMemsetAsync(lvl_, 0xFF, cells * sizeof(uint16_t), stream_));
    GBC_CUDA(cudaMemsetAsync(vmark_, 0xFF, (size_t)ng_ * n * sizeof(int32_t), stream_));
    GBC_CUDA(cudaMemsetAsync(ctl_, 0, sizeof(Ctl), stream_));
    GBC_CUDA(cudaMemsetAsync(ovf_, 0, 32 * sizeof(uint32_t), stream_));
    bytes_ = cells * 2 + (size_t)ng_ * n * 4 + fcap_ * 4 + (need_bc ? cells * 16 + (size_t)ng_ * n * 8 : 0);
    // grid: enough resident CTAs to fill every SM
    int occ = 0;
    GBC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, expand_kernel<1>, BLOCK, 0));
    grid_ = sm_count_ * std::max(1, std::min(occ, 8));
    return GBC_OK;
}


// Graph keys: 0..2 expand MODE; 3 + (log*2 + f64)*2 + refsem: backward.
gbc_status LaneEngine::get_graph(int key, cudaGraphExec_t* out) {
    for (auto& c : graphs_) if (c.key == key) { *out = c.exec; return GBC_OK; }
    KArgs A = LaneAccess::args(*this, key >= 3 ? (((key - 3) & 1) ? GBC_BC_REFERENCE : GBC_BC_BRANDES) : GBC_BC_BRANDES);
    cudaStream_t cs;
    GBC_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    for (int i = 0; i < lpg_ && e == cudaSuccess; i++) {
        switch (key) {
            case 0: expand_kernel<0><<<grid_, BLOCK, 0, cs>>>(A); break;
            case 1: expand_kernel<1><<<grid_, BLOCK, 0, cs>>>(A); break;
            case 2: expand_kernel<2><<<grid_, BLOCK, 0, cs>>>(A); break;
            default: {
                const int v = (key - 3) >> 1;  // log*2 + f64
                if (v == 0) backward_kernel<false, float><<<grid_, BLOCK, 0, cs>>>(A);
                else if (v == 1) backward_kernel<false, double><<<grid_, BLOCK, 0, cs>>>(A);
                else if (v == 2) backward_kernel<true, float><<<grid_, BLOCK, 0, cs>>>(A);
                else backward_kernel<true, double><<<grid_, BLOCK, 0, cs>>>(A);
            }
        }
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
    if (e == cudaSuccess) e = e2;
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e2 == cudaSuccess) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) { set_error("level-loop graph capture failed: %s", cudaGetErrorString(e)); return GBC_ERR_CUDA; }
    graphs_.push_back({key, exec});
    *out = exec;
    return GBC_OK;
}

gbc_status LaneEngine::bc_begin() {
    if (!need_bc_) { set_error("engine has no BC state"); return GBC_ERR_ARG; }
    GBC_CUDA(cudaMemsetAsync(bcg_, 0, (size_t)ng_ * g_->n * sizeof(double), stream_));
    return GBC_OK;
}

gbc_status LaneEngine::bc_finish(double* d_bc) {
    bc_reduce_kernel<<<sm_count_ * 4, 256, 0, stream_>>>(bcg_, ng_, g_->n, d_bc);
    GBC_CUDA(cudaGetLastError());
    return GBC_OK;
}

gbc_status LaneEngine::run(const LaneRequest& rq, LaneResult& res) {
    if (rq.kb < 1 || rq.kb > lanes_) { set_error("batch of %d sources for %d lanes", rq.kb, lanes_); return GBC_ERR_ARG; }
    const bool bc = rq.job != LaneJob::CC;
    if (bc && !need_bc_) { set_error("engine was initialised without BC state"); return GBC_ERR_ARG; }
    const int mode = rq.job == LaneJob::CC ? 0 : (rq.sigma_log ? 2 : 1);
    for (int attempt = 0; attempt < 4; attempt++) {
        KArgs A = LaneAccess::args(*this, rq.semantics);
        GBC_CUDA(cudaMemsetAsync(ctl_, 0, sizeof(Ctl), stream_));
        if (mode == 0) GBC_CUDA(cudaMemsetAsync(ccbuf_, 0, lanes_ * sizeof(unsigned long long), stream_));
        if (mode == 1) GBC_CUDA(cudaMemsetAsync(ovf_, 0, 32 * sizeof(uint32_t), stream_));
        seed_kernel<<<1, 1024, 0, stream_>>>(A, rq.d_src, rq.kb, mode);
        GBC_CUDA(cudaGetLastError());
        res.kernel_launches += 1;
        cudaGraphExec_t fwd;
        GBC_TRY(get_graph(mode, &fwd));
        Ctl* h = (Ctl*)ctl_host_;
        int64_t launched = 0;
        for (;;) {
            GBC_CUDA(cudaGraphLaunch(fwd, stream_));
            res.graph_launches++;
            res.kernel_launches += lpg_;
            launched += lpg_;
            GBC_CUDA(cudaMemcpyAsync(h, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_));
            GBC_CUDA(cudaStreamSynchronize(stream_));
            if (h->done) break;
            if (launched > (int64_t)MAX_LEVEL + 2 * lpg_) { set_error("forward level loop did not terminate"); return GBC_ERR_LIMIT; }
        }
        const int maxlevel = h->maxlevel;
        const unsigned long long entries = std::min<unsigned long long>(h->tail, fcap_);
        if (h->err & 1) {
            // queue overflow: reset the whole lane state, grow the queue, redo the batch
            GBC_CUDA(cudaMemsetAsync(lvl_, 0xFF, (size_t)lanes_ * g_->n * sizeof(uint16_t), stream_));
            GBC_CUDA(cudaMemsetAsync(vmark_, 0xFF, (size_t)ng_ * g_->n * sizeof(int32_t), stream_));
            GBC_CUDA(cudaStreamSynchronize(stream_));
            const unsigned long long maxcap = (unsigned long long)ng_ * g_->n * 32ULL + (1ULL << 16);
            unsigned long long want = std::min(maxcap, std::max(fcap_ * 2, (unsigned long long)h->tail + (1ULL << 20)));
            if (want <= fcap_) { set_error("frontier queue cannot grow"); return GBC_ERR_LIMIT; }
            GBC_TRY(alloc_queue(want));
            continue;
        }
        if (h->err & 2) {
            cleanup_kernel<<<sm_count_ * 4, 256, 0, stream_>>>(A, entries);
            set_error("BFS deeper than %d levels", MAX_LEVEL);
            return GBC_ERR_LIMIT;
        }
        res.levels += maxlevel + 1;
        res.frontier_entries += (int64_t)entries;
        if (rq.job == LaneJob::SSSP) {
            sssp_out_kernel<<<sm_count_ * 8, 256, 0, stream_>>>(A, rq.kb, rq.d_dist, rq.d_sigma);
            GBC_CUDA(cudaGetLastError());
            res.kernel_launches++;
        }
        if (mode == 1) {
            for (int i = 0; i < 32; i++) res.ovf_bits[i] = 0;
            GBC_CUDA(cudaMemcpyAsync(res.ovf_bits, ovf_, ng_ * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
            GBC_CUDA(cudaStreamSynchronize(stream_));
            int cnt = 0;
            for (int i = 0; i < ng_; i++) cnt += __builtin_popcount(res.ovf_bits[i]);
            res.overflow_count += cnt;
            if (cnt && rq.abort_on_overflow) {
                cleanup_kernel<<<sm_count_ * 4, 256, 0, stream_>>>(A, entries);
                GBC_CUDA(cudaGetLastError());
                set_error("exact path counts overflowed uint64 in %d lanes", cnt);
                return GBC_ERR_OVERFLOW;
            }
        }
        if (rq.job == LaneJob::BC && maxlevel >= 1) {
            const int key = 3 + ((rq.sigma_log ? 1 : 0) * 2 + (rq.delta_f64 ? 1 : 0)) * 2 + (rq.semantics == GBC_BC_REFERENCE ? 1 : 0);
            cudaGraphExec_t bwd;
            GBC_TRY(get_graph(key, &bwd));
            bw_begin_kernel<<<1, 1, 0, stream_>>>(A);
            res.kernel_launches++;
            for (int done = 0; done < maxlevel; done += lpg_) {
                GBC_CUDA(cudaGraphLaunch(bwd, stream_));
                res.graph_launches++;
                res.kernel_launches += lpg_;
            }
        }
        if (mode == 0 && rq.d_cc) {
            GBC_CUDA(cudaMemcpyAsync(rq.d_cc, ccbuf_, rq.kb * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, stream_));
        }
        cleanup_kernel<<<sm_count_ * 4, 256, 0, stream_>>>(A, entries);
        GBC_CUDA(cudaGetLastError());
        res.kernel_launches++;
        return GBC_OK;
    }
    set_error("frontier queue overflow persisted");
    return GBC_ERR_LIMIT;
}

}  // namespace gbc
