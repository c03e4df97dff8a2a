// Batched multi-source lane engine for sm_103a: host side, batch set-up and
// reset kernels.  The level kernels and the lane-state layout are described
// in lane_kernels.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "lane_kernels.cuh"

namespace gbc {

namespace {

// One CTA: place each lane's source at level 0 and build F_0.
__global__ void seed_kernel(KArgs A, const int32_t* __restrict__ src, int kb, int mode, int lvl_bytes, int td_only) {
    const int l = threadIdx.x;
    if (A.lcomp && l < (A.ng << A.gs)) {
        const int s = l < kb ? src[l] : -1;
        A.lcomp[l] = (s >= 0 && s < A.n) ? A.vcomp[s] : -1;
    }
    if (l < kb) {
        const int g = l >> A.gs, t = l & ((1 << A.gs) - 1);
        const int s = src[l];
        if (s >= 0 && s < A.n) {
            const size_t i = sidx(g, A.n, s, t, A.gs);
            if (lvl_bytes == 1) reinterpret_cast<uint8_t*>(A.lvl)[i] = 0;
            else reinterpret_cast<uint16_t*>(A.lvl)[i] = 0;
            if (mode == 1) {
                if (A.sig_bytes == 2) reinterpret_cast<uint16_t*>(A.sig)[i] = 1;
                else if (A.sig_bytes == 4) reinterpret_cast<uint32_t*>(A.sig)[i] = 1u;
                else A.sig[i] = 1ULL;
            } else if (mode == 2) {
                A.sig[i] = WONE;
            }
            A.srcw[l] = A.w ? A.w[s] : 1;
            if (A.gs == 0) {
                // one lane per task: every lane's source is its own entry
                A.fq[atomicAdd(&A.ctl->tail, 1ULL)] = ((uint32_t)s << S_LANE_BITS) | (uint32_t)l;
            } else if (atomicExch(&A.vmark[(size_t)g * A.n + s], 0) != 0) {
                const uint32_t ent = ((uint32_t)s << 5) | (uint32_t)g;
                if (is_hub(A, s)) A.hq[atomicAdd(&A.ctl->htail, 1ULL)] = ent;
                else A.fq[atomicAdd(&A.ctl->tail, 1ULL)] = ent;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned long long tail = atomicAdd(&A.ctl->tail, 0ULL);
        const unsigned long long htail = atomicAdd(&A.ctl->htail, 0ULL);
        A.foff[0] = 0;
        A.foff[1] = tail;
        A.hoff[0] = 0;
        A.hoff[1] = htail;
        A.ctl->next = 0;
        A.ctl->hnext = 0;
        A.ctl->level = 0;
        A.ctl->maxlevel = 0;
        A.ctl->done = (tail == 0 && htail == 0);
        A.ctl->err = 0;
        A.ctl->blocks = 0;
        A.ctl->bu = 0;
        A.ctl->td_only = td_only;
        A.ctl->bu_levels = 0;
        A.ctl->fdeg = 0;
        A.ctl->fprev = 0;
        A.ctl->mu = 0;
        A.ctl->bnext = 0;
    }
}

__global__ void bw_begin_kernel(KArgs A) {
    const int L = A.ctl->maxlevel;
    A.ctl->level = L;
    A.ctl->blocks = 0;
    A.ctl->next = A.foff[L];
    A.ctl->hnext = A.hoff[L];
}

// Reset the lane state touched by the batch (every (v,g) of every level).
__global__ void cleanup_kernel(KArgs A, unsigned long long count, unsigned long long hcount, int lvl_bytes) {
    const unsigned long long tid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long total = (count + hcount) << A.gs;
    for (unsigned long long k = tid; k < total; k += stride) {
        const unsigned long long i = k >> A.gs;
        const int t = (int)(k & ((1ULL << A.gs) - 1ULL));
        const uint32_t ent = (i < count) ? A.fq[i] : A.hq[i - count];
        const int v = (int)(ent >> 5), g = (int)(ent & 31u);
        if (lvl_bytes == 1) reinterpret_cast<uint8_t*>(A.lvl)[sidx(g, A.n, v, t, A.gs)] = 0xFFu;
        else reinterpret_cast<uint16_t*>(A.lvl)[sidx(g, A.n, v, t, A.gs)] = 0xFFFFu;
        if (t == 0) A.vmark[(size_t)g * A.n + v] = -1;
    }
}

// Distances and exact counts of lanes [0,kb) into dense [kb][n] arrays.
__global__ void sssp_out_kernel(KArgs A, int kb, int32_t* dist, uint64_t* sigma, int lvl_bytes) {
    const size_t total = (size_t)kb * A.n;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(k / A.n), v = (int)(k % A.n);
        const size_t i = sidx(l >> A.gs, A.n, v, l & ((1 << A.gs) - 1), A.gs);
        int L;
        bool unreached;
        if (lvl_bytes == 1) { L = reinterpret_cast<const uint8_t*>(A.lvl)[i]; unreached = (L == 0xFF); }
        else { L = reinterpret_cast<const uint16_t*>(A.lvl)[i]; unreached = (L == 0xFFFF); }
        if (dist) dist[k] = unreached ? -1 : L;
        if (sigma) {
            const uint64_t sv = A.sig_bytes == 2 ? reinterpret_cast<const uint16_t*>(A.sig)[i]
                              : A.sig_bytes == 4 ? reinterpret_cast<const uint32_t*>(A.sig)[i] : A.sig[i];
            sigma[k] = unreached ? 0ULL : sv;
        }
    }
}

// Level profile of every vertex from the first lane group: (level in lane 0)
// << 16 | (smallest level over lanes 1..31); unreached = all ones.  Used to
// group sources whose BFS levels move together into the same lane group.
__global__ void profile_key_kernel(KArgs A, int lvl_bytes, uint32_t* __restrict__ key) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < A.n; v += gridDim.x * blockDim.x) {
        unsigned l0 = 0xFFFFu, lm = 0xFFFFu;
        for (int t = 0; t < 32; t++) {
            const size_t i = sidx(0, A.n, v, t, A.gs);
            unsigned L = lvl_bytes == 1 ? reinterpret_cast<const uint8_t*>(A.lvl)[i] : reinterpret_cast<const uint16_t*>(A.lvl)[i];
            if (lvl_bytes == 1 && L == 0xFFu) L = 0xFFFFu;
            if (t == 0) l0 = L;
            else lm = min(lm, L);
        }
        key[v] = (l0 << 16) | lm;
    }
}

// *out += number of vertices with more than thr neighbours; whole blocks step
// together so that every lane takes part in the warp sum.
__global__ void count_hubs_kernel(const int64_t* __restrict__ row, int32_t n, int64_t thr, uint32_t* __restrict__ out) {
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = base + threadIdx.x;
        const unsigned c = __reduce_add_sync(0xFFFFFFFFu, (v < n && row[v + 1] - row[v] > thr) ? 1u : 0u);
        if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
    }
}

// *out = 1 when some vertex has more neighbours than the one before it (ids
// not in descending degree order).
__global__ void degree_order_kernel(const int64_t* __restrict__ row, int32_t n, uint32_t* __restrict__ out) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x + 1; v < n; v += (int64_t)gridDim.x * blockDim.x)
        if (row[v + 1] - row[v] > row[v] - row[v - 1]) *out = 1u;
}

// ell[v * q + k / 4] component k % 4 = the k-th neighbour of v, -1 past its degree
// (the one-lane kernels read a vertex's neighbours with q 16-byte loads).
__global__ void ell_build_kernel(const int64_t* __restrict__ row, const int32_t* __restrict__ col, int32_t n, int q,
                                 int32_t* __restrict__ ell) {
    const int w = 4 * q;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)n * w; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = i / w, k = i - v * w;
        const int64_t r0 = row[v], deg = row[v + 1] - r0;
        ell[i] = k < deg ? col[r0 + k] : -1;
    }
}

// bc[v] = sum of the per-32-lane partials, in lane order.
__global__ void bc_reduce_kernel(const double* __restrict__ bcg, int ng, int n, double* __restrict__ bc) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int g = 0; g < ng; g++) s += bcg[(size_t)g * n + v];
        bc[v] = s;
    }
}

constexpr int MAX_LEVEL = Lv<uint16_t>::MAXD;

// One lane per task: bcg[p][v] += the contributions of the lanes of 32-lane
// part p, which the sweep left in the path-count slots of every (vertex, lane)
// it processed (levels 1 and deeper), summed in lane order.  The partials are
// kept per 32 lanes as for lane groups, so served requests can share a batch.
__global__ void lane_bc_reduce_kernel(KArgs A, int lanes) {
    const uint16_t* lv = reinterpret_cast<const uint16_t*>(A.lvl);
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < A.n; v += gridDim.x * blockDim.x) {
        for (int p = 0; p * 32 < lanes; p++) {
            double s = 0.0;
            for (int a = 32 * p; a < min(lanes, 32 * p + 32); a++) {
                const size_t i = (size_t)a * (size_t)A.n + (size_t)v;
                const uint16_t L = lv[i];
                if (L != 0 && L != S_INF) s += __longlong_as_double((long long)A.sig[i]);
            }
            A.bcg[(size_t)p * (size_t)A.n + v] += s;
        }
    }
}

// dst[p][v] += bcg[p][v] for every 32-lane partial p whose destination is set.
// One thread per vertex walks the partials in order, so partials that share a
// destination (one request spanning several of them) never race.
__global__ void bc_scatter_kernel(const double* __restrict__ bcg, int ng, int n, double* const* __restrict__ dst) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        for (int g = 0; g < ng; g++) {
            double* p = dst[g];
            if (p) p[v] += bcg[(size_t)g * n + v];
        }
    }
}

}  // namespace

// Level-kernel tables of the three CTA shapes, filled once.
const LevelKernels& level_kernels(int threads) {
    static const LevelKernels k128 = [] { LevelKernels k{}; level_kernels_128(k); return k; }();
    static const LevelKernels k256 = [] { LevelKernels k{}; level_kernels_256(k); return k; }();
    static const LevelKernels k512 = [] { LevelKernels k{}; level_kernels_512(k); return k; }();
    return threads == 128 ? k128 : threads == 512 ? k512 : k256;
}

// ------------------------------------------------------------------------
struct LaneAccess {
    static KArgs args(const LaneEngine& e, int semantics) {
        KArgs A;
        A.row = e.g_->row; A.col = e.g_->col; A.n = e.g_->n; A.ng = e.ng_;
        A.w = e.g_->w; A.ff = e.g_->ff;
        A.lvl = e.lvl_; A.sig = e.sig_; A.rho = e.rho_; A.vmark = e.vmark_;
        A.fq = e.fq_; A.fcap = e.fcap_; A.foff = e.foff_; A.ctl = (Ctl*)e.ctl_; A.ovf = e.ovf_;
        A.hq = e.hq_; A.hcap = e.hcap_; A.hoff = e.hoff_;
        A.cc = e.ccbuf_; A.bcg = e.bcg_; A.sparse = e.sparse_; A.light = e.light_; A.semantics = semantics;
        A.gs = e.gs_;
        A.hub_deg = e.gs_ == 7 ? HUB_DEG_Q : HUB_DEG;
        A.srcw = e.srcw_;
        A.dir = (e.gs_ == 7 && e.vcomp_) ? 1 : 0;
        A.vcomp = e.vcomp_;
        A.lcomp = e.lcomp_;
        A.done = e.done_;
        A.mtot = (unsigned long long)e.g_->m * (unsigned long long)e.ng_;
        A.hub_lim = e.hub_lim_;
        A.bu_share = (unsigned long long)e.bu_share_;
        A.sig_bytes = e.sig_bytes_;
        A.ell = e.ell_;
        A.ell_q = e.ell_q_;
        return A;
    }
    // Reset the lane state a batch touched: per task when few were touched,
    // else one memset of the level and claim arrays (a 128-lane task rewrites a
    // 128-byte row; on a full R-MAT scale 22 batch the per-task reset wrote
    // 10 GB in 12.5 ms, the memsets write 4.4 GB).
    static void reset(LaneEngine& e, const KArgs& A, unsigned long long entries, unsigned long long hentries) {
        const size_t cells = (size_t)e.lanes_ * e.g_->n;
        if (e.gs_ != 0 && ((entries + hentries) << e.gs_) * 4 < cells) {
            cleanup_kernel<<<e.sm_count_ * 4, 256, 0, e.stream_>>>(A, entries, hentries, e.lvl_bytes_);
        } else {
            cudaMemsetAsync(e.lvl_, 0xFF, cells * e.lvl_bytes_, e.stream_);
            if (e.gs_ != 0) cudaMemsetAsync(e.vmark_, 0xFF, e.vmark_sz_, e.stream_);
        }
    }
};

size_t LaneEngine::bytes_needed(int32_t n, int32_t lanes, bool need_bc, int32_t group) {
    if (group == 1) {   // 16-bit levels, lane-major state, every (vertex, lane) once in the queue
        size_t b = (size_t)lanes * n * (2 + 4) + (size_t)(MAX_LEVEL + 2) * 16 + (1 << 20) + (size_t)n * 32;   // + neighbour table
        if (need_bc) b += (size_t)lanes * n * 16 + (size_t)((lanes + 31) / 32) * n * 8;
        return b;
    }
    const size_t ng = (size_t)lanes / 32;
    size_t b = (size_t)lanes * n * 2 + ng * n * 4 + ng * n * 8 * 4 /*initial queue*/ + (size_t)(MAX_LEVEL + 2) * 8;
    if (need_bc) b += (size_t)lanes * n * 16 + ng * n * 8;
    return b + lanes * 8 + (1 << 20);
}

void LaneEngine::release() {
    for (auto& c : graphs_) if (c.exec) cudaGraphExecDestroy(c.exec);
    graphs_.clear();
    // work on these buffers must be finished before they go back to the cache
    if (stream_) cudaStreamSynchronize(stream_);
    dev_release(lvl_, lvl_sz_);
    dev_release(sig_, sig_sz_);
    dev_release(rho_, rho_sz_);
    dev_release(vmark_, vmark_sz_);
    dev_release(fq_, fcap_ * sizeof(uint32_t));
    dev_release(hq_, hcap_ * sizeof(uint32_t));
    dev_release(bcg_, bcg_sz_);
    fcap_ = hcap_ = 0;
    dev_release(foff_, (MAX_LEVEL + 2) * sizeof(unsigned long long));
    dev_release(hoff_, (MAX_LEVEL + 2) * sizeof(unsigned long long));
    hq_ = nullptr; hoff_ = nullptr;
    dev_release(ctl_, sizeof(Ctl));
    dev_release(ovf_, 32 * sizeof(uint32_t));
    if (ctl_host_) cudaFreeHost(ctl_host_);
    dev_release(ccbuf_, 1024 * sizeof(unsigned long long));
    dev_release(srcw_, 1024 * sizeof(int32_t));
    srcw_ = nullptr;
    dev_release(ell_, ell_sz_);
    ell_ = nullptr;
    ell_q_ = 0;
    ell_sz_ = 0;
    cudaFree(vcomp_);
    cudaFree(lcomp_);
    cudaFree(done_);
    vcomp_ = lcomp_ = nullptr;
    done_ = nullptr;
    done_sz_ = 0;
    lvl_ = nullptr; sig_ = nullptr; rho_ = nullptr; vmark_ = nullptr; fq_ = nullptr; foff_ = nullptr;
    ctl_ = nullptr; ovf_ = nullptr; ctl_host_ = nullptr; bcg_ = nullptr; ccbuf_ = nullptr;
}

LaneEngine::~LaneEngine() {
    release();
    for (auto e : ev_) cudaEventDestroy(e);
}

gbc_status LaneEngine::ensure_events(size_t count) {
    while (ev_.size() < count) {
        cudaEvent_t e;
        GBC_CUDA(cudaEventCreate(&e));
        ev_.push_back(e);
    }
    return GBC_OK;
}

gbc_status LaneEngine::alloc_queue(unsigned long long cap, unsigned long long hcap) {
    if (stream_) cudaStreamSynchronize(stream_);
    dev_release(fq_, fcap_ * sizeof(uint32_t));
    dev_release(hq_, hcap_ * sizeof(uint32_t));
    fq_ = nullptr;
    hq_ = nullptr;
    fcap_ = hcap_ = 0;
    if (dev_alloc((void**)&fq_, cap * sizeof(uint32_t)) != cudaSuccess ||
        dev_alloc((void**)&hq_, hcap * sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        set_error("frontier queue allocation of %llu + %llu entries failed", cap, hcap);
        return GBC_ERR_NOMEM;
    }
    fcap_ = cap;
    hcap_ = hcap;
    for (auto& c : graphs_) if (c.exec) cudaGraphExecDestroy(c.exec);
    graphs_.clear();
    return GBC_OK;
}

gbc_status LaneEngine::init(const DevGraph* g, int32_t lanes, bool need_bc, int sparse_lanes, int levels_per_graph,
                            cudaStream_t stream, int group_lanes) {
    release();
    if (group_lanes != 1 && group_lanes != 32 && group_lanes != 128) { set_error("lanes per group must be 1, 32 or 128"); return GBC_ERR_ARG; }
    const int32_t unit = group_lanes == 1 ? 32 : group_lanes;
    if (lanes < unit || lanes > 1024 || lanes % unit) {
        set_error("lanes must be a multiple of %d in [%d,1024]", unit, unit);
        return GBC_ERR_ARG;
    }
    if (group_lanes == 1 && g->n >= (1 << (32 - S_LANE_BITS))) {
        set_error("one lane per task supports fewer than 2^%d vertices", 32 - S_LANE_BITS);
        return GBC_ERR_ARG;
    }
    if (g->n >= (1 << 27)) { set_error("lane engine supports fewer than 2^27 vertices"); return GBC_ERR_ARG; }
    g_ = g;
    lanes_ = lanes;
    gs_ = group_lanes == 128 ? 7 : group_lanes == 1 ? 0 : 5;
    ng_ = lanes >> gs_;
    need_bc_ = need_bc;
    lvl_bytes_ = (g->level_bytes_hint == 2 || group_lanes == 1) ? 2 : 1;   // one lane per task: 16-bit levels (CAS)
    sig_bytes_ = gs_ == 7 ? g->sigma_bytes_hint : 8;
    set_tuning(sparse_lanes, -1, levels_per_graph);
    stream_ = stream;
    int dev = 0;
    GBC_CUDA(cudaGetDevice(&dev));
    GBC_CUDA(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, dev));
    const size_t n = (size_t)g->n;
    const size_t cells = (size_t)lanes * n;
    bool ok = true;
    lvl_sz_ = cells * sizeof(uint16_t);
    vmark_sz_ = gs_ ? (size_t)ng_ * n * sizeof(int32_t) : sizeof(int32_t);   // one lane per task claims by level CAS
    ok &= dev_alloc((void**)&lvl_, lvl_sz_) == cudaSuccess;
    ok &= dev_alloc((void**)&vmark_, vmark_sz_) == cudaSuccess;
    ok &= dev_alloc((void**)&foff_, (MAX_LEVEL + 2) * sizeof(unsigned long long)) == cudaSuccess;
    ok &= dev_alloc((void**)&hoff_, (MAX_LEVEL + 2) * sizeof(unsigned long long)) == cudaSuccess;
    ok &= dev_alloc((void**)&ctl_, sizeof(Ctl)) == cudaSuccess;
    ok &= dev_alloc((void**)&ovf_, 32 * sizeof(uint32_t)) == cudaSuccess;
    ok &= dev_alloc((void**)&ccbuf_, 1024 * sizeof(unsigned long long)) == cudaSuccess;
    ok &= dev_alloc((void**)&srcw_, 1024 * sizeof(int32_t)) == cudaSuccess;
    // one lane per task on a graph of degree <= 8: a padded neighbour table, so a frontier entry
    // reads its neighbours with one or two 16-byte loads instead of row offsets, then columns
    if (gs_ == 0 && g->max_degree > 0 && g->max_degree <= 8) {
        ell_q_ = g->max_degree <= 4 ? 1 : 2;
        ell_sz_ = (size_t)ell_q_ * n * sizeof(int4);
        ok &= dev_alloc((void**)&ell_, ell_sz_) == cudaSuccess;
    }
    ok &= cudaMallocHost(&ctl_host_, sizeof(Ctl)) == cudaSuccess;
    if (need_bc) {
        sig_sz_ = cells * sizeof(uint64_t);
        rho_sz_ = cells * sizeof(double);
        // BC partials per 32 lanes, for every group width (128-lane groups keep one per quarter)
        bcg_sz_ = (size_t)((lanes + 31) / 32) * n * sizeof(double);
        ok &= dev_alloc((void**)&sig_, sig_sz_) == cudaSuccess;
        ok &= dev_alloc((void**)&rho_, rho_sz_) == cudaSuccess;
        ok &= dev_alloc((void**)&bcg_, bcg_sz_) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        release();
        set_error("lane state allocation failed (n=%zu lanes=%d)", n, lanes);
        return GBC_ERR_NOMEM;
    }
    // hub entries: at most 32 levels' worth per (hub vertex, group) to start with
    {
        uint32_t nh = 0;
        GBC_CUDA(cudaMemsetAsync(ovf_, 0, sizeof(uint32_t), stream_));
        uint32_t unsorted = 0;
        GBC_CUDA(cudaMemsetAsync(ovf_ + 1, 0, sizeof(uint32_t), stream_));
        count_hubs_kernel<<<sm_count_ * 4, 256, 0, stream_>>>(g->row, g->n, gs_ == 7 ? HUB_DEG_Q : HUB_DEG, ovf_);
        GBC_CUDA(cudaGetLastError());
        degree_order_kernel<<<sm_count_ * 4, 256, 0, stream_>>>(g->row, g->n, ovf_ + 1);
        GBC_CUDA(cudaGetLastError());
        GBC_CUDA(cudaMemcpyAsync(&nh, ovf_, sizeof nh, cudaMemcpyDeviceToHost, stream_));
        GBC_CUDA(cudaMemcpyAsync(&unsorted, ovf_ + 1, sizeof unsorted, cudaMemcpyDeviceToHost, stream_));
        GBC_CUDA(cudaStreamSynchronize(stream_));
        n_hubs_ = nh;
        // ids in descending degree order (graphs with hubs): hub <=> id < n_hubs_; no hubs: none
        hub_lim_ = (unsorted && nh > 0) ? -1 : (int)nh;
    }
    if (ell_) {
        ell_build_kernel<<<sm_count_ * 8, 256, 0, stream_>>>(g->row, g->col, g->n, ell_q_, reinterpret_cast<int32_t*>(ell_));
        GBC_CUDA(cudaGetLastError());
    }
    GBC_TRY(alloc_queue(gs_ == 0 ? (unsigned long long)lanes * n + (1ULL << 16) : (unsigned long long)ng_ * n * 8ULL + (1ULL << 16),
                        (unsigned long long)ng_ * n_hubs_ * 8ULL + (1ULL << 12)));
    GBC_CUDA(cudaMemsetAsync(lvl_, 0xFF, cells * sizeof(uint16_t), stream_));
    GBC_CUDA(cudaMemsetAsync(vmark_, 0xFF, vmark_sz_, stream_));
    GBC_CUDA(cudaMemsetAsync(ctl_, 0, sizeof(Ctl), stream_));
    GBC_CUDA(cudaMemsetAsync(ovf_, 0, 32 * sizeof(uint32_t), stream_));
    bytes_ = cells * 2 + vmark_sz_ + (fcap_ + hcap_) * 4 + ell_sz_ + (need_bc ? cells * 16 + bcg_sz_ : 0);
    return GBC_OK;
}


void LaneEngine::set_tuning(int sparse_lanes, int light_steps, int levels_per_graph, int block_threads, int bu_share) {
    const int sp = sparse_lanes < 0 ? 2 : sparse_lanes;
    const int li = light_steps < 0 ? 16 : light_steps;
    // level kernels per captured graph: 16, or 64 on deep graphs (16-bit levels), whose thousands of
    // levels would otherwise cost a graph launch and a host check every 16
    const int lp = levels_per_graph > 0 ? levels_per_graph : (lvl_bytes_ == 2 ? 64 : 16);
    const int bt = (block_threads == 128 || block_threads == 512) ? block_threads : 256;
    const int bs = bu_share < 0 ? 16 : bu_share;
    if (sp == sparse_ && li == light_ && lp == lpg_ && bt == block_ && bs == bu_share_) return;
    sparse_ = sp;
    light_ = li;
    lpg_ = lp;
    block_ = bt;
    bu_share_ = bs;
    for (auto& c : graphs_) if (c.exec) cudaGraphExecDestroy(c.exec);
    graphs_.clear();
}

// Graph keys: forward = MODE + 10 * w; backward = 100 + 20 * w + (wide*2 + f64)*2 + refsem;
// w = path-count width (0: 8 bytes, 1: 4, 2: 2; 128-lane groups only); +1000 with 16-bit levels.
int LaneEngine::width_index() const { return sig_bytes_ == 2 ? 2 : sig_bytes_ == 4 ? 1 : 0; }

gbc_status LaneEngine::get_graph(int key, int count, cudaGraphExec_t* out) {
    const int full = key + 100000 * count;
    for (auto& c : graphs_) if (c.key == full) { *out = c.exec; return GBC_OK; }
    const int lv16 = key >= 1000 ? 1 : 0, k = key % 1000;
    const bool bwd = k >= 100;
    KArgs A = LaneAccess::args(*this, (bwd && ((k - 100) & 1)) ? GBC_BC_REFERENCE : GBC_BC_BRANDES);
    const LevelKernels& K = level_kernels(block_);
    const int w = bwd ? (k - 100) / 20 : k / 10;
    const int v = bwd ? ((k - 100) % 20) >> 1 : k % 10;
    void (*fn)(KArgs) = gs_ == 7 ? (bwd ? K.backward_q[lv16][v][w] : K.expand_q[lv16][v][w])
                      : gs_ == 0 ? (bwd ? K.backward_s[v] : K.expand_s[v])
                                 : (bwd ? K.backward[lv16][v] : K.expand[lv16][v]);
    if (!fn) { set_error("no level kernel for key %d", key); return GBC_ERR_ARG; }
    // one wave: as many CTAs as fit on every SM at once (at most 2048 threads per SM)
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, block_, 0) != cudaSuccess) { cudaGetLastError(); occ = 1; }
    const int grid = sm_count_ * std::max(1, std::min(occ, 2048 / block_));
    cudaStream_t cs;
    GBC_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    for (int i = 0; i < count && e == cudaSuccess; i++) {
        fn<<<grid, block_, 0, cs>>>(A);
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
    if (e == cudaSuccess) e = e2;
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e2 == cudaSuccess) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) { set_error("level-loop graph capture failed: %s", cudaGetErrorString(e)); return GBC_ERR_CUDA; }
    graphs_.push_back({full, exec});
    *out = exec;
    return GBC_OK;
}

namespace {
int pow2_at_least(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}
}  // namespace

gbc_status LaneEngine::bc_begin() {
    if (!need_bc_) { set_error("engine has no BC state"); return GBC_ERR_ARG; }
    GBC_CUDA(cudaMemsetAsync(bcg_, 0, bcg_sz_, stream_));
    return GBC_OK;
}

gbc_status LaneEngine::bc_finish(double* d_bc) {
    bc_reduce_kernel<<<sm_count_ * 4, 256, 0, stream_>>>(bcg_, (lanes_ + 31) / 32, g_->n, d_bc);
    GBC_CUDA(cudaGetLastError());
    return GBC_OK;
}

gbc_status LaneEngine::bc_scatter(double* const* d_dst) {
    bc_scatter_kernel<<<sm_count_ * 8, 256, 0, stream_>>>(bcg_, (lanes_ + 31) / 32, g_->n, d_dst);
    GBC_CUDA(cudaGetLastError());
    return GBC_OK;
}

gbc_status LaneEngine::cc_read(unsigned long long* h_cc, int32_t count) {
    GBC_CUDA(cudaMemcpyAsync(h_cc, ccbuf_, sizeof(unsigned long long) * count, cudaMemcpyDeviceToHost, stream_));
    GBC_CUDA(cudaStreamSynchronize(stream_));
    return GBC_OK;
}

gbc_status LaneEngine::run(const LaneRequest& rq, LaneResult& res) {
    if (rq.kb < 1 || rq.kb > lanes_) { set_error("batch of %d sources for %d lanes", rq.kb, lanes_); return GBC_ERR_ARG; }
    const bool bc = rq.job != LaneJob::CC;
    if (bc && !need_bc_) { set_error("engine was initialised without BC state"); return GBC_ERR_ARG; }
    const int mode = rq.job == LaneJob::CC ? 0 : (rq.sigma_wide ? 2 : 1);
    if (mode == 0 && gs_ == 7 && !vcomp_) {
        // first closeness batch on 128-lane groups: component labels for the bottom-up levels
        const size_t n = (size_t)g_->n;
        done_sz_ = (size_t)ng_ * ((n + 31) / 32) * sizeof(uint32_t);
        if (cudaMalloc(&vcomp_, sizeof(int32_t) * std::max<size_t>(n, 1)) != cudaSuccess ||
            cudaMalloc(&lcomp_, sizeof(int32_t) * 1024) != cudaSuccess || cudaMalloc(&done_, std::max<size_t>(done_sz_, 4)) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(vcomp_); cudaFree(lcomp_); cudaFree(done_);
            vcomp_ = lcomp_ = nullptr;
            done_ = nullptr;
            set_error("bottom-up state allocation");
            return GBC_ERR_NOMEM;
        }
        GBC_TRY(component_labels(g_->row, g_->col, g_->n, stream_, vcomp_));
        for (auto& c : graphs_) if (c.exec) cudaGraphExecDestroy(c.exec);
        graphs_.clear();   // captured level loops hold the arguments without these buffers
    }
    // retries: a queue overflow (grown up to its bound, below), a level-width switch, a sigma re-run
    for (int attempt = 0; attempt < 8; attempt++) {
        res.level_entries.clear();
        res.fwd_launch_ms.clear();
        res.bwd_launch_ms.clear();
        KArgs A = LaneAccess::args(*this, rq.semantics);
        GBC_CUDA(cudaMemsetAsync(ctl_, 0, sizeof(Ctl), stream_));
        if (mode == 0) GBC_CUDA(cudaMemsetAsync(ccbuf_, 0, lanes_ * sizeof(unsigned long long), stream_));
        if (mode != 0) GBC_CUDA(cudaMemsetAsync(ovf_, 0, 32 * sizeof(uint32_t), stream_));
        if (mode == 0 && done_) GBC_CUDA(cudaMemsetAsync(done_, 0, done_sz_, stream_));
        seed_kernel<<<1, 1024, 0, stream_>>>(A, rq.d_src, rq.kb, mode, lvl_bytes_, rq.top_down_only ? 1 : 0);
        GBC_CUDA(cudaGetLastError());
        res.kernel_launches += 1;
        cudaGraphExec_t fwd;
        const int lv16 = (lvl_bytes_ == 2) ? 1000 : 0;
        const int wi = mode == 1 ? width_index() : 0;
        // the first graph as long as the last batch needed (levels + the launch that finds the
        // next frontier empty), so shallow graphs launch few level kernels past their depth;
        // later graphs lpg_ long
        int count = depth_hint_ > 0 ? std::min(lpg_, pow2_at_least(depth_hint_ + 1)) : lpg_;
        Ctl* h = (Ctl*)ctl_host_;
        int64_t launched = 0;
        GBC_TRY(ensure_events(2));
        for (;;) {
            GBC_TRY(get_graph(lv16 + mode + 10 * wi, count, &fwd));
            GBC_CUDA(cudaEventRecord(ev_[0], stream_));
            GBC_CUDA(cudaGraphLaunch(fwd, stream_));
            GBC_CUDA(cudaEventRecord(ev_[1], stream_));
            res.graph_launches++;
            res.kernel_launches += count;
            res.fwd_kernels += count;
            launched += count;
            count = lpg_;
            GBC_CUDA(cudaMemcpyAsync(h, ctl_, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_));
            GBC_CUDA(cudaStreamSynchronize(stream_));
            float ms = 0;
            cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
            res.fwd_ms += ms;
            res.fwd_launch_ms.push_back(ms);
            if (h->done) break;
            if (h->any_ovf && rq.abort_on_overflow) break;   // the batch is redone in wide form anyway
            if (launched > (int64_t)MAX_LEVEL + 2 * lpg_) { set_error("forward level loop did not terminate"); return GBC_ERR_LIMIT; }
        }
        const int maxlevel = h->maxlevel;
        depth_hint_ = maxlevel;
        const unsigned long long entries = std::min<unsigned long long>(h->tail, fcap_);
        const unsigned long long hentries = std::min<unsigned long long>(h->htail, hcap_);
        if (h->err & 1) {
            // queue overflow: reset the whole lane state, grow the queue, redo the batch
            GBC_CUDA(cudaMemsetAsync(lvl_, 0xFF, (size_t)lanes_ * g_->n * sizeof(uint16_t), stream_));
            GBC_CUDA(cudaMemsetAsync(vmark_, 0xFF, vmark_sz_, stream_));
            GBC_CUDA(cudaStreamSynchronize(stream_));
            // a (vertex, group) task recurs at most once per lane of its group.  Grow 4x: on
            // deep graphs with 128-lane groups a task recurs at up to 128 levels, and the
            // forward pass stops at the overflowing level, so its tail understates the need
            const unsigned long long maxcap = (unsigned long long)lanes_ * g_->n + (1ULL << 16);
            const unsigned long long hmax = (unsigned long long)lanes_ * n_hubs_ + (1ULL << 12);
            const unsigned long long want = std::min(maxcap, std::max(fcap_ * 4, (unsigned long long)h->tail + (1ULL << 20)));
            const unsigned long long hwant = std::min(hmax, std::max(hcap_ * 4, (unsigned long long)h->htail + (1ULL << 12)));
            if (want <= fcap_ && hwant <= hcap_) { set_error("frontier queue cannot grow"); return GBC_ERR_LIMIT; }
            GBC_TRY(alloc_queue(std::max(want, fcap_), std::max(hwant, hcap_)));
            continue;
        }
        if (h->err & 2) {
            if (lvl_bytes_ == 1) {
                // deeper than 8-bit levels allow: switch this engine to 16-bit levels, redo
                lvl_bytes_ = 2;
                g_->level_bytes_hint = 2;
                GBC_CUDA(cudaMemsetAsync(lvl_, 0xFF, (size_t)lanes_ * g_->n * sizeof(uint16_t), stream_));
                GBC_CUDA(cudaMemsetAsync(vmark_, 0xFF, vmark_sz_, stream_));
                GBC_CUDA(cudaStreamSynchronize(stream_));
                continue;
            }
            LaneAccess::reset(*this, A, entries, hentries);
            set_error("BFS deeper than %d levels", MAX_LEVEL);
            return GBC_ERR_LIMIT;
        }
        if (mode == 1 && sig_bytes_ < 8 && h->any_ovf) {
            // a path count passed the narrow width: widen (for later batches on this graph too), redo
            sig_bytes_ = sig_bytes_ == 2 ? 4 : 8;
            g_->sigma_bytes_hint = sig_bytes_;
            LaneAccess::reset(*this, A, entries, hentries);
            GBC_CUDA(cudaGetLastError());
            res.kernel_launches++;
            continue;
        }
        res.sigma_bytes = mode == 1 ? sig_bytes_ : 8;
        res.levels += maxlevel + 1;
        res.bottom_up_levels += h->bu_levels;
        res.neighbour_visits += (int64_t)h->visits;
        {
            // frontier entries of every level of this batch: foff / hoff hold the level bounds
            std::vector<unsigned long long> fo(maxlevel + 2), ho(maxlevel + 2);
            GBC_CUDA(cudaMemcpyAsync(fo.data(), foff_, sizeof(unsigned long long) * (maxlevel + 2), cudaMemcpyDeviceToHost, stream_));
            GBC_CUDA(cudaMemcpyAsync(ho.data(), hoff_, sizeof(unsigned long long) * (maxlevel + 2), cudaMemcpyDeviceToHost, stream_));
            GBC_CUDA(cudaStreamSynchronize(stream_));
            res.level_entries.resize(maxlevel + 1);
            for (int dl = 0; dl <= maxlevel; dl++)
                res.level_entries[dl] = (int64_t)(fo[dl + 1] - fo[dl]) + (int64_t)(ho[dl + 1] - ho[dl]);
        }
        res.frontier_entries += (int64_t)(entries + hentries);
        if (rq.d_profile_key) {
            profile_key_kernel<<<sm_count_ * 8, 256, 0, stream_>>>(A, lvl_bytes_, rq.d_profile_key);
            GBC_CUDA(cudaGetLastError());
            res.kernel_launches++;
        }
        if (rq.job == LaneJob::SSSP) {
            sssp_out_kernel<<<sm_count_ * 8, 256, 0, stream_>>>(A, rq.kb, rq.d_dist, rq.d_sigma, lvl_bytes_);
            GBC_CUDA(cudaGetLastError());
            res.kernel_launches++;
        }
        if (mode == 1) {
            for (int i = 0; i < 32; i++) res.ovf_bits[i] = 0;
            GBC_CUDA(cudaMemcpyAsync(res.ovf_bits, ovf_, (lanes_ / 32) * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
            GBC_CUDA(cudaStreamSynchronize(stream_));
            int cnt = 0;
            for (int i = 0; i < lanes_ / 32; i++) cnt += __builtin_popcount(res.ovf_bits[i]);
            res.overflow_count += cnt;
            if (cnt && rq.abort_on_overflow) {
                LaneAccess::reset(*this, A, entries, hentries);
                GBC_CUDA(cudaGetLastError());
                set_error("exact path counts overflowed uint64 in %d lanes", cnt);
                return GBC_ERR_OVERFLOW;
            }
        } else if (mode == 2) {
            uint32_t bits[32] = {};
            GBC_CUDA(cudaMemcpyAsync(bits, ovf_, (lanes_ / 32) * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
            GBC_CUDA(cudaStreamSynchronize(stream_));
            int cnt = 0;
            for (int i = 0; i < lanes_ / 32; i++) cnt += __builtin_popcount(bits[i]);
            if (cnt) {
                LaneAccess::reset(*this, A, entries, hentries);
                GBC_CUDA(cudaGetLastError());
                set_error("path counts exceed 2^524287 in %d lanes", cnt);
                return GBC_ERR_OVERFLOW;
            }
        }
        if (rq.job == LaneJob::BC && maxlevel >= 1) {
            const int key = lv16 + 100 + 20 * wi + ((rq.sigma_wide ? 1 : 0) * 2 + (rq.delta_f64 ? 1 : 0)) * 2 +
                            (rq.semantics == GBC_BC_REFERENCE ? 1 : 0);
            // the sweep runs levels maxlevel .. 1: graphs of lpg_ level kernels, then one of the
            // power of two that covers the rest
            const int nfull = maxlevel / lpg_, rest = maxlevel % lpg_;
            const int nl = nfull + (rest ? 1 : 0);
            cudaGraphExec_t bwd_full = nullptr, bwd_rest = nullptr;
            if (nfull) GBC_TRY(get_graph(key, lpg_, &bwd_full));
            if (rest) GBC_TRY(get_graph(key, pow2_at_least(rest), &bwd_rest));
            bw_begin_kernel<<<1, 1, 0, stream_>>>(A);
            res.kernel_launches++;
            GBC_TRY(ensure_events(2 * nl));
            for (int i = 0; i < nl; i++) {
                const bool last_rest = rest && i == nfull;
                const int cnt = last_rest ? pow2_at_least(rest) : lpg_;
                GBC_CUDA(cudaEventRecord(ev_[2 * i], stream_));
                GBC_CUDA(cudaGraphLaunch(last_rest ? bwd_rest : bwd_full, stream_));
                GBC_CUDA(cudaEventRecord(ev_[2 * i + 1], stream_));
                res.graph_launches++;
                res.kernel_launches += cnt;
                res.bwd_kernels += cnt;
            }
            GBC_CUDA(cudaStreamSynchronize(stream_));
            for (int i = 0; i < nl; i++) {
                float ms = 0;
                cudaEventElapsedTime(&ms, ev_[2 * i], ev_[2 * i + 1]);
                res.bwd_ms += ms;
                res.bwd_launch_ms.push_back(ms);
            }
        }
        if (rq.job == LaneJob::BC && gs_ == 0 && maxlevel >= 1) {
            lane_bc_reduce_kernel<<<sm_count_ * 8, 256, 0, stream_>>>(A, lanes_);
            GBC_CUDA(cudaGetLastError());
            res.kernel_launches++;
        }
        if (mode == 0 && rq.d_cc) {
            GBC_CUDA(cudaMemcpyAsync(rq.d_cc, ccbuf_, rq.kb * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, stream_));
        }
        LaneAccess::reset(*this, A, entries, hentries);
        GBC_CUDA(cudaGetLastError());
        res.kernel_launches++;
        return GBC_OK;
    }
    set_error("frontier queue overflow persisted");
    return GBC_ERR_LIMIT;
}

}  // namespace gbc
