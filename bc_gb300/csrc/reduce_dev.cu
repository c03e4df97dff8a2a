// D1 folding and biconnected blocks on the device.
//
// Folding (the peeling of Lib/D1Process/D1Process.c:32-73) runs in rounds:
// round k folds every vertex whose live degree is 1 at the start of the round
// into its one live neighbour p (r[p] += r[u], ff[p] += r[u] + ff[u], integer
// atomics, so the sums do not depend on the order); a vertex whose degree
// drops to 1 is a leaf of round k+1.  A vertex never receives a fold in the
// round it folds in (it would have two live neighbours), so r[u] and ff[u]
// are final when u folds.  Two leaves that are each other's live neighbour
// are the last two vertices of a tree component: the larger id folds into
// the smaller one, which stays as the component's root.
//
// Blocks (the articulation points and parts of Lib/AP_Process/AP_Process.c)
// follow Tarjan and Vishkin's parallel biconnectivity, which works on any
// rooted spanning forest:
//   * components by union-find (roots hooked under smaller roots, so each
//     set ends at its smallest vertex, which becomes the tree root);
//   * a BFS forest from those roots; parent = first neighbour, in row order,
//     one level up (deterministic);
//   * subtree sizes nd (bottom-up by level), preorder numbers pre (top-down:
//     children in row order), low/high = min/max of pre over a subtree and
//     its non-tree neighbours (bottom-up);
//   * tree edges are named by their child vertex c and joined by union-find:
//     (a) a non-tree edge u-w between unrelated vertices joins c=u and c=w;
//     (b) the edge into c joins the edge into its parent v (v not a root) when
//         low(c) < pre(v) or high(c) >= pre(v) + nd(v).
//     Each resulting set is one block; a non-tree edge belongs to the block of
//     the tree edge into its endpoint with the larger preorder number.
// A vertex is an articulation point when the tree edges at it lie in two or
// more blocks.  Slots are the distinct (block, vertex) pairs, sorted as
// 64-bit keys; the block graph is every core entry mapped to its block's
// slots, sorted.  All integer work: the result does not depend on thread
// timing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cub/cub.cuh>
#include <memory>

#include "engine.h"
#include "reduce.h"

namespace gbc {

namespace {

constexpr int RB = 256;
constexpr unsigned FULLM = 0xFFFFFFFFu;
constexpr int UF_TRIES = 1 << 22;   // union retries before a kernel reports failure (never reached in practice)

int grid_threads(int64_t items) { return (int)std::max<int64_t>(1, std::min<int64_t>((items + RB - 1) / RB, 152 * 32)); }
int grid_warps(int64_t items) { return grid_threads(items * 32); }

template <typename T>
struct DBuf {
    T* p = nullptr;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { if (p) cudaFree(p); }
    bool alloc(size_t k) {
        if (p) { cudaFree(p); p = nullptr; }
        if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(k, 1)) != cudaSuccess) { cudaGetLastError(); p = nullptr; return false; }
        return true;
    }
};

#define RD_ALLOC(buf, k)                                               \
    do {                                                               \
        if (!(buf).alloc(k)) { set_error("reduction: device allocation of %s", #buf); return GBC_ERR_NOMEM; } \
    } while (0)

// Warp-aggregated append of `val` where `pred`; all 32 lanes call it.
__device__ __forceinline__ void warp_push(int32_t* q, unsigned* qn, bool pred, int32_t val) {
    const unsigned m = __ballot_sync(FULLM, pred);
    if (!m) return;
    const int t = threadIdx.x & 31;
    unsigned base = 0;
    if (t == __ffs(m) - 1) base = atomicAdd(qn, (unsigned)__popc(m));
    base = __shfl_sync(FULLM, base, __ffs(m) - 1);
    if (pred) q[base + __popc(m & ((1u << t) - 1u))] = val;
}

// Union-find with every link pointing to a smaller id, so walks end.
__device__ __forceinline__ int32_t uf_find(int32_t* uf, int32_t x) {
    for (;;) {
        const int32_t p = *(volatile int32_t*)&uf[x];
        if (p == x) return x;
        const int32_t g = *(volatile int32_t*)&uf[p];
        if (g != p) *(volatile int32_t*)&uf[x] = g;   // path halving; g is an ancestor either way
        x = g;
    }
}

__device__ __forceinline__ void uf_union(int32_t* uf, int32_t a, int32_t b, int* err) {
    for (int it = 0; it < UF_TRIES; it++) {
        a = uf_find(uf, a);
        b = uf_find(uf, b);
        if (a == b) return;
        if (a > b) { const int32_t t = a; a = b; b = t; }
        if (atomicCAS(&uf[b], b, a) == b) return;
    }
    atomicExch(err, 1);
}

// ------------------------------------------------------------- CSR checks --
// bad[0] = smallest v with row[v+1] < row[v], bad[1] = smallest e with col[e]
// outside [0, n) (0xFFFFFFFF: none).  Whole blocks step together so that every
// lane takes part in the warp minimum.
__global__ void csr_entries_check_kernel(const int64_t* __restrict__ row, const int32_t* __restrict__ col, int32_t n,
                                         int64_t m, unsigned* __restrict__ bad) {
    const int64_t len = (int64_t)n > m ? (int64_t)n : m;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < len; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        unsigned br = ~0u, bc = ~0u;
        if (i < n && row[i + 1] < row[i]) br = (unsigned)i;
        if (i < m && (uint32_t)col[i] >= (uint32_t)n) bc = (unsigned)i;
        br = __reduce_min_sync(FULLM, br);
        bc = __reduce_min_sync(FULLM, bc);
        if ((threadIdx.x & 31) == 0) {
            if (br != ~0u) atomicMin(&bad[0], br);
            if (bc != ~0u) atomicMin(&bad[1], bc);
        }
    }
}

// bad[2] = smallest v that lists itself (rows already known to be monotone)
__global__ void self_loop_check_kernel(const int64_t* __restrict__ row, const int32_t* __restrict__ col, int32_t n,
                                       unsigned* __restrict__ bad) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += nw) {
        bool loop = false;
        for (int64_t j = row[v] + t; j < row[v + 1]; j += 32) loop |= col[j] == v;
        if (__any_sync(FULLM, loop) && t == 0) atomicMin(&bad[2], (unsigned)v);
    }
}

// ---------------------------------------------------------------- folding --
__global__ void fold_init_kernel(const int64_t* __restrict__ row, int32_t n, int32_t start, int32_t* __restrict__ deg,
                                 uint8_t* __restrict__ alive, int32_t* __restrict__ fround, int32_t* __restrict__ parent,
                                 int32_t* __restrict__ cand, unsigned long long* __restrict__ r,
                                 unsigned long long* __restrict__ ff, int32_t* __restrict__ q, unsigned* __restrict__ qn) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); b < n; b += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = (int32_t)(b + (threadIdx.x & 31));
        bool leaf = false;
        if (v < n) {
            const int32_t d = v >= start ? (int32_t)(row[v + 1] - row[v]) : 0;
            deg[v] = d;
            alive[v] = v >= start;
            fround[v] = -1;
            parent[v] = -1;
            cand[v] = -1;
            r[v] = 1;
            ff[v] = 0;
            leaf = v >= start && d == 1;
        }
        warp_push(q, qn, leaf, v);
    }
}

// cand[u] = round for the leaves of this round
__global__ void fold_mark_kernel(const int32_t* __restrict__ q, unsigned cnt, const int32_t* __restrict__ deg,
                                 int32_t* __restrict__ cand, int32_t round) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const int32_t u = q[i];
        if (deg[u] == 1) cand[u] = round;
    }
}

__global__ void fold_step_kernel(const int64_t* __restrict__ row, const int32_t* __restrict__ col,
                                 const int32_t* __restrict__ q, unsigned cnt, int32_t* __restrict__ deg,
                                 uint8_t* __restrict__ alive, const int32_t* __restrict__ cand, int32_t round,
                                 int32_t* __restrict__ parent, int32_t* __restrict__ fround,
                                 unsigned long long* __restrict__ r, unsigned long long* __restrict__ ff,
                                 int32_t* __restrict__ nq, unsigned* __restrict__ nqn) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); b < cnt; b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = b + (threadIdx.x & 31);
        bool push = false;
        int32_t p = -1;
        if (i < cnt) {
            const int32_t u = q[i];
            if (cand[u] == round) {
                for (int64_t e = row[u]; e < row[u + 1]; e++) {
                    const int32_t w = col[e];
                    if (*(volatile uint8_t*)&alive[w]) { p = w; break; }
                }
                // p < 0: u's partner of a last pair folded into u first
                if (p >= 0 && (cand[p] != round || u > p)) {
                    parent[u] = p;
                    fround[u] = round;
                    alive[u] = 0;
                    deg[u] = 0;
                    const unsigned long long ru = r[u];
                    atomicAdd(&r[p], ru);
                    atomicAdd(&ff[p], ru + ff[u]);
                    push = atomicSub(&deg[p], 1) == 2;
                }
            }
        }
        warp_push(nq, nqn, push, p);
    }
}

// ------------------------------------------------------------ core graph --
__global__ void alive_i32_kernel(const uint8_t* __restrict__ alive, int32_t n, int32_t* __restrict__ a) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) a[v] = alive[v];
}

__global__ void core_ids_kernel(const uint8_t* __restrict__ alive, const int32_t* __restrict__ cid,
                                const int32_t* __restrict__ deg, int32_t n, int32_t* __restrict__ core_v,
                                int64_t* __restrict__ cdeg) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (alive[v]) {
            core_v[cid[v]] = v;
            cdeg[cid[v]] = deg[v];
        }
}

// one warp per core vertex: its live neighbours in row order, in core ids
__global__ void core_fill_kernel(const int64_t* __restrict__ row, const int32_t* __restrict__ col,
                                 const uint8_t* __restrict__ alive, const int32_t* __restrict__ cid,
                                 const int32_t* __restrict__ core_v, const int64_t* __restrict__ crow, int32_t nc,
                                 int32_t* __restrict__ ccol, int* err) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nc; i += nw) {
        const int32_t v = core_v[i];
        int64_t out = crow[i];
        for (int64_t jb = row[v]; jb < row[v + 1]; jb += 32) {
            const int64_t j = jb + t;
            const int32_t w = j < row[v + 1] ? col[j] : 0;
            const bool a = j < row[v + 1] && alive[w];
            const unsigned m = __ballot_sync(FULLM, a);
            const int64_t o = out + __popc(m & ((1u << t) - 1u));
            if (a && o < crow[i + 1]) ccol[o] = cid[w];
            out += __popc(m);
        }
        // a live degree that differs from the live neighbours found: the CSR is not symmetric
        if (t == 0 && out != crow[i + 1]) atomicExch(err, 2);
    }
}

// ----------------------------------------------------- spanning forest --
__global__ void iota_kernel(int32_t* __restrict__ a, int32_t n) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) a[v] = v;
}

// union of the endpoints of every entry (one warp per vertex)
__global__ void cc_union_kernel(const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol, int32_t nc,
                                int32_t* uf, int* err) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nc; u += nw)
        for (int64_t j = crow[u] + t; j < crow[u + 1]; j += 32) {
            const int32_t w = ccol[j];
            if (w > u) uf_union(uf, (int32_t)u, w, err);
        }
}

// Link every vertex with its first two neighbours (one warp per vertex): on a
// power-law graph this forms most of the giant component with little
// contention, so that the full pass below mostly finds equal roots at once.
__global__ void cc_link_sample_kernel(const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol, int32_t nc,
                                      int32_t* uf, int* err) {
    for (int32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nc; u += gridDim.x * blockDim.x)
        for (int64_t j = crow[u]; j < crow[u + 1] && j < crow[u] + 2; j++) uf_union(uf, u, ccol[j], err);
}

// uf[v] = root of v, in place (no unions run meanwhile, so the roots are fixed)
__global__ void uf_compress_kernel(int32_t* uf, int32_t nc) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nc; v += gridDim.x * blockDim.x) uf[v] = uf_find(uf, v);
}

// lab[v] = smallest vertex of v's set; roots[v] = 1 for the smallest vertices
__global__ void uf_flatten_kernel(int32_t* uf, int32_t nc, int32_t* __restrict__ lab, int32_t* __restrict__ isroot) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nc; v += gridDim.x * blockDim.x) {
        const int32_t l = uf_find(uf, v);
        lab[v] = l;
        if (isroot) isroot[v] = (l == v);
    }
}

__global__ void forest_init_kernel(const int32_t* __restrict__ lab, const int32_t* __restrict__ cpos, int32_t nc,
                                   int32_t* __restrict__ comp, int32_t* __restrict__ level, int32_t* __restrict__ parent,
                                   int32_t* __restrict__ nd, int32_t* __restrict__ pre, int32_t* __restrict__ q) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nc; v += gridDim.x * blockDim.x) {
        const int32_t l = lab[v];
        comp[v] = cpos[l];
        const bool root = l == v;
        level[v] = root ? 0 : -1;
        parent[v] = -1;
        nd[v] = 1;
        pre[v] = 0;
        if (root) q[cpos[v]] = v;   // level 0 of the BFS order: the roots, by id
    }
}

// one warp per frontier vertex: claim unreached neighbours for level L+1
__global__ void bfs_level_kernel(const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                                 const int32_t* __restrict__ q, unsigned cnt, int32_t L, int32_t* level,
                                 int32_t* __restrict__ nq, unsigned* __restrict__ nqn) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += nw) {
        const int32_t u = q[i];
        for (int64_t jb = crow[u]; jb < crow[u + 1]; jb += 32) {
            const int64_t j = jb + t;
            bool got = false;
            int32_t w = 0;
            if (j < crow[u + 1]) {
                w = ccol[j];
                got = *(volatile int32_t*)&level[w] < 0 && atomicCAS(&level[w], -1, L + 1) == -1;
            }
            warp_push(nq, nqn, got, w);
        }
    }
}

// parent = first neighbour in row order one level up (one warp per vertex)
__global__ void parent_kernel(const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                              const int32_t* __restrict__ level, int32_t nc, int32_t* __restrict__ parent, int* err) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nc; v += nw) {
        const int32_t lv = level[v];
        if (lv == 0) continue;
        bool found = false;
        for (int64_t jb = crow[v]; jb < crow[v + 1]; jb += 32) {
            const int64_t j = jb + t;
            const int32_t w = j < crow[v + 1] ? ccol[j] : 0;
            const unsigned m = __ballot_sync(FULLM, j < crow[v + 1] && level[w] == lv - 1);
            if (m) {
                if (t == __ffs(m) - 1) parent[v] = w;
                found = true;
                break;
            }
        }
        if (!found && t == 0) atomicExch(err, 3);   // reached from a vertex it does not list
    }
}

__global__ void nd_up_kernel(const int32_t* __restrict__ q, unsigned cnt, const int32_t* __restrict__ parent,
                             int32_t* nd) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const int32_t v = q[i], p = parent[v];
        if (p >= 0) atomicAdd(&nd[p], nd[v]);
    }
}

// preorder numbers of the children of one level (one warp per vertex, children in row order)
__global__ void pre_down_kernel(const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                                const int32_t* __restrict__ q, unsigned cnt, const int32_t* __restrict__ parent,
                                const int32_t* __restrict__ nd, int32_t* pre) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += nw) {
        const int32_t v = q[i];
        int32_t next = pre[v] + 1;
        for (int64_t jb = crow[v]; jb < crow[v + 1]; jb += 32) {
            const int64_t j = jb + t;
            const int32_t w = j < crow[v + 1] ? ccol[j] : 0;
            const bool child = j < crow[v + 1] && parent[w] == v;
            int32_t x = child ? nd[w] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(FULLM, x, o);
                if (t >= o) x += y;
            }
            if (child) pre[w] = next + x - nd[w];
            next += __shfl_sync(FULLM, x, 31);
        }
    }
}

// low/high of each vertex over itself and its non-tree neighbours (one warp per vertex)
__global__ void lohi_local_kernel(const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                                  const int32_t* __restrict__ parent, const int32_t* __restrict__ pre, int32_t nc,
                                  int32_t* __restrict__ lo, int32_t* __restrict__ hi) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nc; v += nw) {
        int32_t a = pre[v], z = pre[v];
        const int32_t pv = parent[v];
        for (int64_t j = crow[v] + t; j < crow[v + 1]; j += 32) {
            const int32_t w = ccol[j];
            if (w == pv || parent[w] == v) continue;
            a = min(a, pre[w]);
            z = max(z, pre[w]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = min(a, __shfl_xor_sync(FULLM, a, o));
            z = max(z, __shfl_xor_sync(FULLM, z, o));
        }
        if (t == 0) { lo[v] = a; hi[v] = z; }
    }
}

__global__ void lohi_up_kernel(const int32_t* __restrict__ q, unsigned cnt, const int32_t* __restrict__ parent,
                               int32_t* lo, int32_t* hi) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const int32_t v = q[i], p = parent[v];
        if (p < 0) continue;
        atomicMin(&lo[p], lo[v]);
        atomicMax(&hi[p], hi[v]);
    }
}

// The two joining rules over tree edges (named by their child vertex).
// (b): the edge into u joins the edge into its parent (one per vertex); run
// first, so that the many cross edges of rule (a) mostly find equal roots.
__global__ void tv_union_tree_kernel(const int32_t* __restrict__ parent, const int32_t* __restrict__ pre,
                                     const int32_t* __restrict__ nd, const int32_t* __restrict__ lo,
                                     const int32_t* __restrict__ hi, int32_t nc, int32_t* uf, int* err) {
    for (int32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nc; u += gridDim.x * blockDim.x) {
        const int32_t pu = parent[u];
        if (pu >= 0 && parent[pu] >= 0) {
            const int32_t pv = pre[pu];
            if (lo[u] < pv || hi[u] >= pv + nd[pu]) uf_union(uf, u, pu, err);
        }
    }
}

// (a): a non-tree edge between unrelated endpoints joins the edges into both (one warp per vertex)
__global__ void tv_union_cross_kernel(const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                                      const int32_t* __restrict__ parent, const int32_t* __restrict__ pre,
                                      const int32_t* __restrict__ nd, int32_t nc, int32_t* uf, int* err) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nc; u += nw) {
        const int32_t pu = parent[u], preu = pre[u], ndu = nd[u];
        for (int64_t j = crow[u] + t; j < crow[u + 1]; j += 32) {
            const int32_t w = ccol[j];
            if (w == pu || parent[w] == u) continue;
            const int32_t pw = pre[w];
            if (pw > preu && pw >= preu + ndu) uf_union(uf, (int32_t)u, w, err);
        }
    }
}

// articulation points, and slot key counts per vertex (one warp per vertex)
__global__ void ap_kernel(const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                          const int32_t* __restrict__ parent, const int32_t* __restrict__ blab, int32_t nc,
                          uint8_t* __restrict__ ap, int32_t* __restrict__ nkeys) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nc; v += nw) {
        const int32_t pv = parent[v];
        int32_t a = pv >= 0 ? blab[v] : INT32_MAX, z = pv >= 0 ? blab[v] : -1;
        for (int64_t j = crow[v] + t; j < crow[v + 1]; j += 32) {
            const int32_t w = ccol[j];
            if (parent[w] != v) continue;
            a = min(a, blab[w]);
            z = max(z, blab[w]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = min(a, __shfl_xor_sync(FULLM, a, o));
            z = max(z, __shfl_xor_sync(FULLM, z, o));
        }
        if (t == 0) {
            ap[v] = z >= 0 && a != z;
            // the edge into v gives slots (block, v) and (block, parent); an isolated vertex is its own block
            nkeys[v] = pv >= 0 ? 2 : (crow[v + 1] == crow[v] ? 1 : 0);
        }
    }
}

__global__ void slot_keys_kernel(const int32_t* __restrict__ parent, const int32_t* __restrict__ blab,
                                 const int32_t* __restrict__ kpos, const int32_t* __restrict__ nkeys, int32_t nc,
                                 uint64_t* __restrict__ keys) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nc; v += gridDim.x * blockDim.x) {
        const int32_t k = nkeys[v], o = kpos[v];
        if (k == 2) {
            const uint64_t hi = (uint64_t)(uint32_t)blab[v] << 32;
            keys[o] = hi | (uint32_t)v;
            keys[o + 1] = hi | (uint32_t)parent[v];
        } else if (k == 1) {
            keys[o] = ((uint64_t)(uint32_t)v << 32) | (uint32_t)v;
        }
    }
}

__global__ void block_flags_kernel(const uint64_t* __restrict__ skeys, int32_t ns, int32_t* __restrict__ flag) {
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x)
        flag[s] = s == 0 || (skeys[s] >> 32) != (skeys[s - 1] >> 32);
}

__global__ void slots_kernel(const uint64_t* __restrict__ skeys, const int32_t* __restrict__ flag,
                             const int32_t* __restrict__ bid, int32_t ns, int32_t* __restrict__ slot_core,
                             int64_t* __restrict__ bvoff, int32_t* __restrict__ blk_of_lab, int32_t* vslot) {
    for (int32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const uint64_t k = skeys[s];
        const int32_t v = (int32_t)(uint32_t)k;
        slot_core[s] = v;
        atomicMin(&vslot[v], s);
        if (flag[s]) {
            bvoff[bid[s]] = s;
            blk_of_lab[(int32_t)(k >> 32)] = bid[s];
        }
    }
}

__global__ void fill_i32_kernel(int32_t* __restrict__ a, int64_t n, int32_t val) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = val;
}

__device__ __forceinline__ int32_t slot_in(const int32_t* __restrict__ slot_core, const int64_t* __restrict__ bvoff,
                                           const int32_t* __restrict__ vslot, const uint8_t* __restrict__ ap, int32_t b,
                                           int32_t v) {
    if (!ap[v]) return vslot[v];
    const int64_t end = bvoff[b + 1];
    int64_t a = bvoff[b], z = end;   // slots of block b, ascending core ids
    while (a < z) {
        const int64_t m = (a + z) >> 1;
        if (slot_core[m] < v) a = m + 1;
        else z = m;
    }
    return a < end && slot_core[a] == v ? (int32_t)a : -1;
}

// every core entry u->w as (slot of u, slot of w) in the block of edge u-w (one warp per vertex)
__global__ void bg_keys_kernel(const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                               const int32_t* __restrict__ parent, const int32_t* __restrict__ pre,
                               const int32_t* __restrict__ blab, const int32_t* __restrict__ blk_of_lab,
                               const int32_t* __restrict__ slot_core, const int64_t* __restrict__ bvoff,
                               const int32_t* __restrict__ vslot, const uint8_t* __restrict__ ap, int32_t nc,
                               uint64_t* __restrict__ keys, int32_t* bdeg, int* err) {
    const int t = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nc; u += nw) {
        const int32_t pu = parent[u];
        for (int64_t j = crow[u] + t; j < crow[u + 1]; j += 32) {
            const int32_t w = ccol[j];
            int32_t l;
            if (parent[w] == u) l = blab[w];
            else if (pu == w) l = blab[u];
            else l = pre[u] > pre[w] ? blab[u] : blab[w];
            const int32_t b = blk_of_lab[l];
            const int32_t su = b >= 0 ? slot_in(slot_core, bvoff, vslot, ap, b, (int32_t)u) : -1;
            const int32_t sw = b >= 0 ? slot_in(slot_core, bvoff, vslot, ap, b, w) : -1;
            if (su < 0 || sw < 0) {   // an edge whose block misses an endpoint: not a symmetric CSR
                atomicExch(err, 4);
                keys[j] = 0;
                continue;
            }
            keys[j] = ((uint64_t)(uint32_t)su << 32) | (uint32_t)sw;
            atomicAdd(&bdeg[su], 1);
        }
    }
}

__global__ void key_lo_kernel(const uint64_t* __restrict__ keys, int64_t m, int32_t* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)(uint32_t)keys[i];
}

__global__ void i32_to_i64_kernel(const int32_t* __restrict__ a, int32_t n, int64_t* __restrict__ b) {
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = a[i];
}

int bits_for(uint64_t x) {
    int b = 1;
    while (b < 64 && (x >> b)) b++;
    return b;
}

// CUB calls with their own temporary storage.
template <typename F>
gbc_status cub_run(F f, cudaStream_t s, const char* what) {
    size_t bytes = 0;
    if (f(nullptr, bytes) != cudaSuccess) { cudaGetLastError(); set_error("reduction: %s sizing", what); return GBC_ERR_CUDA; }
    DBuf<char> tmp;
    if (!tmp.alloc(bytes)) { set_error("reduction: %s scratch", what); return GBC_ERR_NOMEM; }
    if (f(tmp.p, bytes) != cudaSuccess) { cudaGetLastError(); set_error("reduction: %s", what); return GBC_ERR_CUDA; }
    GBC_CUDA(cudaStreamSynchronize(s));   // tmp is freed on return
    return GBC_OK;
}

gbc_status check_err(const int* d_err, cudaStream_t s) {
    int e = 0;
    GBC_CUDA(cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    if (e == 1) { set_error("internal: union-find did not settle"); return GBC_ERR_LIMIT; }
    if (e) { set_error("reduction: the CSR is not symmetric (check %d)", e); return GBC_ERR_ARG; }
    return GBC_OK;
}

gbc_status read_u32(const unsigned* d, unsigned* h, cudaStream_t s) {
    GBC_CUDA(cudaMemcpyAsync(h, d, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    return GBC_OK;
}

}  // namespace

gbc_status component_labels(const int64_t* d_row, const int32_t* d_col, int32_t n, cudaStream_t s, int32_t* d_lab) {
    if (n <= 0) return GBC_OK;
    DBuf<int32_t> uf;
    DBuf<int> err;
    RD_ALLOC(uf, n);
    RD_ALLOC(err, 1);
    GBC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    iota_kernel<<<grid_threads(n), RB, 0, s>>>(uf.p, n);
    cc_link_sample_kernel<<<grid_threads(n), RB, 0, s>>>(d_row, d_col, n, uf.p, err.p);
    uf_compress_kernel<<<grid_threads(n), RB, 0, s>>>(uf.p, n);
    cc_union_kernel<<<grid_warps(n), RB, 0, s>>>(d_row, d_col, n, uf.p, err.p);
    uf_flatten_kernel<<<grid_threads(n), RB, 0, s>>>(uf.p, n, d_lab, nullptr);
    GBC_CUDA(cudaGetLastError());
    return check_err(err.p, s);   // synchronises: uf is freed on return
}

gbc_status check_csr_device(const int64_t* d_row, const int32_t* d_col, int32_t n, int64_t M, const int32_t* host_col,
                            cudaStream_t s) {
    DBuf<unsigned> bad;
    RD_ALLOC(bad, 3);
    GBC_CUDA(cudaMemsetAsync(bad.p, 0xFF, 3 * sizeof(unsigned), s));
    csr_entries_check_kernel<<<grid_threads(std::max<int64_t>(n, M)), RB, 0, s>>>(d_row, d_col, n, M, bad.p);
    unsigned h[3];
    GBC_CUDA(cudaMemcpyAsync(h, bad.p, sizeof h, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    if (h[0] != ~0u) { set_error("row offsets decrease at %lld", (long long)h[0]); return GBC_ERR_ARG; }
    if (h[1] != ~0u) {
        int32_t val = 0;
        if (host_col) val = host_col[h[1]];
        else GBC_CUDA(cudaMemcpy(&val, d_col + h[1], sizeof val, cudaMemcpyDeviceToHost));
        set_error("col[%lld]=%d out of range", (long long)h[1], val);
        return GBC_ERR_ARG;
    }
    self_loop_check_kernel<<<grid_warps(n), RB, 0, s>>>(d_row, d_col, n, bad.p);
    GBC_CUDA(cudaMemcpyAsync(h, bad.p, sizeof h, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    if (h[2] != ~0u) { set_error("self-loop at vertex %d", (int)h[2]); return GBC_ERR_ARG; }
    return GBC_OK;
}

gbc_status fold_split_device(const int64_t* d_row, const int32_t* d_col, int32_t n, int64_t M, int32_t start,
                             cudaStream_t s, FoldSplit& out) {
    out = FoldSplit();
    // ---- folding rounds
    DBuf<int32_t> deg, fround, parent, cand, qa, qb;
    DBuf<uint8_t> alive;
    DBuf<unsigned long long> r, ff;
    DBuf<unsigned> qn;
    DBuf<int> err;
    RD_ALLOC(deg, n); RD_ALLOC(fround, n); RD_ALLOC(parent, n); RD_ALLOC(cand, n); RD_ALLOC(qa, n); RD_ALLOC(qb, n);
    RD_ALLOC(alive, n); RD_ALLOC(r, n); RD_ALLOC(ff, n); RD_ALLOC(qn, 2); RD_ALLOC(err, 1);
    GBC_CUDA(cudaMemsetAsync(qn.p, 0, 2 * sizeof(unsigned), s));
    GBC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    if (n > 0)
        fold_init_kernel<<<grid_threads(n), RB, 0, s>>>(d_row, n, start, deg.p, alive.p, fround.p, parent.p, cand.p,
                                                        r.p, ff.p, qa.p, qn.p);
    GBC_CUDA(cudaGetLastError());
    unsigned cnt = 0;
    GBC_TRY(read_u32(qn.p, &cnt, s));
    int32_t* q = qa.p;
    int32_t* nq = qb.p;
    int32_t round = 0;
    while (cnt > 0) {
        fold_mark_kernel<<<grid_threads(cnt), RB, 0, s>>>(q, cnt, deg.p, cand.p, round);
        GBC_CUDA(cudaMemsetAsync(qn.p + 1, 0, sizeof(unsigned), s));
        fold_step_kernel<<<grid_threads(cnt), RB, 0, s>>>(d_row, d_col, q, cnt, deg.p, alive.p, cand.p, round, parent.p,
                                                          fround.p, r.p, ff.p, nq, qn.p + 1);
        GBC_CUDA(cudaGetLastError());
        GBC_TRY(read_u32(qn.p + 1, &cnt, s));
        std::swap(q, nq);
        round++;
    }
    out.rounds = round;
    out.parent.resize(n);
    out.fround.resize(n);
    out.r.resize(n);
    out.ff.resize(n);
    if (n > 0) {
        GBC_CUDA(cudaMemcpyAsync(out.parent.data(), parent.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaMemcpyAsync(out.fround.data(), fround.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaMemcpyAsync(out.r.data(), r.p, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaMemcpyAsync(out.ff.data(), ff.p, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, s));
    }

    // ---- the folded graph in core ids
    DBuf<int32_t> a32, cid, core_v;
    RD_ALLOC(a32, n); RD_ALLOC(cid, n); RD_ALLOC(core_v, n);
    int32_t nc = 0;
    if (n > 0) {
        alive_i32_kernel<<<grid_threads(n), RB, 0, s>>>(alive.p, n, a32.p);
        GBC_TRY(cub_run([&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, a32.p, cid.p, n, s); }, s, "core ids"));
        int32_t last[2];
        GBC_CUDA(cudaMemcpyAsync(&last[0], cid.p + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaMemcpyAsync(&last[1], a32.p + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaStreamSynchronize(s));
        nc = last[0] + last[1];
    }
    DBuf<int64_t> cdeg, crow;
    RD_ALLOC(cdeg, (size_t)nc + 1);
    RD_ALLOC(crow, (size_t)nc + 1);
    GBC_CUDA(cudaMemsetAsync(cdeg.p, 0, sizeof(int64_t) * ((size_t)nc + 1), s));
    if (n > 0) core_ids_kernel<<<grid_threads(n), RB, 0, s>>>(alive.p, cid.p, deg.p, n, core_v.p, cdeg.p);
    GBC_TRY(cub_run([&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, cdeg.p, crow.p, nc + 1, s); }, s, "core rows"));
    int64_t Mc = 0;
    GBC_CUDA(cudaMemcpyAsync(&Mc, crow.p + nc, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    DBuf<int32_t> ccol;
    RD_ALLOC(ccol, (size_t)Mc);
    if (nc > 0) core_fill_kernel<<<grid_warps(nc), RB, 0, s>>>(d_row, d_col, alive.p, cid.p, core_v.p, crow.p, nc, ccol.p, err.p);
    GBC_CUDA(cudaGetLastError());
    GBC_TRY(check_err(err.p, s));
    if (nc > (INT32_MAX >> 1)) { set_error("reduction: %d vertices left after folding, above 2^30", nc); return GBC_ERR_ARG; }
    out.core_v.resize(nc);
    out.core.n = nc;
    out.core_m = Mc;
    if (nc > 0) GBC_CUDA(cudaMemcpyAsync(out.core_v.data(), core_v.p, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    // the folding buffers are no longer needed
    deg.alloc(0); fround.alloc(0); parent.alloc(0); cand.alloc(0); alive.alloc(0); r.alloc(0); ff.alloc(0);
    a32.alloc(0); cid.alloc(0); core_v.alloc(0); cdeg.alloc(0);
    out.bvoff.assign(1, 0);
    if (nc == 0) {
        out.d_core_row = crow.p;
        out.d_core_col = ccol.p;
        crow.p = nullptr;
        ccol.p = nullptr;
        return GBC_OK;
    }

    // ---- components and the BFS forest
    DBuf<int32_t> uf, lab, isroot, cpos, comp, level, par, nd, pre, lo, hi, order;
    RD_ALLOC(uf, nc); RD_ALLOC(lab, nc); RD_ALLOC(isroot, nc); RD_ALLOC(cpos, nc); RD_ALLOC(comp, nc);
    RD_ALLOC(level, nc); RD_ALLOC(par, nc); RD_ALLOC(nd, nc); RD_ALLOC(pre, nc); RD_ALLOC(lo, nc); RD_ALLOC(hi, nc);
    RD_ALLOC(order, nc);
    iota_kernel<<<grid_threads(nc), RB, 0, s>>>(uf.p, nc);
    cc_link_sample_kernel<<<grid_threads(nc), RB, 0, s>>>(crow.p, ccol.p, nc, uf.p, err.p);
    uf_compress_kernel<<<grid_threads(nc), RB, 0, s>>>(uf.p, nc);
    cc_union_kernel<<<grid_warps(nc), RB, 0, s>>>(crow.p, ccol.p, nc, uf.p, err.p);
    uf_flatten_kernel<<<grid_threads(nc), RB, 0, s>>>(uf.p, nc, lab.p, isroot.p);
    GBC_TRY(cub_run([&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, isroot.p, cpos.p, nc, s); }, s, "component ids"));
    {
        int32_t last[2];
        GBC_CUDA(cudaMemcpyAsync(&last[0], cpos.p + nc - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaMemcpyAsync(&last[1], isroot.p + nc - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaStreamSynchronize(s));
        out.n_comp = last[0] + last[1];
    }
    forest_init_kernel<<<grid_threads(nc), RB, 0, s>>>(lab.p, cpos.p, nc, comp.p, level.p, par.p, nd.p, pre.p, order.p);
    GBC_CUDA(cudaGetLastError());
    std::vector<int64_t> loff{0, out.n_comp};
    for (int32_t L = 0;; L++) {
        const unsigned c = (unsigned)(loff[L + 1] - loff[L]);
        GBC_CUDA(cudaMemsetAsync(qn.p, 0, sizeof(unsigned), s));
        bfs_level_kernel<<<grid_warps(c), RB, 0, s>>>(crow.p, ccol.p, order.p + loff[L], c, L, level.p,
                                                      order.p + loff[L + 1], qn.p);
        GBC_CUDA(cudaGetLastError());
        unsigned got = 0;
        GBC_TRY(read_u32(qn.p, &got, s));
        if (got == 0) break;
        loff.push_back(loff.back() + got);
        if (loff.back() > nc) { set_error("internal: BFS forest visited %lld of %d vertices", (long long)loff.back(), nc); return GBC_ERR_LIMIT; }
    }
    const int32_t nlev = (int32_t)loff.size() - 1;
    if (loff.back() != nc) { set_error("internal: BFS forest reached %lld of %d vertices", (long long)loff.back(), nc); return GBC_ERR_LIMIT; }
    out.levels = nlev;
    parent_kernel<<<grid_warps(nc), RB, 0, s>>>(crow.p, ccol.p, level.p, nc, par.p, err.p);
    for (int32_t L = nlev - 1; L >= 1; L--) {
        const unsigned c = (unsigned)(loff[L + 1] - loff[L]);
        nd_up_kernel<<<grid_threads(c), RB, 0, s>>>(order.p + loff[L], c, par.p, nd.p);
    }
    for (int32_t L = 0; L + 1 < nlev; L++) {
        const unsigned c = (unsigned)(loff[L + 1] - loff[L]);
        pre_down_kernel<<<grid_warps(c), RB, 0, s>>>(crow.p, ccol.p, order.p + loff[L], c, par.p, nd.p, pre.p);
    }
    lohi_local_kernel<<<grid_warps(nc), RB, 0, s>>>(crow.p, ccol.p, par.p, pre.p, nc, lo.p, hi.p);
    for (int32_t L = nlev - 1; L >= 1; L--) {
        const unsigned c = (unsigned)(loff[L + 1] - loff[L]);
        lohi_up_kernel<<<grid_threads(c), RB, 0, s>>>(order.p + loff[L], c, par.p, lo.p, hi.p);
    }
    GBC_CUDA(cudaGetLastError());

    // ---- blocks
    DBuf<int32_t> blab, nkeys, kpos;
    DBuf<uint8_t> ap;
    RD_ALLOC(blab, nc); RD_ALLOC(nkeys, nc); RD_ALLOC(kpos, nc); RD_ALLOC(ap, nc);
    iota_kernel<<<grid_threads(nc), RB, 0, s>>>(uf.p, nc);
    tv_union_tree_kernel<<<grid_threads(nc), RB, 0, s>>>(par.p, pre.p, nd.p, lo.p, hi.p, nc, uf.p, err.p);
    uf_compress_kernel<<<grid_threads(nc), RB, 0, s>>>(uf.p, nc);
    tv_union_cross_kernel<<<grid_warps(nc), RB, 0, s>>>(crow.p, ccol.p, par.p, pre.p, nd.p, nc, uf.p, err.p);
    uf_flatten_kernel<<<grid_threads(nc), RB, 0, s>>>(uf.p, nc, blab.p, nullptr);
    ap_kernel<<<grid_warps(nc), RB, 0, s>>>(crow.p, ccol.p, par.p, blab.p, nc, ap.p, nkeys.p);
    GBC_TRY(cub_run([&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, nkeys.p, kpos.p, nc, s); }, s, "slot key offsets"));
    int32_t nkeys_total = 0;
    {
        int32_t last[2];
        GBC_CUDA(cudaMemcpyAsync(&last[0], kpos.p + nc - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaMemcpyAsync(&last[1], nkeys.p + nc - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        int herr = 0;
        GBC_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaStreamSynchronize(s));
        if (herr == 1) { set_error("internal: union-find did not settle"); return GBC_ERR_LIMIT; }
        if (herr) { set_error("reduction: the CSR is not symmetric (check %d)", herr); return GBC_ERR_ARG; }
        nkeys_total = last[0] + last[1];
    }
    DBuf<uint64_t> k0, k1;
    DBuf<int32_t> nsel;
    RD_ALLOC(k0, nkeys_total); RD_ALLOC(k1, nkeys_total); RD_ALLOC(nsel, 1);
    slot_keys_kernel<<<grid_threads(nc), RB, 0, s>>>(par.p, blab.p, kpos.p, nkeys.p, nc, k0.p);
    const int kbits = 32 + bits_for((uint64_t)nc);
    cub::DoubleBuffer<uint64_t> db(k0.p, k1.p);
    GBC_TRY(cub_run([&](void* t, size_t& b) { return cub::DeviceRadixSort::SortKeys(t, b, db, nkeys_total, 0, kbits, s); }, s, "slot sort"));
    uint64_t* sorted = db.Current();
    uint64_t* uniq = sorted == k0.p ? k1.p : k0.p;
    GBC_TRY(cub_run([&](void* t, size_t& b) { return cub::DeviceSelect::Unique(t, b, sorted, uniq, nsel.p, nkeys_total, s); }, s, "slot unique"));
    int32_t ns = 0;
    GBC_CUDA(cudaMemcpyAsync(&ns, nsel.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    if (ns >= (1 << 27)) { set_error("block graph too large (%d slots)", ns); return GBC_ERR_ARG; }
    DBuf<int32_t> flag, bid, slot_core, blk_of_lab, vslot;
    DBuf<int64_t> bvoff;
    RD_ALLOC(flag, ns); RD_ALLOC(bid, ns); RD_ALLOC(slot_core, ns); RD_ALLOC(blk_of_lab, nc); RD_ALLOC(vslot, nc);
    block_flags_kernel<<<grid_threads(ns), RB, 0, s>>>(uniq, ns, flag.p);
    GBC_TRY(cub_run([&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, flag.p, bid.p, ns, s); }, s, "block ids"));
    int32_t nb = 0;
    {
        int32_t last[2];
        GBC_CUDA(cudaMemcpyAsync(&last[0], bid.p + ns - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaMemcpyAsync(&last[1], flag.p + ns - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaStreamSynchronize(s));
        nb = last[0] + last[1];
    }
    RD_ALLOC(bvoff, (size_t)nb + 1);
    fill_i32_kernel<<<grid_threads(nc), RB, 0, s>>>(vslot.p, nc, INT32_MAX);
    fill_i32_kernel<<<grid_threads(nc), RB, 0, s>>>(blk_of_lab.p, nc, -1);
    slots_kernel<<<grid_threads(ns), RB, 0, s>>>(uniq, flag.p, bid.p, ns, slot_core.p, bvoff.p, blk_of_lab.p, vslot.p);
    {
        const int64_t e = ns;
        GBC_CUDA(cudaMemcpyAsync(bvoff.p + nb, &e, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    }
    // block graph: sorted (slot, slot) keys of every core entry
    DBuf<uint64_t> e0, e1;
    DBuf<int32_t> bdeg, bcol;
    DBuf<int64_t> bdeg64, brow;
    RD_ALLOC(e0, (size_t)Mc); RD_ALLOC(e1, (size_t)Mc); RD_ALLOC(bdeg, ns); RD_ALLOC(bcol, (size_t)Mc);
    RD_ALLOC(bdeg64, (size_t)ns + 1); RD_ALLOC(brow, (size_t)ns + 1);
    GBC_CUDA(cudaMemsetAsync(bdeg.p, 0, sizeof(int32_t) * ns, s));
    GBC_CUDA(cudaMemsetAsync(bdeg64.p, 0, sizeof(int64_t) * ((size_t)ns + 1), s));
    bg_keys_kernel<<<grid_warps(nc), RB, 0, s>>>(crow.p, ccol.p, par.p, pre.p, blab.p, blk_of_lab.p, slot_core.p, bvoff.p,
                                                 vslot.p, ap.p, nc, e0.p, bdeg.p, err.p);
    GBC_CUDA(cudaGetLastError());
    const int ebits = 32 + bits_for((uint64_t)ns);
    cub::DoubleBuffer<uint64_t> eb(e0.p, e1.p);
    GBC_TRY(cub_run([&](void* t, size_t& b) { return cub::DeviceRadixSort::SortKeys(t, b, eb, Mc, 0, ebits, s); }, s, "block graph sort"));
    key_lo_kernel<<<grid_threads(Mc), RB, 0, s>>>(eb.Current(), Mc, bcol.p);
    i32_to_i64_kernel<<<grid_threads(ns), RB, 0, s>>>(bdeg.p, ns, bdeg64.p);
    GBC_TRY(cub_run([&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, bdeg64.p, brow.p, ns + 1, s); }, s, "block graph rows"));

    GBC_TRY(check_err(err.p, s));
    // ---- back to the host
    out.core_comp.resize(nc);
    out.core_ap.resize(nc);
    out.core_vslot.resize(nc);
    out.bvoff.resize((size_t)nb + 1);
    out.slot_core.resize(ns);
    out.bg.n = ns;
    out.bg_m = Mc;
    GBC_CUDA(cudaMemcpyAsync(out.core_comp.data(), comp.p, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaMemcpyAsync(out.core_ap.data(), ap.p, nc, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaMemcpyAsync(out.core_vslot.data(), vslot.p, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaMemcpyAsync(out.bvoff.data(), bvoff.p, sizeof(int64_t) * ((size_t)nb + 1), cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaMemcpyAsync(out.slot_core.data(), slot_core.p, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    // the two graphs stay on the device, owned by the caller from here
    out.d_core_row = crow.p;
    out.d_core_col = ccol.p;
    out.d_bg_row = brow.p;
    out.d_bg_col = bcol.p;
    crow.p = nullptr;
    ccol.p = nullptr;
    brow.p = nullptr;
    bcol.p = nullptr;
    return GBC_OK;
}

}  // namespace gbc
