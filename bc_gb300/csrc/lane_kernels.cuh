// Level kernels of the batched multi-source lane engine for sm_103a (the
// engine's host side is lanes.cu).
//
// B sources ("lanes") of one batch run level-synchronous BFS together.  Lane
// state is lane-interleaved: for lane group g (32 lanes, one per warp thread)
// and vertex v the 32 entries lvl/sigma/rho[g][v][0..31] are contiguous, so a
// warp that visits a neighbour x touches one 32- or 64-byte (lvl, 8/16-bit)
// and one 128/256-byte (sigma, rho) segment for all 32 lanes of its group.
// The frontier of level d is a list of (vertex, group) entries; the lists of
// all levels are kept (fq + foff) and replayed in reverse by the dependency
// sweep.
//
// Forward, one kernel per level (expand): for every entry (v,g) of F_d and
// every lane with lvl == d, pull sigma(v) from the level-(d-1) neighbours
// (no atomics, deterministic) and discover level d+1 among the neighbours
// (plain store of d+1, enqueue once per (x,g) via vmark).  A task with little
// work (active lanes x degree) is expanded by one thread, 32 tasks per warp; a
// task whose active lanes are few expands edge-parallel (threads over
// neighbours, lanes in turn); the rest lane-parallel (threads over lanes,
// neighbours in turn).  Hubs (degree > 1024) take a whole CTA.
// Backward, one kernel per level (pull): delta(v) = sigma(v) * sum over
// successors w of rho(w), rho(v) = (1 + delta(v)) / sigma(v); per-group FP64
// partials of BC accumulate without atomics.  Levels are read from a device
// control block and advanced by the last CTA of each launch, so a fixed run
// of level launches is captured once as a CUDA graph and replayed.
//
// The kernels are templates over the CTA size NT (128, 256 or 512 threads);
// lanes_nt128.cu, lanes_nt256.cu and lanes_nt512.cu each instantiate one
// shape (compiled in parallel) and hand lanes.cu a table of entry points, so
// the autotuner can pick the shape per graph.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "engine.h"

namespace gbc {

struct Ctl {
    int level;
    int maxlevel;
    int done;
    int err;            // bit0: a frontier queue overflowed, bit1: level cap of the level type
    unsigned blocks;    // finished-CTA counter of the running launch
    int any_ovf;        // some lane's exact path count overflowed uint64
    unsigned long long tail;    // append position, regular queue
    unsigned long long htail;   // append position, hub queue
    unsigned long long next;    // fetch position of the running level, regular queue
    unsigned long long hnext;   // fetch position of the running level, hub queue
    // direction switching (closeness, 128-lane groups)
    int bu;                     // the running level discovers bottom-up
    int td_only;                // this batch stays top-down
    int bu_levels;              // bottom-up levels of this batch
    unsigned long long fdeg;    // degree sum of the entries appended for the next level
    unsigned long long fprev;   // the same for the running level
    unsigned long long mu;      // bottom-up level: degree sum of (vertex, group) pairs still unreached in some lane
    unsigned long long bnext;   // bottom-up level: fetch position over the done-bitmap words
    unsigned long long visits;  // neighbour visits of top-down forward tasks (degree summed over entries)
};

struct KArgs {
    const int64_t* __restrict__ row;
    const int32_t* __restrict__ col;
    int n;
    int ng;
    const int32_t* w;      // nullable vertex weights
    const int64_t* ff;     // nullable folded distance sums
    void* lvl;
    uint64_t* sig;
    void* rho;
    int32_t* vmark;
    uint32_t* fq;          // regular frontier entries, all levels
    unsigned long long fcap;
    unsigned long long* foff;
    uint32_t* hq;          // hub frontier entries (vertex degree > hub_deg), all levels
    unsigned long long hcap;
    unsigned long long* hoff;
    Ctl* ctl;
    uint32_t* ovf;
    unsigned long long* cc;
    double* bcg;
    int32_t* srcw;         // per-lane source weight (vertex weight of the lane's source, 1 without weights)
    int sparse;            // entries with <= sparse active lanes expand edge-parallel
    int light;             // entries with (active lanes x degree) <= light expand one per thread
    int semantics;
    int gs;                // lanes per group = 1 << gs (5: 32 lanes, one per thread; 7: 128, four per thread)
    int hub_deg;           // entries of vertices with a higher degree go to the hub queue (CTA per entry)
    // direction switching (closeness, 128-lane groups); dir = 0 disables it
    int dir;
    const int32_t* vcomp;  // component label of every vertex
    int32_t* lcomp;        // component label of every lane's source (-1: empty lane)
    uint32_t* done;        // [ng][ceil(n/32)] bits: (vertex, group) has no reachable unreached lane
    unsigned long long mtot;   // directed entries x lane groups
    // vertices numbered by descending degree: the hubs are exactly the ids below hub_lim
    // (-1: not known to be so numbered; the degree is read instead)
    int hub_lim;
    // closeness direction switching: bottom-up once past the frontier peak while
    // frontier edges x bu_share exceed mtot (0: never)
    unsigned long long bu_share;
    // bytes per exact path count (128-lane groups: 2 or 4 while every count fits, else 8)
    int sig_bytes;
    // one lane per task on graphs of degree <= 8: every vertex's neighbours in ell_q int4 slots
    // (ell[v * ell_q + q], -1 past the degree), read in place of row offsets and columns; 0: none
    const int4* ell;
    int ell_q;
};

// Entry points of the level kernels of one CTA shape.
struct LevelKernels {
    void (*expand[2][3])(KArgs);       // 32-lane groups: [16-bit levels][MODE]
    void (*backward[2][4])(KArgs);     // [16-bit levels][wide sigma * 2 + FP64 delta]
    void (*expand_q[2][3][3])(KArgs);    // 128-lane groups: [16-bit levels][MODE][path-count width 8/4/2 bytes]
    void (*backward_q[2][4][3])(KArgs);  // [16-bit levels][wide sigma * 2 + FP64 delta][width]
    void (*expand_s[3])(KArgs);          // one lane per task: [MODE]
    void (*backward_s[4])(KArgs);        // [wide sigma * 2 + FP64 delta]
};
void level_kernels_128(LevelKernels& k);   // lanes_nt128.cu
void level_kernels_256(LevelKernels& k);   // lanes_nt256.cu
void level_kernels_512(LevelKernels& k);   // lanes_nt512.cu

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;


// Level storage: uint8_t while every BFS stays under 254 levels, uint16_t
// after a batch went deeper.  All-ones is "unreached".
template <typename LT>
struct Lv {
    static constexpr int INF = (int)(LT)~(LT)0;
    static constexpr int MAXD = INF - 2;   // deepest level that can still be expanded
};





constexpr int HUB_DEG = 1024;   // 32-lane groups: entries of higher-degree vertices are expanded by a whole CTA
constexpr int HUB_DEG_Q = 1024; // the same for 128-lane groups
constexpr int FETCH = 32;       // regular entries a warp takes per fetch, one per thread
constexpr int LIGHT_U = 4;      // one-thread tasks: neighbours whose loads are issued together
constexpr int STG = 128;        // regular-queue entries a warp stages in shared memory per append
// Minimum resident CTAs per SM of the forward kernels.  Deep graphs (16-bit
// levels) have small, latency-bound levels and need 4 (64 registers); so do
// the wide-sigma variants, which would otherwise take over 100 registers.
// For exact sigma on 8-bit levels 0 leaves the choice to the compiler, which
// also lands on 64 registers and measured 4-6% faster on R-MAT scale 22 than
// forcing 4 or 5 (48 registers); unbounded (113+ registers, 2 CTAs) is 35%
// slower.  The dependency sweep is always compiled for 4 (its compensated
// sums would otherwise take 80 registers, 5% slower on R-MAT scale 22).
// Other CTA shapes are held to the same 64 registers (1024 / NT CTAs per SM).
template <typename LT, bool WIDE, int NT> constexpr int MINB = (sizeof(LT) == 2 || WIDE || NT != 256) ? 1024 / NT : 0;

__device__ __forceinline__ size_t sidx(int g, int n, int v, int t, int gs) {
    return ((((size_t)g * (size_t)n) + (size_t)v) << gs) + (size_t)t;
}

__device__ __forceinline__ bool is_hub(const KArgs& A, int x) {
    return A.hub_lim >= 0 ? x < A.hub_lim : (A.row[x + 1] - A.row[x]) > A.hub_deg;
}

// ---- wide-exponent path counts ---------------------------------------------
// Path counts past uint64 are held as (1 + f/2^44) * 2^(e - WBIAS) in one
// 64-bit word e << 44 | f (the word 0 is zero): 44 fraction bits (relative
// step 5.7e-14) and a 20-bit exponent, so |log2| < 2^19.  A sum aligns the
// exponents with integer arithmetic and adds once in FP64; the dependency
// sweep multiplies mantissas and adds exponents.  No exp2/log2 is evaluated,
// which matters on a part whose FP64 rate is a small fraction of FP32.
constexpr int WFRAC = 44;
constexpr int WBIAS = 1 << 19;
constexpr int WEMAX = (1 << (64 - WFRAC)) - 1;
constexpr unsigned long long WFMASK = (1ULL << WFRAC) - 1ULL;
constexpr unsigned long long WONE = (unsigned long long)WBIAS << WFRAC;
constexpr int WEMPTY = -0x7FFFFFFF;   // exponent of an empty accumulator

// x * 2^k for positive normal x; 0 below the normal range.
__device__ __forceinline__ double pow2s(double x, int k) {
    const long long b = __double_as_longlong(x);
    const int be = (int)((b >> 52) & 0x7FF) + k;
    if (be < 1) return 0.0;
    if (be > 2046) return INFINITY;
    return __longlong_as_double(b + (long long)k * (1LL << 52));
}
__device__ __forceinline__ float pow2s(float x, int k) {
    const int b = __float_as_int(x);
    const int be = ((b >> 23) & 0xFF) + k;
    if (be < 1) return 0.0f;
    if (be > 254) return INFINITY;
    return __int_as_float(b + k * (1 << 23));
}

__device__ __forceinline__ int wexp(uint64_t u) { return (int)(u >> WFRAC) - WBIAS; }
template <typename T> __device__ __forceinline__ T wmant(uint64_t u);
template <> __device__ __forceinline__ double wmant<double>(uint64_t u) {
    return __longlong_as_double((long long)((1023ULL << 52) | ((u & WFMASK) << (52 - WFRAC))));
}
template <> __device__ __forceinline__ float wmant<float>(uint64_t u) {   // rounded to 24 bits
    return __uint_as_float(0x3F800000u + (unsigned)(((u & WFMASK) + (1ULL << (WFRAC - 24))) >> (WFRAC - 23)));
}

// Word of s * 2^E for positive normal s, rounded to 44 fraction bits.  Below
// the range gives 0; above it sets of.
__device__ __forceinline__ uint64_t wpack(double s, int E, bool& of) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(s);
    int e = E + (int)((b >> 52) & 0x7FF) - 1023;
    unsigned long long f = ((b & ((1ULL << 52) - 1ULL)) + (1ULL << (51 - WFRAC))) >> (52 - WFRAC);
    if (f >> WFRAC) { f = 0; e++; }
    const int eb = e + WBIAS;
    if (eb < 1) return 0ULL;
    if (eb > WEMAX) { of = true; return ~0ULL; }
    return ((unsigned long long)eb << WFRAC) | f;
}
__device__ __forceinline__ uint64_t wpack(float s, int E, bool& of) {
    const unsigned b = __float_as_uint(s);
    const int eb = E + (int)((b >> 23) & 0xFF) - 127 + WBIAS;
    if (eb < 1) return 0ULL;
    if (eb > WEMAX) { of = true; return ~0ULL; }
    return ((unsigned long long)eb << WFRAC) | ((unsigned long long)(b & 0x7FFFFFu) << (WFRAC - 23));
}

// Accumulators s * 2^E (E == WEMPTY: empty).
__device__ __forceinline__ void wadd(double& s, int& E, uint64_t u) {
    const int e = wexp(u);
    const double m = wmant<double>(u);
    if (E == WEMPTY) { s = m; E = e; }
    else if (e > E) { s = pow2s(s, E - e) + m; E = e; }
    else s += pow2s(m, e - E);
}
__device__ __forceinline__ void wmerge(double& s, int& E, double s2, int E2) {
    if (E2 == WEMPTY) return;
    if (E == WEMPTY) { s = s2; E = E2; }
    else if (E2 > E) { s = pow2s(s, E - E2) + s2; E = E2; }
    else s += pow2s(s2, E2 - E);
}

// sigma(v) * rho(w) as a plain T, sigma(v) given as mantissa mv and exponent ev.
template <typename T>
__device__ __forceinline__ T wterm(T mv, int ev, uint64_t r) {
    return pow2s(mv * wmant<T>(r), ev + wexp(r));
}

// Running sum of the dependency sweep: compensated (Kahan) in FP32, so a
// hub's sum over thousands of successor terms keeps FP32-ulp accuracy instead
// of losing ~sqrt(terms) ulps; plain in FP64.  The terms are non-negative, and
// Kahan's recurrence bounds the error by (2u + O(n u^2)) times the sum of the
// terms' magnitudes in any order, so it needs no magnitude test (Neumaier's
// variant, which also handles cancelling terms, costs twice the instructions
// per term).  c holds the part of the sum not yet in s: the value is s + c.
template <typename T>
struct Sum {
    T s = T(0), c = T(0);
    __device__ __forceinline__ void add(T x) {
        if (sizeof(T) == 4) {
            const T y = x + c;
            const T t = s + y;
            c = y - (t - s);
            s = t;
        } else {
            s += x;
        }
    }
    // add another partial (its sum, then its carried compensation)
    __device__ __forceinline__ void merge(T s2, T c2) {
        add(s2);
        c += c2;
    }
    __device__ __forceinline__ T value() const { return s + c; }
};

// ---- frontier appends ------------------------------------------------------
// A warp stages the regular entries it discovers in shared memory and appends
// them to the queue with one atomic per STG entries (or at the end of the
// launch), so the queue tail sees few atomics even when every entry of a level
// discovers one or two vertices.
struct Stage {
    uint32_t* buf;
    int cnt;                   // uniform across the warp
    unsigned long long fdeg;   // this thread's degree sum of appended entries (direction switching)
};

__device__ __forceinline__ void stage_flush(const KArgs& A, Stage& S) {
    const int t = threadIdx.x & 31;
    __syncwarp();
    if (S.cnt == 0) return;
    unsigned long long base = 0;
    if (t == 0) base = atomicAdd(&A.ctl->tail, (unsigned long long)S.cnt);
    base = __shfl_sync(FULL, base, 0);
    for (int k = t; k < S.cnt; k += 32) {
        const unsigned long long pos = base + (unsigned long long)k;
        if (pos < A.fcap) A.fq[pos] = S.buf[k];
    }
    __syncwarp();
    S.cnt = 0;
}

// Start of the next FETCH regular entries of level d for this warp (e: the
// level's end).  The first round is assigned statically -- warp w of the grid
// takes the entries at foff[d] + w*FETCH -- so a level with fewer entries than
// the grid has threads costs no atomic on the level counter, and a large one
// one atomic fewer per warp; later rounds take FETCH at a time from the
// counter (which starts at foff[d]) past that static region.
__device__ __forceinline__ unsigned long long warp_fetch(const KArgs& A, int d, bool& first) {
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    if (first) {
        first = false;
        return A.foff[d] + ((unsigned long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * FETCH;
    }
    unsigned long long base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(&A.ctl->next, (unsigned long long)FETCH) + warps * FETCH;
    return __shfl_sync(FULL, base, 0);
}

// Neighbour visits counted by the threads of a warp, added to the control block.
__device__ __forceinline__ void add_visits(const KArgs& A, unsigned long long vis) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vis += __shfl_xor_sync(FULL, vis, o);
    if ((threadIdx.x & 31) == 0 && vis) atomicAdd(&A.ctl->visits, vis);
}

// Entries of threads with has == true: hub entries straight to the hub queue,
// the rest to the warp's stage.
__device__ __forceinline__ void warp_append(const KArgs& A, Stage& S, bool has, bool hub, uint32_t ent) {
    const int t = threadIdx.x & 31;
    const unsigned lt = (1u << t) - 1u;
    const unsigned hm = __ballot_sync(FULL, has && hub);
    if (hm) {
        const int leader = __ffs(hm) - 1;
        unsigned long long base = 0;
        if (t == leader) base = atomicAdd(&A.ctl->htail, (unsigned long long)__popc(hm));
        base = __shfl_sync(FULL, base, leader);
        if (has && hub) {
            const unsigned long long pos = base + __popc(hm & lt);
            if (pos < A.hcap) A.hq[pos] = ent;
        }
    }
    const unsigned m = __ballot_sync(FULL, has && !hub);
    if (!m) return;
    if (S.cnt + __popc(m) > STG) stage_flush(A, S);
    if (has && !hub) S.buf[S.cnt + __popc(m & lt)] = ent;
    S.cnt += __popc(m);
}

// First claim of (x, g) for level lev.  Only a thread that saw one of x's
// active lanes unreached (and wrote d+1 there) claims: a lane already at d+1
// was written by a thread that claims, so the claim happens once per
// discovered (x, g) without a vmark access for the (many) later visits of the
// level.  Repeats are then rare (two warps that saw the same lane unreached),
// so the exchange goes straight to the atomic: one round trip, where a plain
// read to filter repeats first made it two.
__device__ __forceinline__ bool claim(const KArgs& A, size_t gbase, int x, int lev) {
    return atomicExch(&A.vmark[gbase + x], lev) != lev;
}

// Direction of the next closeness level (128-lane groups).  Top-down until
// the frontier has passed its peak (the next frontier's edges no more than
// the running one's) while still holding over 1/bu_share of all edges (x lane
// groups; 16 unless autotuned): before the peak the lanes of a group sit at several distances from
// most vertices, so a bottom-up scan of a row rarely stops early.  After a
// bottom-up level, which measured the edges still unreached (mu), stay
// bottom-up while the frontier's edges exceed half of those.
constexpr unsigned long long BU_ALPHA = 2;

// Last CTA of a forward launch publishes the next level's frontier bounds.
__device__ __forceinline__ void fwd_last_block(const KArgs& A, int d, int done, int maxd, bool dir = false) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&A.ctl->blocks, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            A.ctl->blocks = 0;
            if (!done) {
                const unsigned long long tail = atomicAdd(&A.ctl->tail, 0ULL);
                const unsigned long long htail = atomicAdd(&A.ctl->htail, 0ULL);
                if (tail > A.fcap || htail > A.hcap) {
                    A.ctl->err |= 1;
                    A.ctl->done = 1;
                    A.ctl->maxlevel = d;
                } else {
                    A.foff[d + 2] = tail;
                    A.hoff[d + 2] = htail;
                    A.ctl->next = A.foff[d + 1];
                    A.ctl->hnext = A.hoff[d + 1];
                    if (tail == A.foff[d + 1] && htail == A.hoff[d + 1]) { A.ctl->done = 1; A.ctl->maxlevel = d; }
                    else if (A.sig_bytes < 8 && *(volatile int*)&A.ctl->any_ovf) { A.ctl->done = 1; A.ctl->maxlevel = d; }
                    else if (d + 1 >= maxd) { A.ctl->err |= 2; A.ctl->done = 1; A.ctl->maxlevel = d; }
                    else A.ctl->level = d + 1;
                    if (dir && !A.ctl->td_only) {
                        const unsigned long long mf = atomicAdd(&A.ctl->fdeg, 0ULL);
                        const unsigned long long mu = atomicAdd(&A.ctl->mu, 0ULL);
                        A.ctl->bu = A.ctl->bu ? (mf * BU_ALPHA > mu)
                                              : (mf <= A.ctl->fprev && mf * A.bu_share > A.mtot);
                        A.ctl->fprev = mf;
                        A.ctl->bu_levels += A.ctl->bu;
                        A.ctl->fdeg = 0;
                        A.ctl->mu = 0;
                        A.ctl->bnext = 0;
                    }
                }
            }
        }
    }
}

// Levels of 32 lanes are one 32-byte (uint8) or 64-byte (uint16) row per
// vertex.  In lane-parallel expansion a thread owns one 32-bit word of a
// neighbour's row (LPW lanes) and compares all of them at once; a warp covers
// SLOTS neighbours per load instruction.
template <typename LT> struct Simd;
template <> struct Simd<uint8_t> {
    static constexpr int LPW = 4;
    __device__ static __forceinline__ bool any_inf(unsigned w) { return __vcmpeq4(w, 0xFFFFFFFFu) != 0u; }
    __device__ static __forceinline__ unsigned bc(int d) { return ((unsigned)d & 0xFFu) * 0x01010101u; }
    __device__ static __forceinline__ unsigned eq(unsigned a, unsigned b) { return __vcmpeq4(a, b); }
    __device__ static __forceinline__ unsigned gt(unsigned a, unsigned b) { return __vcmpgtu4(a, b); }
    __device__ static __forceinline__ bool has(unsigned m, int j) { return (m >> (8 * j)) & 1u; }
};
template <> struct Simd<uint16_t> {
    __device__ static __forceinline__ bool any_inf(unsigned w) { return __vcmpeq2(w, 0xFFFFFFFFu) != 0u; }
    static constexpr int LPW = 2;
    __device__ static __forceinline__ unsigned bc(int d) { return ((unsigned)d & 0xFFFFu) * 0x00010001u; }
    __device__ static __forceinline__ unsigned eq(unsigned a, unsigned b) { return __vcmpeq2(a, b); }
    __device__ static __forceinline__ unsigned gt(unsigned a, unsigned b) { return __vcmpgtu2(a, b); }
    __device__ static __forceinline__ bool has(unsigned m, int j) { return (m >> (16 * j)) & 1u; }
};

// Lanes of one level row whose level equals d, as a 32-bit mask (bit t = lane
// t), read with 16-byte loads by a single thread.  The byte (half-word) compare
// leaves the top bit of each matching lane set; one multiply gathers those
// bits, whose shifted copies land on distinct positions, into the top nibble.
__device__ __forceinline__ unsigned row_mask(const uint8_t* r, int d) {
    const uint4* p = reinterpret_cast<const uint4*>(r);
    const uint4 a = p[0], b = p[1];
    const unsigned w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    const unsigned d4 = Simd<uint8_t>::bc(d);
    unsigned m = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) m |= (((__vcmpeq4(w[k], d4) & 0x80808080u) * 0x00204081u) >> 28) << (4 * k);
    return m;
}
__device__ __forceinline__ unsigned row_mask(const uint16_t* r, int d) {
    const uint4* p = reinterpret_cast<const uint4*>(r);
    const unsigned d2 = Simd<uint16_t>::bc(d);
    unsigned m = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const uint4 a = p[q];
        const unsigned w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
        for (int k = 0; k < 4; k++) m |= (((__vcmpeq2(w[k], d2) & 0x80008000u) * 0x8001u) >> 30) << (8 * q + 2 * k);
    }
    return m;
}

// One regular entry per thread of a fetch: its active-lane mask and CSR row.
template <typename LT>
__device__ __forceinline__ void fetch_entry(const KArgs& A, int d, unsigned long long i, unsigned long long e,
                                            uint32_t& ent, unsigned& am, long long& r0, long long& r1) {
    ent = 0;
    am = 0;
    r0 = r1 = 0;
    if (i >= e) return;
    ent = A.fq[i];
    const int v = (int)(ent >> 5), g = (int)(ent & 31u);
    am = row_mask(reinterpret_cast<const LT*>(A.lvl) + ((((size_t)g * (size_t)A.n) + (size_t)v) << 5), d);
    r0 = A.row[v];
    r1 = A.row[v + 1];
}

// Lane-parallel forward scan of v's neighbour chunks (r0 + 32*sub, step
// 32*nsub).  Result for lane t is returned in thread t.  Path counts of the
// LPW lanes a thread owns are read as 16-byte pairs; per-slot partial sums
// meet in shared memory and are added in slot order.
template <int MODE, typename LT, int NT>
__device__ __forceinline__ void fwd_lanes(const KArgs& A, Stage& S, int d, int g, size_t gbase, LT* lv, int v,
                                          long long r0, long long r1, int sub, int nsub, uint64_t& acc, bool& of,
                                          int& we_out, double& ws_out) {
    using Sd = Simd<LT>;
    constexpr int LPW = Sd::LPW, WPV = 32 / LPW, SLOTS = 32 / WPV, ITER = 32 / SLOTS;
    constexpr unsigned PAIR = (LPW == 4) ? 0xFFFFu : 0xFFFFFFFFu;   // level bits of one pair of lanes
    constexpr int WARPS = NT / 32;
    __shared__ uint64_t part_a[WARPS][SLOTS][32];
    __shared__ double part_s[MODE == 2 ? WARPS : 1][SLOTS][32];
    __shared__ unsigned char part_o[WARPS][SLOTS][32];
    const int t = threadIdx.x & 31, s = t / WPV, w = t % WPV, wib = threadIdx.x >> 5;
    const unsigned* lvw = reinterpret_cast<const unsigned*>(lv);
    const unsigned d4 = Sd::bc(d), dp4 = Sd::bc(d - 1);
    const unsigned act4 = Sd::eq(lvw[(size_t)v * WPV + w], d4);
    const uint64_t* sg = A.sig + (gbase << 5) + w * LPW;
    uint64_t a[LPW];
    int we[LPW];
    double ws[LPW];
    unsigned ofm = 0;
#pragma unroll
    for (int j = 0; j < LPW; j++) { a[j] = 0; we[j] = WEMPTY; ws[j] = 0.0; }
    for (long long jb = r0 + 32LL * sub; jb < r1; jb += 32LL * nsub) {
        const int cnt = (int)min(32LL, r1 - jb);
        const int kmax = (cnt + SLOTS - 1) / SLOTS;   // uniform across the warp
        const int xm = (t < cnt) ? A.col[jb + t] : 0;
        unsigned Lw[ITER];
        int xs[ITER];
#pragma unroll
        for (int k = 0; k < ITER; k++) {
            if (k >= kmax) break;
            const int q = k * SLOTS + s;
            xs[k] = __shfl_sync(FULL, xm, q);
            Lw[k] = (q < cnt) ? lvw[(size_t)xs[k] * WPV + w] : d4;
        }
        if (MODE != 0 && d > 0) {
#pragma unroll
            for (int k = 0; k < ITER; k++) {
                if (k >= kmax) break;
                const unsigned pm = Sd::eq(Lw[k], dp4) & act4;
                if (!pm) continue;
                const size_t xo = (size_t)xs[k] << 5;
#pragma unroll
                for (int pr = 0; pr < LPW / 2; pr++) {
                    const unsigned pmp = (pm >> (pr * 2 * (32 / LPW))) & PAIR;
                    if (!pmp) continue;
                    const ulonglong2 vv = *reinterpret_cast<const ulonglong2*>(sg + xo + 2 * pr);
                    const uint64_t v2[2] = {vv.x, vv.y};
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        if (!Sd::has(pm, 2 * pr + h)) continue;
                        if (MODE == 1) {
                            const uint64_t na = a[2 * pr + h] + v2[h];
                            ofm |= (unsigned)(na < a[2 * pr + h]) << (2 * pr + h);
                            a[2 * pr + h] = na;
                        } else {
                            wadd(ws[2 * pr + h], we[2 * pr + h], v2[h]);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < ITER; k++) {
            if (k >= kmax) break;
            const int q = k * SLOTS + s;
            const unsigned un = Sd::eq(Lw[k], 0xFFFFFFFFu) & act4;   // unreached, in active lanes
            if (un) {
                LT* px = lv + ((size_t)xs[k] << 5) + w * LPW;
#pragma unroll
                for (int j = 0; j < LPW; j++)
                    if (Sd::has(un, j)) px[j] = (LT)(d + 1);
            }
            const unsigned bal = __ballot_sync(FULL, un != 0u);
            const unsigned slotm = (bal >> (s * WPV)) & ((1u << WPV) - 1u);
            const bool has = (w == 0) && (q < cnt) && slotm && claim(A, gbase, xs[k], d + 1);
            warp_append(A, S, has, has && is_hub(A, xs[k]), ((uint32_t)xs[k] << 5) | (uint32_t)g);
        }
    }
    if (MODE == 0) return;
    // slot partials -> shared memory (indexed by lane), then thread t adds its lane's slots in order
#pragma unroll
    for (int j = 0; j < LPW; j++) {
        const int lane = w * LPW + j;
        if (MODE == 1) { part_a[wib][s][lane] = a[j]; part_o[wib][s][lane] = (ofm >> j) & 1u; }
        else { part_a[wib][s][lane] = (uint64_t)(long long)we[j]; part_s[wib][s][lane] = ws[j]; }
    }
    __syncwarp();
    if (MODE == 1) {
        uint64_t r = part_a[wib][0][t];
        bool o = part_o[wib][0][t];
#pragma unroll
        for (int k = 1; k < SLOTS; k++) {
            const uint64_t p = part_a[wib][k][t];
            const uint64_t na = r + p;
            o = o || part_o[wib][k][t] || (na < r);
            r = na;
        }
        acc = r;
        of = o;
    } else {
        int ee = (int)(long long)part_a[wib][0][t];
        double ss = part_s[wib][0][t];
#pragma unroll
        for (int k = 1; k < SLOTS; k++) wmerge(ss, ee, part_s[wib][k][t], (int)(long long)part_a[wib][k][t]);
        we_out = ee;
        ws_out = ss;
    }
    __syncwarp();
}

// Lane-parallel dependency scan: sum of sigma(v)*rho(w) (WIDE) or rho(w) over
// successors, predecessor count, for lane t in thread t.  mvt/evt: sigma(v) of
// lane t in wide form.
template <bool WIDE, typename T, typename LT, int NT>
__device__ __forceinline__ void bwd_lanes(const KArgs& A, int d, size_t gbase, const LT* lv, int v, T mvt, int evt,
                                          long long r0, long long r1, int sub, int nsub, T& acc, int& pc) {
    using Sd = Simd<LT>;
    constexpr int LPW = Sd::LPW, WPV = 32 / LPW, SLOTS = 32 / WPV, ITER = 32 / SLOTS;
    constexpr unsigned PAIR = (LPW == 4) ? 0xFFFFu : 0xFFFFFFFFu;
    constexpr int WARPS = NT / 32;
    __shared__ T part_s[WARPS][SLOTS][32];
    __shared__ T part_c[WARPS][SLOTS][32];
    __shared__ int part_p[WARPS][SLOTS][32];
    const int t = threadIdx.x & 31, s = t / WPV, w = t % WPV, wib = threadIdx.x >> 5;
    const unsigned* lvw = reinterpret_cast<const unsigned*>(lv);
    const unsigned d4 = Sd::bc(d), dp4 = Sd::bc(d - 1), dn4 = Sd::bc(d + 1);
    const unsigned act4 = Sd::eq(lvw[(size_t)v * WPV + w], d4);
    const T* rh = reinterpret_cast<const T*>(A.rho) + (gbase << 5) + w * LPW;
    const uint64_t* rw = reinterpret_cast<const uint64_t*>(A.rho) + (gbase << 5) + w * LPW;
    Sum<T> a[LPW];
    int pcs[LPW];
    T mj[LPW];
    int ej[LPW];
#pragma unroll
    for (int j = 0; j < LPW; j++) {
        pcs[j] = 0;
        mj[j] = WIDE ? __shfl_sync(FULL, mvt, w * LPW + j) : T(0);
        ej[j] = WIDE ? __shfl_sync(FULL, evt, w * LPW + j) : 0;
    }
    for (long long jb = r0 + 32LL * sub; jb < r1; jb += 32LL * nsub) {
        const int cnt = (int)min(32LL, r1 - jb);
        const int kmax = (cnt + SLOTS - 1) / SLOTS;
        const int xm = (t < cnt) ? A.col[jb + t] : 0;
        unsigned Lw[ITER];
        int xs[ITER];
#pragma unroll
        for (int k = 0; k < ITER; k++) {
            if (k >= kmax) break;
            const int q = k * SLOTS + s;
            xs[k] = __shfl_sync(FULL, xm, q);
            Lw[k] = (q < cnt) ? lvw[(size_t)xs[k] * WPV + w] : d4;
        }
#pragma unroll
        for (int k = 0; k < ITER; k++) {
            if (k >= kmax) break;
            const unsigned sm = Sd::eq(Lw[k], dn4) & act4;
            if (A.semantics == GBC_BC_REFERENCE) {   // predecessor counts: the reference semantics only
                const unsigned pm = Sd::eq(Lw[k], dp4) & act4;
#pragma unroll
                for (int j = 0; j < LPW; j++) pcs[j] += Sd::has(pm, j);
            }
            if (!sm) continue;
            const size_t xo = (size_t)xs[k] << 5;
            if (!WIDE && sizeof(T) == 4 && LPW == 4) {
                const float4 vv = *reinterpret_cast<const float4*>(rh + xo);
                const float v4[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
                for (int j = 0; j < LPW; j++)
                    if (Sd::has(sm, j)) a[j].add((T)v4[j]);
            } else {
#pragma unroll
                for (int pr = 0; pr < LPW / 2; pr++) {
                    const unsigned smp = (sm >> (pr * 2 * (32 / LPW))) & PAIR;
                    if (!smp) continue;
                    if (WIDE) {
                        const ulonglong2 vv = *reinterpret_cast<const ulonglong2*>(rw + xo + 2 * pr);
                        const uint64_t v2[2] = {vv.x, vv.y};
#pragma unroll
                        for (int h = 0; h < 2; h++)
                            if (Sd::has(sm, 2 * pr + h)) a[2 * pr + h].add(wterm<T>(mj[2 * pr + h], ej[2 * pr + h], v2[h]));
                    } else if (sizeof(T) == 8) {
                        const double2 vv = *reinterpret_cast<const double2*>(reinterpret_cast<const double*>(rh) + xo + 2 * pr);
                        const double v2[2] = {vv.x, vv.y};
#pragma unroll
                        for (int h = 0; h < 2; h++)
                            if (Sd::has(sm, 2 * pr + h)) a[2 * pr + h].add((T)v2[h]);
                    } else {
                        const float2 vv = *reinterpret_cast<const float2*>(rh + xo + 2 * pr);
                        const float v2[2] = {vv.x, vv.y};
#pragma unroll
                        for (int h = 0; h < 2; h++)
                            if (Sd::has(sm, 2 * pr + h)) a[2 * pr + h].add((T)v2[h]);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < LPW; j++) {
        part_s[wib][s][w * LPW + j] = a[j].s;
        part_c[wib][s][w * LPW + j] = a[j].c;
        part_p[wib][s][w * LPW + j] = pcs[j];
    }
    __syncwarp();
    Sum<T> r;
    r.s = part_s[wib][0][t];
    r.c = part_c[wib][0][t];
    int p = part_p[wib][0][t];
#pragma unroll
    for (int k = 1; k < SLOTS; k++) {
        r.merge(part_s[wib][k][t], part_c[wib][k][t]);
        p += part_p[wib][k][t];
    }
    acc = r.value();
    pc = p;
    __syncwarp();
}

// ---- forward --------------------------------------------------------------
// Neighbour chunks r0 + 32*sub, stepping 32*nsub (nsub warps share a hub).
// Pulls sigma from level d-1 neighbours into (acc, of) or (we, ws) and
// discovers level d+1.
template <int MODE, typename LT, int NT>
__device__ __forceinline__ void fwd_scan(const KArgs& A, Stage& S, int d, int g, size_t gbase, LT* lv, int v,
                                         unsigned am, long long r0, long long r1, int sub, int nsub, uint64_t& acc,
                                         bool& of, int& we, double& ws) {
    constexpr LT INF = (LT)Lv<LT>::INF;
    const int t = threadIdx.x & 31;
    const LT dl = (LT)d, dprev = (LT)(d - 1), dnext = (LT)(d + 1);
    if (__popc(am) > A.sparse) {
        fwd_lanes<MODE, LT, NT>(A, S, d, g, gbase, lv, v, r0, r1, sub, nsub, acc, of, we, ws);
    } else {
        // edge-parallel: threads over neighbours, active lanes in turn
        unsigned rem = am;
        while (rem) {
            const int a = __ffs(rem) - 1;
            rem &= rem - 1u;
            uint64_t pacc = 0;
            bool pof = false;
            int pe = WEMPTY;
            double ps = 0.0;
            for (long long jb = r0 + 32LL * sub; jb < r1; jb += 32LL * nsub) {
                const long long j = jb + t;
                bool has = false;
                int x = 0;
                if (j < r1) {
                    x = A.col[j];
                    LT* px = lv + ((size_t)x << 5) + a;
                    const LT Lx = *px;
                    if (MODE != 0 && d > 0 && Lx == dprev) {
                        const uint64_t sv = A.sig[((gbase + (size_t)x) << 5) + a];
                        if (MODE == 1) {
                            const uint64_t na = pacc + sv;
                            pof |= (na < pacc);
                            pacc = na;
                        } else {
                            wadd(ps, pe, sv);
                        }
                    }
                    if (Lx == INF) {
                        *px = dnext;
                        has = claim(A, gbase, x, d + 1);
                    }
                }
                warp_append(A, S, has, has && is_hub(A, x), ((uint32_t)x << 5) | (uint32_t)g);
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
                    const int e2 = __shfl_xor_sync(FULL, pe, o);
                    const double s2 = __shfl_xor_sync(FULL, ps, o);
                    wmerge(ps, pe, s2, e2);
                }
                if (t == a) { we = pe; ws = ps; }
            }
        }
    }
}

// Store sigma of (v, lane a) of group g; flag lanes whose count left the range.
template <int MODE>
__device__ __forceinline__ void fwd_store(const KArgs& A, int g, size_t gbase, int v, int a, uint64_t acc, bool of,
                                          int we, double ws) {
    const size_t vi = ((gbase + (size_t)v) << 5) + a;
    if (MODE == 2) acc = wpack(ws, we, of);
    A.sig[vi] = acc;
    if (of) {
        atomicOr(&A.ovf[g], 1u << a);
        A.ctl->any_ovf = 1;
    }
}

// Light entries, one per thread: the thread walks its entry's active lanes in
// order and, for each, the neighbours in CSR order.  Threads step together so
// that discoveries can be appended warp-wide after every step.
template <int MODE, typename LT>
__device__ __forceinline__ void fwd_light(const KArgs& A, Stage& S, int d, uint32_t ent, unsigned am, long long r0,
                                          long long r1, unsigned long long* cc_sh) {
    constexpr LT INF = (LT)Lv<LT>::INF;
    constexpr int U = LIGHT_U;
    const LT dl = (LT)d, dprev = (LT)(d - 1), dnext = (LT)(d + 1);
    const int v = (int)(ent >> 5), g = (int)(ent & 31u);
    const size_t gbase = (size_t)g * (size_t)A.n;
    LT* lv = reinterpret_cast<LT*>(A.lvl) + (gbase << 5);
    if (MODE == 0 && am) {
        const long long c = (A.w ? (long long)d * (long long)A.w[v] : (long long)d) + (A.ff ? A.ff[v] : 0LL);
        for (unsigned r = am; r; r &= r - 1u) atomicAdd(&cc_sh[g * 32 + __ffs(r) - 1], (unsigned long long)c);
    }
    // one step = up to U neighbours of one active lane, their loads issued together
    const int steps = __popc(am) * (int)((r1 - r0 + U - 1) / U);
    const int maxs = __reduce_max_sync(FULL, steps);
    unsigned rem = am;
    int a = 0;
    long long j = r1;
    uint64_t acc = 0;
    bool of = false;
    int we = WEMPTY;
    double ws = 0.0;
    for (int it = 0; it < maxs; it++) {
        const bool on = it < steps;
        if (on && j == r1) {
            a = __ffs(rem) - 1;
            rem &= rem - 1u;
            j = r0;
            acc = 0;
            of = false;
            we = WEMPTY;
            ws = 0.0;
        }
        int x[U];
        LT L[U];
#pragma unroll
        for (int u = 0; u < U; u++) x[u] = (on && j + u < r1) ? A.col[j + u] : -1;
#pragma unroll
        for (int u = 0; u < U; u++) L[u] = x[u] >= 0 ? lv[((size_t)x[u] << 5) + a] : dl;   // dl: neither case below
        // path-count loads, then the discovery stores and claim atomics, then the sums:
        // the claims' round trip overlaps the loads' instead of following it
        uint64_t sv[U];
#pragma unroll
        for (int u = 0; u < U; u++)
            sv[u] = (MODE != 0 && d > 0 && L[u] == dprev) ? A.sig[((gbase + (size_t)x[u]) << 5) + a] : 0ULL;
        bool has[U];
#pragma unroll
        for (int u = 0; u < U; u++)
            if (L[u] == INF) lv[((size_t)x[u] << 5) + a] = dnext;
#pragma unroll
        for (int u = 0; u < U; u++) has[u] = L[u] == INF && atomicExch(&A.vmark[gbase + x[u]], d + 1) != d + 1;
        if (MODE != 0 && d > 0) {
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (L[u] != dprev) continue;
                if (MODE == 1) {
                    const uint64_t na = acc + sv[u];
                    of |= (na < acc);
                    acc = na;
                } else {
                    wadd(ws, we, sv[u]);
                }
            }
        }
        if (on) {
            j = min(j + U, r1);
            if (j == r1 && MODE != 0 && d > 0) fwd_store<MODE>(A, g, gbase, v, a, acc, of, we, ws);
        }
#pragma unroll
        for (int u = 0; u < U; u++) warp_append(A, S, has[u], has[u] && is_hub(A, x[u]), ((uint32_t)x[u] << 5) | (uint32_t)g);
    }
}

// Forward level kernel.  MODE 0: distances only (closeness sums per lane);
// 1: exact uint64 sigma; 2: wide-exponent sigma.
template <int MODE, typename LT, int NT>
__global__ void __launch_bounds__(NT, (MINB<LT, MODE == 2, NT>)) expand_kernel(KArgs A) {
    constexpr int WARPS = NT / 32;
    __shared__ unsigned long long cc_sh[MODE == 0 ? 32 * 32 : 1];
    __shared__ uint64_t h_acc[WARPS][32];
    __shared__ double h_ws[MODE == 2 ? WARPS : 1][32];
    __shared__ unsigned char h_of[WARPS][32];
    __shared__ uint32_t stg[WARPS][STG];
    __shared__ unsigned long long s_i;
    if (MODE == 0) {
        for (int i = threadIdx.x; i < A.ng * 32; i += blockDim.x) cc_sh[i] = 0ULL;
        __syncthreads();
    }
    const int done = *(volatile int*)&A.ctl->done;
    const int d = *(volatile int*)&A.ctl->level;
    const int t = threadIdx.x & 31, wib = threadIdx.x >> 5;
    Stage S{stg[wib], 0};
    unsigned long long vis = 0;
    if (!done) {
        const LT dl = (LT)d;
        // hub entries: one CTA per entry, warps split the neighbours
        const unsigned long long he = A.hoff[d + 1];
        for (;;) {
            if (threadIdx.x == 0) s_i = atomicAdd(&A.ctl->hnext, 1ULL);
            __syncthreads();
            const unsigned long long i = s_i;
            __syncthreads();
            if (i >= he) break;
            const uint32_t ent = A.hq[i];
            const int v = (int)(ent >> 5), g = (int)(ent & 31u);
            const size_t gbase = (size_t)g * (size_t)A.n;
            LT* lv = reinterpret_cast<LT*>(A.lvl) + (gbase << 5);
            const bool act = (lv[((size_t)v << 5) + t] == dl);
            const unsigned am = __ballot_sync(FULL, act);
            if (am == 0u) continue;   // uniform across the CTA
            if (threadIdx.x == 0) vis += (unsigned long long)(A.row[v + 1] - A.row[v]);
            if (MODE == 0 && act && wib == 0) {
                const long long c = (A.w ? (long long)d * (long long)A.w[v] : (long long)d) + (A.ff ? A.ff[v] : 0LL);
                atomicAdd(&cc_sh[g * 32 + t], (unsigned long long)c);
            }
            uint64_t acc = 0;
            bool of = false;
            int we = WEMPTY;
            double ws = 0.0;
            fwd_scan<MODE, LT, NT>(A, S, d, g, gbase, lv, v, am, A.row[v], A.row[v + 1], wib, WARPS, acc, of, we, ws);
            if (MODE != 0) {
                if (MODE == 1) h_acc[wib][t] = acc;
                else { h_acc[wib][t] = (uint64_t)(long long)we; h_ws[wib][t] = ws; }
                h_of[wib][t] = of;
                __syncthreads();
                if (wib == 0 && act && d > 0) {
                    for (int w = 1; w < WARPS; w++) {
                        if (MODE == 1) {
                            const uint64_t na = acc + h_acc[w][t];
                            of = of || h_of[w][t] || (na < acc);
                            acc = na;
                        } else {
                            wmerge(ws, we, h_ws[w][t], (int)(long long)h_acc[w][t]);
                        }
                    }
                    fwd_store<MODE>(A, g, gbase, v, t, acc, of, we, ws);
                }
                __syncthreads();
            }
        }
        // regular entries: a warp takes FETCH per fetch; light ones are expanded
        // one per thread, the others by the whole warp in turn
        const unsigned long long e = A.foff[d + 1];
        bool first = true;
        for (;;) {
            const unsigned long long base = warp_fetch(A, d, first);
            if (base >= e) break;
            uint32_t ent;
            unsigned am;
            long long r0, r1;
            fetch_entry<LT>(A, d, base + t, e, ent, am, r0, r1);
            if (am) vis += (unsigned long long)(r1 - r0);
            const bool light = am && (long long)__popc(am) * (r1 - r0) <= A.light;
            fwd_light<MODE, LT>(A, S, d, ent, light ? am : 0u, r0, r1, cc_sh);
            unsigned hv = __ballot_sync(FULL, am && !light);
            while (hv) {
                const int k = __ffs(hv) - 1;
                hv &= hv - 1u;
                const uint32_t ek = __shfl_sync(FULL, ent, k);
                const unsigned amk = __shfl_sync(FULL, am, k);
                const long long k0 = __shfl_sync(FULL, r0, k), k1 = __shfl_sync(FULL, r1, k);
                const int v = (int)(ek >> 5), g = (int)(ek & 31u);
                const size_t gbase = (size_t)g * (size_t)A.n;
                LT* lv = reinterpret_cast<LT*>(A.lvl) + (gbase << 5);
                const bool act = (amk >> t) & 1u;
                if (MODE == 0 && act) {
                    const long long c = (A.w ? (long long)d * (long long)A.w[v] : (long long)d) + (A.ff ? A.ff[v] : 0LL);
                    atomicAdd(&cc_sh[g * 32 + t], (unsigned long long)c);
                }
                uint64_t acc = 0;
                bool of = false;
                int we = WEMPTY;
                double ws = 0.0;
                fwd_scan<MODE, LT, NT>(A, S, d, g, gbase, lv, v, amk, k0, k1, 0, 1, acc, of, we, ws);
                if (MODE != 0 && act && d > 0) fwd_store<MODE>(A, g, gbase, v, t, acc, of, we, ws);
            }
        }
    }
    stage_flush(A, S);
    add_visits(A, vis);
    if (MODE == 0) {
        __syncthreads();
        for (int i = threadIdx.x; i < A.ng * 32; i += blockDim.x)
            if (cc_sh[i]) atomicAdd(&A.cc[i], cc_sh[i]);
    }
    fwd_last_block(A, d, done, Lv<LT>::MAXD);
}

// ---- dependency sweep -------------------------------------------------------
// WIDE: sigma in wide form, rho(w) = (1 + delta(w)) / sigma(w) also in wide
// form, and each successor term sigma(v)*rho(w) formed as a plain T.
template <bool WIDE, typename T, typename LT, int NT>
__device__ __forceinline__ void bwd_scan(const KArgs& A, int d, size_t gbase, const LT* lv, int v, unsigned am, T mv,
                                         int ev, long long r0, long long r1, int sub, int nsub, T& acc, int& pc) {
    const int t = threadIdx.x & 31;
    const LT dprev = (LT)(d - 1), dnext = (LT)(d + 1);
    const T* rho = reinterpret_cast<const T*>(A.rho);
    const uint64_t* rw = reinterpret_cast<const uint64_t*>(A.rho);
    if (__popc(am) > A.sparse) {
        bwd_lanes<WIDE, T, LT, NT>(A, d, gbase, lv, v, mv, ev, r0, r1, sub, nsub, acc, pc);
    } else {
        unsigned rem = am;
        while (rem) {
            const int a = __ffs(rem) - 1;
            rem &= rem - 1u;
            const T mva = WIDE ? __shfl_sync(FULL, mv, a) : T(0);
            const int eva = WIDE ? __shfl_sync(FULL, ev, a) : 0;
            Sum<T> ps;
            int ppc = 0;
            for (long long jb = r0 + 32LL * sub; jb < r1; jb += 32LL * nsub) {
                const long long j = jb + t;
                if (j < r1) {
                    const int x = A.col[j];
                    const LT Lx = lv[((size_t)x << 5) + a];
                    if (Lx == dnext) {
                        const size_t xi = ((gbase + (size_t)x) << 5) + a;
                        ps.add(WIDE ? wterm<T>(mva, eva, rw[xi]) : rho[xi]);
                    } else if (Lx == dprev) {
                        ppc++;
                    }
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const T s2 = __shfl_xor_sync(FULL, ps.s, o), c2 = __shfl_xor_sync(FULL, ps.c, o);
                ps.merge(s2, c2);
                ppc += __shfl_xor_sync(FULL, ppc, o);
            }
            if (t == a) { acc = ps.value(); pc = ppc; }
        }
    }
}

// delta and rho of (v, lane a) of group g from the successor sum; returns the
// lane's BC contribution to v.
template <bool WIDE, typename T>
__device__ __forceinline__ double bwd_lane(const KArgs& A, int g, size_t gbase, int v, int a, T mv, int ev, T acc,
                                           int pc, bool refsem) {
    const size_t vi = ((gbase + (size_t)v) << 5) + a;
    // with vertex weights (reach of folded vertices) a target v counts w[v]
    // times and a source s contributes w[s] times
    const T tw = A.w ? (T)A.w[v] : T(1);
    T delta;
    if (WIDE) {
        delta = acc;
        bool of = false;
        reinterpret_cast<uint64_t*>(A.rho)[vi] = wpack((T)((tw + delta) / mv), -ev, of);
    } else {
        const T sv = (T)A.sig[vi];
        delta = sv * acc;
        reinterpret_cast<T*>(A.rho)[vi] = (tw + delta) / sv;
    }
    return (double)delta * (double)A.srcw[(g << 5) + a] * (refsem ? (double)pc : 1.0);
}

// Lane t of (v, g), warp-summed into bcg.
template <bool WIDE, typename T>
__device__ __forceinline__ void bwd_finish(const KArgs& A, int g, size_t gbase, int v, bool act, T mv, int ev, T acc,
                                           int pc, bool refsem) {
    const int t = threadIdx.x & 31;
    double contrib = act ? bwd_lane<WIDE, T>(A, g, gbase, v, t, mv, ev, acc, pc, refsem) : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(FULL, contrib, o);
    if (t == 0) atomicAdd(&A.bcg[gbase + v], contrib);   // one writer per (v, g) and level: a fire-and-forget add
}

// Light entries, one per thread: lanes in order, neighbours in CSR order.
template <bool WIDE, typename T, typename LT>
__device__ __forceinline__ void bwd_light(const KArgs& A, int d, uint32_t ent, unsigned am, long long r0, long long r1,
                                          bool refsem) {
    if (!am) return;
    constexpr int U = LIGHT_U;
    const LT dl = (LT)d, dprev = (LT)(d - 1), dnext = (LT)(d + 1);
    const int v = (int)(ent >> 5), g = (int)(ent & 31u);
    const size_t gbase = (size_t)g * (size_t)A.n;
    const LT* lv = reinterpret_cast<const LT*>(A.lvl) + (gbase << 5);
    const T* rho = reinterpret_cast<const T*>(A.rho);
    const uint64_t* rw = reinterpret_cast<const uint64_t*>(A.rho);
    double contrib = 0.0;
    for (unsigned rem = am; rem; rem &= rem - 1u) {
        const int a = __ffs(rem) - 1;
        T mv = T(0);
        int ev = 0;
        if (WIDE) {
            const uint64_t sw = A.sig[((gbase + (size_t)v) << 5) + a];
            mv = wmant<T>(sw);
            ev = wexp(sw);
        }
        Sum<T> acc;
        int pc = 0;
        // U neighbours per step: their column, level and rho loads issued together
        for (long long j = r0; j < r1; j += U) {
            int x[U];
            LT L[U];
#pragma unroll
            for (int u = 0; u < U; u++) x[u] = j + u < r1 ? A.col[j + u] : -1;
#pragma unroll
            for (int u = 0; u < U; u++) L[u] = x[u] >= 0 ? lv[((size_t)x[u] << 5) + a] : dl;
            uint64_t rv[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const size_t xi = ((gbase + (size_t)x[u]) << 5) + a;
                rv[u] = 0;
                if (L[u] == dnext) {
                    if (WIDE || sizeof(T) == 8) rv[u] = rw[xi];
                    else rv[u] = __float_as_uint(reinterpret_cast<const float*>(rho)[xi]);
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (L[u] == dnext) {
                    if (WIDE) acc.add(wterm<T>(mv, ev, rv[u]));
                    else if (sizeof(T) == 8) acc.add((T)__longlong_as_double((long long)rv[u]));
                    else acc.add((T)__uint_as_float((unsigned)rv[u]));
                } else if (L[u] == dprev) {
                    pc++;
                }
            }
        }
        contrib += bwd_lane<WIDE, T>(A, g, gbase, v, a, mv, ev, acc.value(), pc, refsem);
    }
    atomicAdd(&A.bcg[gbase + v], contrib);   // one writer per (v, g) and level: a fire-and-forget add
}

template <bool WIDE, typename T, typename LT, int NT>
__global__ void __launch_bounds__(NT, 4 * 256 / NT) backward_kernel(KArgs A) {
    constexpr int WARPS = NT / 32;
    __shared__ double h_acc[WARPS][32];
    __shared__ int h_pc[WARPS][32];
    __shared__ unsigned long long s_i;
    const int d = *(volatile int*)&A.ctl->level;
    const int t = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const bool refsem = (A.semantics == GBC_BC_REFERENCE);
    if (d >= 1) {
        const LT dl = (LT)d;
        const unsigned long long he = A.hoff[d + 1];
        for (;;) {
            if (threadIdx.x == 0) s_i = atomicAdd(&A.ctl->hnext, 1ULL);
            __syncthreads();
            const unsigned long long i = s_i;
            __syncthreads();
            if (i >= he) break;
            const uint32_t ent = A.hq[i];
            const int v = (int)(ent >> 5), g = (int)(ent & 31u);
            const size_t gbase = (size_t)g * (size_t)A.n;
            const LT* lv = reinterpret_cast<const LT*>(A.lvl) + (gbase << 5);
            const bool act = (lv[((size_t)v << 5) + t] == dl);
            const unsigned am = __ballot_sync(FULL, act);
            if (am == 0u) continue;
            const uint64_t sw = (WIDE && act) ? A.sig[((gbase + (size_t)v) << 5) + t] : 0ULL;
            const T mv = (WIDE && act) ? wmant<T>(sw) : T(0);
            const int ev = (WIDE && act) ? wexp(sw) : 0;
            T acc = T(0);
            int pc = 0;
            bwd_scan<WIDE, T, LT, NT>(A, d, gbase, lv, v, am, mv, ev, A.row[v], A.row[v + 1], wib, WARPS, acc, pc);
            h_acc[wib][t] = (double)acc;
            h_pc[wib][t] = pc;
            __syncthreads();
            if (wib == 0) {
                for (int w = 1; w < WARPS; w++) {
                    acc += (T)h_acc[w][t];
                    pc += h_pc[w][t];
                }
                bwd_finish<WIDE, T>(A, g, gbase, v, act, mv, ev, acc, pc, refsem);
            }
            __syncthreads();
        }
        const unsigned long long e = A.foff[d + 1];
        bool first = true;
        for (;;) {
            const unsigned long long base = warp_fetch(A, d, first);
            if (base >= e) break;
            uint32_t ent;
            unsigned am;
            long long r0, r1;
            fetch_entry<LT>(A, d, base + t, e, ent, am, r0, r1);
            const bool light = am && (long long)__popc(am) * (r1 - r0) <= A.light;
            bwd_light<WIDE, T, LT>(A, d, ent, light ? am : 0u, r0, r1, refsem);
            unsigned hv = __ballot_sync(FULL, am && !light);
            while (hv) {
                const int k = __ffs(hv) - 1;
                hv &= hv - 1u;
                const uint32_t ek = __shfl_sync(FULL, ent, k);
                const unsigned amk = __shfl_sync(FULL, am, k);
                const long long k0 = __shfl_sync(FULL, r0, k), k1 = __shfl_sync(FULL, r1, k);
                const int v = (int)(ek >> 5), g = (int)(ek & 31u);
                const size_t gbase = (size_t)g * (size_t)A.n;
                const LT* lv = reinterpret_cast<const LT*>(A.lvl) + (gbase << 5);
                const bool act = (amk >> t) & 1u;
                const uint64_t sw = (WIDE && act) ? A.sig[((gbase + (size_t)v) << 5) + t] : 0ULL;
                const T mv = (WIDE && act) ? wmant<T>(sw) : T(0);
                const int ev = (WIDE && act) ? wexp(sw) : 0;
                T acc = T(0);
                int pc = 0;
                bwd_scan<WIDE, T, LT, NT>(A, d, gbase, lv, v, amk, mv, ev, k0, k1, 0, 1, acc, pc);
                bwd_finish<WIDE, T>(A, g, gbase, v, act, mv, ev, acc, pc, refsem);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&A.ctl->blocks, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            A.ctl->blocks = 0;
            if (d >= 1) {
                A.ctl->level = d - 1;
                A.ctl->next = A.foff[d - 1];
                A.ctl->hnext = A.hoff[d - 1];
            }
        }
    }
}

// ---- 128-lane groups ---------------------------------------------------------
// A lane group of 128 sources: thread t of a warp owns lanes 4t..4t+3, so one
// warp-wide load of a neighbour's level row (128 B with 8-bit levels) serves
// the whole group, and a thread keeps its four lanes' sums to itself (no
// cross-thread combine).  With lanes that move together (sources grouped by
// level profile on a power-law graph), 128-lane groups carry the same work
// in about 0.3x the frontier entries and neighbour visits of 32-lane groups.

// The four levels of lanes 4t..4t+3 in one row, and 4-bit lane masks of them.
template <typename LT> struct Quad;
template <> struct Quad<uint8_t> {
    unsigned w;
    __device__ static __forceinline__ Quad load(const uint8_t* row, int t) {
        return {reinterpret_cast<const unsigned*>(row)[t]};
    }
    __device__ static __forceinline__ Quad none() { return {0xFFFFFFFFu}; }
    __device__ static __forceinline__ unsigned bits(unsigned m) { return ((m & 0x80808080u) * 0x00204081u) >> 28; }
    // 0x80 in every zero byte of x, 0 elsewhere: the masked add cannot carry
    // across bytes, so each byte's result is exact
    __device__ static __forceinline__ unsigned zero_bytes(unsigned x) {
        return ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u;
    }
    __device__ __forceinline__ unsigned eq(int d) const {
        return (zero_bytes(w ^ Simd<uint8_t>::bc(d)) * 0x00204081u) >> 28;
    }
    __device__ __forceinline__ unsigned gt(int d) const { return bits(__vcmpgtu4(w, Simd<uint8_t>::bc(d))); }
    __device__ __forceinline__ unsigned unreached() const { return (zero_bytes(~w) * 0x00204081u) >> 28; }
};
template <> struct Quad<uint16_t> {
    uint2 w;
    __device__ static __forceinline__ Quad load(const uint16_t* row, int t) {
        return {reinterpret_cast<const uint2*>(row)[t]};
    }
    __device__ static __forceinline__ Quad none() { return {make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu)}; }
    __device__ static __forceinline__ unsigned bits(unsigned m) { return ((m & 0x80008000u) * 0x8001u) >> 30; }
    __device__ __forceinline__ unsigned eq(int d) const {
        const unsigned b = Simd<uint16_t>::bc(d);
        return bits(__vcmpeq2(w.x, b)) | (bits(__vcmpeq2(w.y, b)) << 2);
    }
    __device__ __forceinline__ unsigned gt(int d) const {
        const unsigned b = Simd<uint16_t>::bc(d);
        return bits(__vcmpgtu2(w.x, b)) | (bits(__vcmpgtu2(w.y, b)) << 2);
    }
    __device__ __forceinline__ unsigned unreached() const {
        return bits(__vcmpeq2(w.x, 0xFFFFFFFFu)) | (bits(__vcmpeq2(w.y, 0xFFFFFFFFu)) << 2);
    }
};

// Exact path counts of 128-lane groups are stored in SB bytes per lane (8,
// or 4 / 2 while every count of the graph fits, which keeps the predecessor
// reads of the forward at 512 / 256 instead of 1024 bytes per neighbour row).
template <int SB> struct SigW;
template <> struct SigW<8> { using type = uint64_t; static constexpr uint64_t MAXV = ~0ULL; };
template <> struct SigW<4> { using type = uint32_t; static constexpr uint64_t MAXV = 0xFFFFFFFFULL; };
template <> struct SigW<2> { using type = uint16_t; static constexpr uint64_t MAXV = 0xFFFFULL; };

constexpr int Q_ITER = 8;   // neighbours whose level quads are loaded before any is used
constexpr int FETCH_Q = 8;  // regular tasks a warp takes per fetch in 128-lane groups (8: 3% faster than 32 on R-MAT s22)
constexpr unsigned long long TAIL_Q = 16384;   // fewer regular tasks left than this: take one per fetch

// Column of thread t in the chunk of 32 neighbours starting at jb (0 past r1).
// The scans load the next chunk's columns while they work on the current one,
// and a task's first chunk is loaded with its own level row, so a column load
// is never a round trip of its own.
__device__ __forceinline__ int q_col(const KArgs& A, long long jb, long long r1) {
    const long long j = jb + (threadIdx.x & 31);
    return j < r1 ? A.col[j] : 0;
}

// Next regular tasks of the level for this warp: FETCH_Q per atomic while
// many remain, then one at a time, so that no warp is left holding several
// heavy tasks while the rest of the GPU has finished the level.
__device__ __forceinline__ unsigned long long q_fetch(const KArgs& A, unsigned long long e, int& take) {
    unsigned long long base = 0;
    int tk = FETCH_Q;
    if ((threadIdx.x & 31) == 0) {
        const unsigned long long cur = *(volatile unsigned long long*)&A.ctl->next;
        tk = cur + TAIL_Q < e ? FETCH_Q : 1;
        base = atomicAdd(&A.ctl->next, (unsigned long long)tk);
    }
    take = __shfl_sync(FULL, tk, 0);
    return __shfl_sync(FULL, base, 0);
}

// Forward scan of one (v, g) task over neighbour chunks r0 + 32*sub, step
// 32*nsub: thread t pulls sigma for its active lanes (act4) and discovers
// level d+1.  Results stay in the thread: acc/ofm (exact) or ws/we (wide).
template <int MODE, typename LT, int SB>
__device__ __forceinline__ void q_fwd_scan(const KArgs& A, Stage& S, int d, int g, size_t gbase, LT* lv, unsigned act4,
                                           long long r0, long long r1, int sub, int nsub, int xm0, uint64_t (&acc)[4],
                                           unsigned& ofm, int (&we)[4], double (&ws)[4]) {
    const int t = threadIdx.x & 31;
    // 2-byte counts: 32-bit sums, clamped to 2^16 after every chunk of 32 neighbours (a lane past
    // 2^16 - 1 is over the width, so its batch is redone wider), so that they never wrap
    unsigned a32[4] = {0u, 0u, 0u, 0u};
    int xm = xm0;   // columns of the chunk at r0 + 32*sub
    for (long long jb = r0 + 32LL * sub; jb < r1; jb += 32LL * nsub, xm = xm0) {
        const int cnt = (int)min(32LL, r1 - jb);
        xm0 = q_col(A, jb + 32LL * nsub, r1);   // the next chunk's columns
        unsigned want = 0;   // bit k: neighbour jb + k had an active lane unreached (d+1 stored there)
        for (int k0 = 0; k0 < cnt; k0 += Q_ITER) {          // uniform across the warp
            Quad<LT> q[Q_ITER];
            int xs[Q_ITER];
#pragma unroll
            for (int i = 0; i < Q_ITER; i++) {
                xs[i] = __shfl_sync(FULL, xm, (k0 + i) & 31);
                q[i] = (k0 + i < cnt && act4) ? Quad<LT>::load(lv + ((size_t)xs[i] << 7), t) : Quad<LT>::none();
            }
            if (MODE != 0 && d > 0) {
#pragma unroll
                for (int i = 0; i < Q_ITER; i++) {
                    const unsigned pm = (k0 + i < cnt) ? (q[i].eq(d - 1) & act4) : 0u;
                    if (!pm) continue;
                    if (MODE == 1 && SB < 8) {
                        // narrow counts: the four lanes in one 8- or 16-byte load; no carry in a 64-bit sum
                        const typename SigW<SB>::type* sn =
                            reinterpret_cast<const typename SigW<SB>::type*>(A.sig) + ((gbase + (size_t)xs[i]) << 7) + 4 * t;
                        unsigned w4[4];
                        if (SB == 4) {
                            const uint4 w = *reinterpret_cast<const uint4*>(sn);
                            w4[0] = w.x; w4[1] = w.y; w4[2] = w.z; w4[3] = w.w;
                        } else {
                            const uint2 w = *reinterpret_cast<const uint2*>(sn);
                            w4[0] = w.x & 0xFFFFu; w4[1] = w.x >> 16; w4[2] = w.y & 0xFFFFu; w4[3] = w.y >> 16;
                        }
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            if (!((pm >> j) & 1u)) continue;
                            if (SB == 2) a32[j] += w4[j];
                            else acc[j] += w4[j];
                        }
                        continue;
                    }
                    const uint64_t* sg = A.sig + ((gbase + (size_t)xs[i]) << 7) + 4 * t;
#pragma unroll
                    for (int pr = 0; pr < 2; pr++) {
                        if (!((pm >> (2 * pr)) & 3u)) continue;
                        const ulonglong2 vv = *reinterpret_cast<const ulonglong2*>(sg + 2 * pr);
                        const uint64_t v2[2] = {vv.x, vv.y};
#pragma unroll
                        for (int h = 0; h < 2; h++) {
                            const int j = 2 * pr + h;
                            if (!((pm >> j) & 1u)) continue;
                            if (MODE == 1) {
                                const uint64_t na = acc[j] + v2[h];
                                ofm |= (unsigned)(na < acc[j]) << j;
                                acc[j] = na;
                            } else {
                                wadd(ws[j], we[j], v2[h]);
                            }
                        }
                    }
                }
            }
            // discovery: store d+1 in the unreached active lanes; bit i of mine: neighbour k0+i had one
            unsigned mine = 0;
#pragma unroll
            for (int i = 0; i < Q_ITER; i++) {
                const bool inr = k0 + i < cnt;
                const unsigned un = inr ? (q[i].unreached() & act4) : 0u;
                if (un) {
                    LT* px = lv + ((size_t)xs[i] << 7) + 4 * t;
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if ((un >> j) & 1u) px[j] = (LT)(d + 1);
                    mine |= 1u << i;
                }
            }
            want |= __reduce_or_sync(FULL, mine) << k0;
        }
        // claims of the whole 32-neighbour chunk at once: thread k claims its own
        // column xm, so one claim round trip serves up to 32 neighbours
        const bool has = ((want >> t) & 1u) && claim(A, gbase, xm, d + 1);
        if (MODE == 0 && has) S.fdeg += (unsigned long long)(A.row[xm + 1] - A.row[xm]);
        warp_append(A, S, has, has && is_hub(A, xm), ((uint32_t)xm << 5) | (uint32_t)g);
        if (MODE == 1 && SB == 2) {
#pragma unroll
            for (int j = 0; j < 4; j++) a32[j] = min(a32[j], 0x10000u);
        }
    }
    if (MODE == 1 && SB == 2) {
#pragma unroll
        for (int j = 0; j < 4; j++) acc[j] += a32[j];
    }
}

// Store sigma of thread t's active lanes of (v, g); flag lanes past the range.
template <int MODE, int SB>
__device__ __forceinline__ void q_fwd_store(const KArgs& A, int g, size_t gbase, int v, unsigned act4,
                                            const uint64_t (&acc)[4], unsigned ofm, const int (&we)[4],
                                            const double (&ws)[4]) {
    const int t = threadIdx.x & 31;
    typedef typename SigW<(MODE == 1 ? SB : 8)>::type ST;
    ST* sv = reinterpret_cast<ST*>(A.sig) + ((gbase + (size_t)v) << 7) + 4 * t;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        if (!((act4 >> j) & 1u)) continue;
        bool of = (ofm >> j) & 1u;
        if (MODE == 1 && SB < 8) of = of || acc[j] > SigW<(MODE == 1 ? SB : 8)>::MAXV;   // the batch is redone wider
        sv[j] = MODE == 2 ? (ST)wpack(ws[j], we[j], of) : (ST)acc[j];
        if (of) {
            const int lane = (g << 7) + 4 * t + j;
            atomicOr(&A.ovf[lane >> 5], 1u << (lane & 31));
            A.ctl->any_ovf = 1;
        }
    }
}

// Edge-parallel forward for tasks with few active lanes: threads over
// neighbours, one active lane at a time; the lane's owner keeps the sum.
template <int MODE, typename LT, int SB>
__device__ __forceinline__ void q_fwd_edges(const KArgs& A, Stage& S, int d, int g, size_t gbase, LT* lv, unsigned act4,
                                            long long r0, long long r1, int sub, int nsub, uint64_t (&acc)[4],
                                            unsigned& ofm, int (&we)[4], double (&ws)[4]) {
    constexpr LT INF = (LT)Lv<LT>::INF;
    const int t = threadIdx.x & 31;
    const LT dl = (LT)d, dprev = (LT)(d - 1), dnext = (LT)(d + 1);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        unsigned owners = __ballot_sync(FULL, (act4 >> j) & 1u);
        while (owners) {
            const int o = __ffs(owners) - 1;
            owners &= owners - 1u;
            const int a = 4 * o + j;
            uint64_t pacc = 0;
            bool pof = false;
            int pe = WEMPTY;
            double ps = 0.0;
            for (long long jb = r0 + 32LL * sub; jb < r1; jb += 32LL * nsub) {
                const long long jj = jb + t;
                bool has = false;
                int x = 0;
                if (jj < r1) {
                    x = A.col[jj];
                    LT* px = lv + ((size_t)x << 7) + a;
                    const LT Lx = *px;
                    if (MODE != 0 && d > 0 && Lx == dprev) {
                        const uint64_t sv = (MODE == 1 && SB < 8)
                            ? (uint64_t)reinterpret_cast<const typename SigW<(MODE == 1 ? SB : 8)>::type*>(A.sig)[((gbase + (size_t)x) << 7) + a]
                            : A.sig[((gbase + (size_t)x) << 7) + a];
                        if (MODE == 1) {
                            const uint64_t na = pacc + sv;
                            pof |= (na < pacc);
                            pacc = na;
                        } else {
                            wadd(ps, pe, sv);
                        }
                    }
                    if (Lx == INF) {
                        *px = dnext;
                        has = claim(A, gbase, x, d + 1);
                    }
                }
                if (MODE == 0 && has) S.fdeg += (unsigned long long)(A.row[x + 1] - A.row[x]);
                warp_append(A, S, has, has && is_hub(A, x), ((uint32_t)x << 5) | (uint32_t)g);
            }
            if (MODE == 1) {
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const uint64_t p2 = __shfl_xor_sync(FULL, pacc, off);
                    const int f2 = __shfl_xor_sync(FULL, (int)pof, off);
                    const uint64_t na = pacc + p2;
                    pof = pof || f2 || (na < pacc);
                    pacc = na;
                }
                if (t == o) {
                    acc[j] = pacc;
                    ofm |= (unsigned)pof << j;
                }
            } else if (MODE == 2) {
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const int e2 = __shfl_xor_sync(FULL, pe, off);
                    const double s2 = __shfl_xor_sync(FULL, ps, off);
                    wmerge(ps, pe, s2, e2);
                }
                if (t == o) { we[j] = pe; ws[j] = ps; }
            }
        }
    }
}

template <int MODE, typename LT>
__device__ __forceinline__ void q_cc_add(const KArgs& A, unsigned long long* cc_sh, int d, int g, int v, unsigned act4) {
    if (MODE != 0 || !act4) return;
    const int t = threadIdx.x & 31;
    const long long c = (A.w ? (long long)d * (long long)A.w[v] : (long long)d) + (A.ff ? A.ff[v] : 0LL);
#pragma unroll
    for (int j = 0; j < 4; j++)
        if ((act4 >> j) & 1u) atomicAdd(&cc_sh[(g << 7) + 4 * t + j], (unsigned long long)c);
}

// ---- bottom-up closeness levels (128-lane groups) ---------------------------
constexpr int BU_WORDS = 4;   // done-bitmap words (32 vertices of one group each) a warp takes per fetch

// One (x, g) of a bottom-up level: the lanes of x still unreached, among those
// whose source lies in x's component, look for a level-d neighbour; the scan
// stops as soon as every one of them has found one.  Returns true when no
// such lane is left (x is done in group g).
template <typename LT>
__device__ __forceinline__ bool q_bu_vertex(const KArgs& A, Stage& S, int d, int g, int x, unsigned long long& mu) {
    const int t = threadIdx.x & 31;
    LT* lv = reinterpret_cast<LT*>(A.lvl) + (((size_t)g * (size_t)A.n) << 7);
    LT* own = lv + ((size_t)x << 7);
    unsigned um = Quad<LT>::load(own, t).unreached();
    if (!__any_sync(FULL, um != 0u)) return true;
    {
        const int cx = A.vcomp[x];
        const int4 c4 = *reinterpret_cast<const int4*>(A.lcomp + (g << 7) + 4 * t);
        um &= (unsigned)(c4.x == cx) | ((unsigned)(c4.y == cx) << 1) | ((unsigned)(c4.z == cx) << 2) |
              ((unsigned)(c4.w == cx) << 3);
    }
    if (!__any_sync(FULL, um != 0u)) return true;
    const long long r0 = A.row[x], r1 = A.row[x + 1];
    unsigned found = 0;
    bool open = true;   // uniform: some lane is still looking
    for (long long jb = r0; jb < r1 && open; jb += 32) {
        const int cnt = (int)min(32LL, r1 - jb);
        const int ym = (t < cnt) ? A.col[jb + t] : 0;
        for (int k0 = 0; k0 < cnt && open; k0 += Q_ITER) {
            Quad<LT> q[Q_ITER];
#pragma unroll
            for (int i = 0; i < Q_ITER; i++) {
                const int y = __shfl_sync(FULL, ym, (k0 + i) & 31);
                q[i] = (k0 + i < cnt) ? Quad<LT>::load(lv + ((size_t)y << 7), t) : Quad<LT>::none();
            }
#pragma unroll
            for (int i = 0; i < Q_ITER; i++) {
                const unsigned f = q[i].eq(d) & um;
                found |= f;
                um &= ~f;
            }
            open = __any_sync(FULL, um != 0u);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; j++)
        if ((found >> j) & 1u) own[4 * t + j] = (LT)(d + 1);
    const long long dx = r1 - r0;
    if (__any_sync(FULL, found != 0u)) {
        if (t == 0) {
            A.vmark[(size_t)g * A.n + x] = d + 1;
            S.fdeg += (unsigned long long)dx;
        }
        warp_append(A, S, t == 0, is_hub(A, x), ((uint32_t)x << 5) | (uint32_t)g);
    }
    if (open && t == 0) mu += (unsigned long long)dx;
    return !open;
}

// A bottom-up closeness level d: the closeness terms of the level-d entries
// (which a top-down level adds while expanding them), then discovery of level
// d+1 from the unreached side over every (vertex, group) not yet done.
template <typename LT>
__device__ __forceinline__ void q_bottom_up(const KArgs& A, Stage& S, unsigned long long* cc_sh, int d,
                                            unsigned long long& mu) {
    const int t = threadIdx.x & 31;
    for (int pass = 0; pass < 2; pass++) {
        unsigned long long* ctr = pass == 0 ? &A.ctl->hnext : &A.ctl->next;
        const uint32_t* q = pass == 0 ? A.hq : A.fq;
        const unsigned long long e = pass == 0 ? A.hoff[d + 1] : A.foff[d + 1];
        for (;;) {
            unsigned long long base = 0;
            if (t == 0) base = atomicAdd(ctr, 32ULL);
            base = __shfl_sync(FULL, base, 0);
            if (base >= e) break;
            const uint32_t ment = base + t < e ? q[base + t] : 0u;
            const int cnt = (int)min(32ULL, e - base);
            for (int k = 0; k < cnt; k++) {
                const uint32_t ent = __shfl_sync(FULL, ment, k);
                const int v = (int)(ent >> 5), g = (int)(ent & 31u);
                const LT* lv = reinterpret_cast<const LT*>(A.lvl) + (((size_t)g * (size_t)A.n) << 7);
                q_cc_add<0, LT>(A, cc_sh, d, g, v, Quad<LT>::load(lv + ((size_t)v << 7), t).eq(d));
            }
        }
    }
    const unsigned long long nwords = (unsigned long long)((A.n + 31) >> 5);
    const unsigned long long total = (unsigned long long)A.ng * nwords;
    for (;;) {
        unsigned long long wbase = 0;
        if (t == 0) wbase = atomicAdd(&A.ctl->bnext, (unsigned long long)BU_WORDS);
        wbase = __shfl_sync(FULL, wbase, 0);
        if (wbase >= total) break;
        const int nw = (int)min((unsigned long long)BU_WORDS, total - wbase);
        for (int k = 0; k < nw; k++) {
            const unsigned long long wi = wbase + k;
            const int g = (int)(wi / nwords);
            const int x0 = (int)(wi - (unsigned long long)g * nwords) << 5;
            const uint32_t dw = A.done[wi];
            uint32_t cand = ~dw;
            if (x0 + 32 > A.n) cand &= (1u << (A.n - x0)) - 1u;
            // thread t reads the whole row of vertex x0 + t: rows with no unreached lane are done
            bool un = false;
            if ((cand >> t) & 1u) {
                const uint4* r = reinterpret_cast<const uint4*>(reinterpret_cast<const LT*>(A.lvl) +
                                                                ((((size_t)g * (size_t)A.n) + (size_t)(x0 + t)) << 7));
#pragma unroll
                for (int i = 0; i < (int)(sizeof(LT) * 8); i++) {
                    const uint4 w = r[i];
                    un |= Simd<LT>::any_inf(w.x) | Simd<LT>::any_inf(w.y) | Simd<LT>::any_inf(w.z) | Simd<LT>::any_inf(w.w);
                }
            }
            const uint32_t um32 = __ballot_sync(FULL, un);
            uint32_t nd = cand & ~um32;
            cand &= um32;
            while (cand) {
                const int b = __ffs(cand) - 1;
                cand &= cand - 1u;
                if (q_bu_vertex<LT>(A, S, d, g, x0 + b, mu)) nd |= 1u << b;
            }
            if (nd && t == 0) A.done[wi] = dw | nd;
        }
    }
}

// Forward level kernel, 128-lane groups.
template <int MODE, typename LT, int NT, int SB>
__global__ void __launch_bounds__(NT, 4 * 256 / NT) expand_q_kernel(KArgs A) {
    constexpr int WARPS = NT / 32;
    __shared__ unsigned long long cc_sh[MODE == 0 ? 1024 : 1];
    __shared__ uint64_t h_acc[MODE != 0 ? WARPS : 1][128];
    __shared__ double h_ws[MODE == 2 ? WARPS : 1][128];
    __shared__ unsigned char h_of[MODE != 0 ? WARPS : 1][128];
    __shared__ uint32_t stg[WARPS][STG];
    __shared__ unsigned long long s_i;
    if (MODE == 0) {
        for (int i = threadIdx.x; i < (A.ng << 7); i += blockDim.x) cc_sh[i] = 0ULL;
        __syncthreads();
    }
    const int done = *(volatile int*)&A.ctl->done;
    const int d = *(volatile int*)&A.ctl->level;
    const int t = threadIdx.x & 31, wib = threadIdx.x >> 5;
    Stage S{stg[wib], 0};
    unsigned long long vis = 0;
    const bool bu = MODE == 0 && A.dir && *(volatile int*)&A.ctl->bu;
    unsigned long long mu = 0;
    if (!done && bu) {
        q_bottom_up<LT>(A, S, cc_sh, d, mu);
    } else if (!done) {
        // hub entries: one CTA per entry, warps split the neighbours
        const unsigned long long he = A.hoff[d + 1];
        for (;;) {
            if (threadIdx.x == 0) s_i = atomicAdd(&A.ctl->hnext, 1ULL);
            __syncthreads();
            const unsigned long long i = s_i;
            __syncthreads();
            if (i >= he) break;
            const uint32_t ent = A.hq[i];
            const int v = (int)(ent >> 5), g = (int)(ent & 31u);
            const size_t gbase = (size_t)g * (size_t)A.n;
            LT* lv = reinterpret_cast<LT*>(A.lvl) + (gbase << 7);
            const unsigned act4 = Quad<LT>::load(lv + ((size_t)v << 7), t).eq(d);
            const int nact = __reduce_add_sync(FULL, __popc(act4));
            if (nact == 0) continue;   // uniform across the CTA
            if (threadIdx.x == 0) vis += (unsigned long long)(A.row[v + 1] - A.row[v]);
            if (wib == 0) q_cc_add<MODE, LT>(A, cc_sh, d, g, v, act4);
            uint64_t acc[4] = {0, 0, 0, 0};
            unsigned ofm = 0;
            int we[4] = {WEMPTY, WEMPTY, WEMPTY, WEMPTY};
            double ws[4] = {0.0, 0.0, 0.0, 0.0};
            if (nact > A.sparse) q_fwd_scan<MODE, LT, SB>(A, S, d, g, gbase, lv, act4, A.row[v], A.row[v + 1], wib, WARPS,
                                                      q_col(A, A.row[v] + 32LL * wib, A.row[v + 1]), acc, ofm, we, ws);
            else q_fwd_edges<MODE, LT, SB>(A, S, d, g, gbase, lv, act4, A.row[v], A.row[v + 1], wib, WARPS, acc, ofm, we, ws);
            if (MODE != 0) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int l = 4 * t + j;
                    if (MODE == 1) h_acc[wib][l] = acc[j];
                    else { h_acc[wib][l] = (uint64_t)(long long)we[j]; h_ws[wib][l] = ws[j]; }
                    h_of[wib][l] = (ofm >> j) & 1u;
                }
                __syncthreads();
                if (wib == 0 && act4 && d > 0) {
                    for (int w = 1; w < WARPS; w++) {
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const int l = 4 * t + j;
                            if (MODE == 1) {
                                const uint64_t na = acc[j] + h_acc[w][l];
                                ofm |= (unsigned)(h_of[w][l] || (na < acc[j])) << j;
                                acc[j] = na;
                            } else {
                                wmerge(ws[j], we[j], h_ws[w][l], (int)(long long)h_acc[w][l]);
                            }
                        }
                    }
                    q_fwd_store<MODE, SB>(A, g, gbase, v, act4, acc, ofm, we, ws);
                }
                __syncthreads();
            }
        }
        // regular entries: a warp takes FETCH at a time and expands them in turn
        const unsigned long long e = A.foff[d + 1];
        for (;;) {
            int take;
            const unsigned long long base = q_fetch(A, e, take);
            if (base >= e) break;
            const unsigned long long my = base + t;
            const bool mine = t < take && my < e;
            const uint32_t ment = mine ? A.fq[my] : 0u;
            const long long m0 = mine ? A.row[ment >> 5] : 0, m1 = mine ? A.row[(ment >> 5) + 1] : 0;
            const int cntE = (int)min((unsigned long long)take, e - base);
            for (int k = 0; k < cntE; k++) {
                const uint32_t ent = __shfl_sync(FULL, ment, k);
                const long long r0 = __shfl_sync(FULL, m0, k), r1 = __shfl_sync(FULL, m1, k);
                const int v = (int)(ent >> 5), g = (int)(ent & 31u);
                const size_t gbase = (size_t)g * (size_t)A.n;
                LT* lv = reinterpret_cast<LT*>(A.lvl) + (gbase << 7);
                const unsigned act4 = Quad<LT>::load(lv + ((size_t)v << 7), t).eq(d);
                const int xm0 = q_col(A, r0, r1);   // the first chunk's columns, loaded with the level row
                const int nact = __reduce_add_sync(FULL, __popc(act4));
                if (nact == 0) continue;
                if (t == 0) vis += (unsigned long long)(r1 - r0);
                q_cc_add<MODE, LT>(A, cc_sh, d, g, v, act4);
                uint64_t acc[4] = {0, 0, 0, 0};
                unsigned ofm = 0;
                int we[4] = {WEMPTY, WEMPTY, WEMPTY, WEMPTY};
                double ws[4] = {0.0, 0.0, 0.0, 0.0};
                if (nact > A.sparse) q_fwd_scan<MODE, LT, SB>(A, S, d, g, gbase, lv, act4, r0, r1, 0, 1, xm0, acc, ofm, we, ws);
                else q_fwd_edges<MODE, LT, SB>(A, S, d, g, gbase, lv, act4, r0, r1, 0, 1, acc, ofm, we, ws);
                if (MODE != 0 && d > 0) q_fwd_store<MODE, SB>(A, g, gbase, v, act4, acc, ofm, we, ws);
            }
        }
    }
    stage_flush(A, S);
    add_visits(A, vis);
    if (MODE == 0) {
        if (A.dir) {   // the next level's frontier edges, and the edges left unreached by a bottom-up level
            unsigned long long f = S.fdeg, m = mu;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                f += __shfl_xor_sync(FULL, f, o);
                m += __shfl_xor_sync(FULL, m, o);
            }
            if (t == 0 && f) atomicAdd(&A.ctl->fdeg, f);
            if (t == 0 && m) atomicAdd(&A.ctl->mu, m);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < (A.ng << 7); i += blockDim.x)
            if (cc_sh[i]) atomicAdd(&A.cc[i], cc_sh[i]);
    }
    fwd_last_block(A, d, done, Lv<LT>::MAXD, MODE == 0 && A.dir != 0);
}

// Dependency-sweep scan of one (v, g) task: per active lane of thread t, the
// compensated sum of rho (or sigma(v)*rho in wide form) over successors and
// the predecessor count.
template <bool WIDE, typename T, typename LT>
__device__ __forceinline__ void q_bwd_scan(const KArgs& A, int d, size_t gbase, const LT* lv, unsigned act4,
                                           const T (&mv)[4], const int (&ev)[4], long long r0, long long r1, int sub,
                                           int nsub, int xm0, Sum<T> (&acc)[4], int (&pc)[4]) {
    const int t = threadIdx.x & 31;
    const bool refsem = A.semantics == GBC_BC_REFERENCE;   // predecessor counts: the reference semantics only
    int xm = xm0;   // columns of the chunk at r0 + 32*sub
    for (long long jb = r0 + 32LL * sub; jb < r1; jb += 32LL * nsub, xm = xm0) {
        const int cnt = (int)min(32LL, r1 - jb);
        xm0 = q_col(A, jb + 32LL * nsub, r1);   // the next chunk's columns
        for (int k0 = 0; k0 < cnt; k0 += Q_ITER) {
            Quad<LT> q[Q_ITER];
            int xs[Q_ITER];
#pragma unroll
            for (int i = 0; i < Q_ITER; i++) {
                xs[i] = __shfl_sync(FULL, xm, (k0 + i) & 31);
                q[i] = (k0 + i < cnt && act4) ? Quad<LT>::load(lv + ((size_t)xs[i] << 7), t) : Quad<LT>::none();
            }
#pragma unroll
            for (int i = 0; i < Q_ITER; i++) {
                if (k0 + i >= cnt) continue;
                const unsigned sm = q[i].eq(d + 1) & act4;
                if (refsem) {
                    const unsigned pm = q[i].eq(d - 1) & act4;
#pragma unroll
                    for (int j = 0; j < 4; j++) pc[j] += (pm >> j) & 1u;
                }
                if (!sm) continue;
                const size_t xo = ((gbase + (size_t)xs[i]) << 7) + 4 * t;
                if (WIDE) {
                    const uint64_t* rw = reinterpret_cast<const uint64_t*>(A.rho) + xo;
#pragma unroll
                    for (int pr = 0; pr < 2; pr++) {
                        if (!((sm >> (2 * pr)) & 3u)) continue;
                        const ulonglong2 vv = *reinterpret_cast<const ulonglong2*>(rw + 2 * pr);
                        if ((sm >> (2 * pr)) & 1u) acc[2 * pr].add(wterm<T>(mv[2 * pr], ev[2 * pr], vv.x));
                        if ((sm >> (2 * pr + 1)) & 1u) acc[2 * pr + 1].add(wterm<T>(mv[2 * pr + 1], ev[2 * pr + 1], vv.y));
                    }
                } else if (sizeof(T) == 4) {
                    const float4 vv = *reinterpret_cast<const float4*>(reinterpret_cast<const float*>(A.rho) + xo);
                    const float v4[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if ((sm >> j) & 1u) acc[j].add((T)v4[j]);
                } else {
                    const double* rd = reinterpret_cast<const double*>(A.rho) + xo;
#pragma unroll
                    for (int pr = 0; pr < 2; pr++) {
                        if (!((sm >> (2 * pr)) & 3u)) continue;
                        const double2 vv = *reinterpret_cast<const double2*>(rd + 2 * pr);
                        if ((sm >> (2 * pr)) & 1u) acc[2 * pr].add((T)vv.x);
                        if ((sm >> (2 * pr + 1)) & 1u) acc[2 * pr + 1].add((T)vv.y);
                    }
                }
            }
        }
    }
}

// Edge-parallel sweep for tasks with few active lanes.
template <bool WIDE, typename T, typename LT>
__device__ __forceinline__ void q_bwd_edges(const KArgs& A, int d, size_t gbase, const LT* lv, unsigned act4,
                                            const T (&mv)[4], const int (&ev)[4], long long r0, long long r1, int sub,
                                            int nsub, Sum<T> (&acc)[4], int (&pc)[4]) {
    const int t = threadIdx.x & 31;
    const bool refsem = A.semantics == GBC_BC_REFERENCE;
    const LT dprev = (LT)(d - 1), dnext = (LT)(d + 1);
    const T* rho = reinterpret_cast<const T*>(A.rho);
    const uint64_t* rw = reinterpret_cast<const uint64_t*>(A.rho);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        unsigned owners = __ballot_sync(FULL, (act4 >> j) & 1u);
        while (owners) {
            const int o = __ffs(owners) - 1;
            owners &= owners - 1u;
            const int a = 4 * o + j;
            const T mva = WIDE ? __shfl_sync(FULL, mv[j], o) : T(0);
            const int eva = WIDE ? __shfl_sync(FULL, ev[j], o) : 0;
            Sum<T> ps;
            int ppc = 0;
            for (long long jb = r0 + 32LL * sub; jb < r1; jb += 32LL * nsub) {
                const long long jj = jb + t;
                if (jj < r1) {
                    const int x = A.col[jj];
                    const LT Lx = lv[((size_t)x << 7) + a];
                    if (Lx == dnext) {
                        const size_t xi = ((gbase + (size_t)x) << 7) + a;
                        ps.add(WIDE ? wterm<T>(mva, eva, rw[xi]) : rho[xi]);
                    } else if (Lx == dprev) {
                        ppc++;
                    }
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const T s2 = __shfl_xor_sync(FULL, ps.s, off), c2 = __shfl_xor_sync(FULL, ps.c, off);
                ps.merge(s2, c2);
                if (refsem) ppc += __shfl_xor_sync(FULL, ppc, off);
            }
            if (t == o) {
                acc[j].merge(ps.s, ps.c);
                pc[j] += ppc;
            }
        }
    }
}

// delta, rho and BC contributions of thread t's active lanes of (v, g),
// summed per 32-lane quarter of the group (threads 8q..8q+7 hold lanes
// 32q..32q+31) into bcg row 4g+q: BC partials are kept per 32 lanes for every
// group width, so a lane batch can carry a different request in each quarter.
template <bool WIDE, typename T, int SB>
__device__ __forceinline__ void q_bwd_finish(const KArgs& A, int g, size_t gbase, int v, unsigned act4, const T (&mv)[4],
                                             const int (&ev)[4], const Sum<T> (&acc)[4], const int (&pc)[4], bool refsem) {
    const int t = threadIdx.x & 31;
    double contrib = 0.0;
    const size_t vb = ((gbase + (size_t)v) << 7) + 4 * t;
    const T tw = A.w ? (T)A.w[v] : T(1);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        if (!((act4 >> j) & 1u)) continue;
        T delta;
        if (WIDE) {
            delta = acc[j].value();
            bool of = false;
            reinterpret_cast<uint64_t*>(A.rho)[vb + j] = wpack((T)((tw + delta) / mv[j]), -ev[j], of);
        } else {
            const T sv = (T)reinterpret_cast<const typename SigW<SB>::type*>(A.sig)[vb + j];
            delta = sv * acc[j].value();
            reinterpret_cast<T*>(A.rho)[vb + j] = (tw + delta) / sv;
        }
        contrib += (double)delta * (double)A.srcw[(g << 7) + 4 * t + j] * (refsem ? (double)pc[j] : 1.0);
    }
#pragma unroll
    for (int off = 4; off > 0; off >>= 1) contrib += __shfl_xor_sync(FULL, contrib, off);
    // one writer per (v, quarter) and level: a fire-and-forget add
    if ((t & 7) == 0) atomicAdd(&A.bcg[4 * gbase + (size_t)(t >> 3) * (size_t)A.n + v], contrib);
}

template <bool WIDE, typename T>
__device__ __forceinline__ void q_sigma_of(const KArgs& A, size_t gbase, int v, unsigned act4, T (&mv)[4], int (&ev)[4]) {
    const int t = threadIdx.x & 31;
#pragma unroll
    for (int j = 0; j < 4; j++) { mv[j] = T(0); ev[j] = 0; }
    if (!WIDE || !act4) return;
    const uint64_t* sv = A.sig + ((gbase + (size_t)v) << 7) + 4 * t;
#pragma unroll
    for (int j = 0; j < 4; j++)
        if ((act4 >> j) & 1u) { mv[j] = wmant<T>(sv[j]); ev[j] = wexp(sv[j]); }
}

// Dependency-sweep level kernel, 128-lane groups.
template <bool WIDE, typename T, typename LT, int NT, int SB>
__global__ void __launch_bounds__(NT, 4 * 256 / NT) backward_q_kernel(KArgs A) {
    constexpr int WARPS = NT / 32;
    __shared__ T h_s[WARPS][128];
    __shared__ T h_c[WARPS][128];
    __shared__ int h_pc[WARPS][128];
    __shared__ unsigned long long s_i;
    const int d = *(volatile int*)&A.ctl->level;
    const int t = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const bool refsem = (A.semantics == GBC_BC_REFERENCE);
    if (d >= 1) {
        const unsigned long long he = A.hoff[d + 1];
        for (;;) {
            if (threadIdx.x == 0) s_i = atomicAdd(&A.ctl->hnext, 1ULL);
            __syncthreads();
            const unsigned long long i = s_i;
            __syncthreads();
            if (i >= he) break;
            const uint32_t ent = A.hq[i];
            const int v = (int)(ent >> 5), g = (int)(ent & 31u);
            const size_t gbase = (size_t)g * (size_t)A.n;
            const LT* lv = reinterpret_cast<const LT*>(A.lvl) + (gbase << 7);
            const unsigned act4 = Quad<LT>::load(lv + ((size_t)v << 7), t).eq(d);
            const int nact = __reduce_add_sync(FULL, __popc(act4));
            if (nact == 0) continue;
            T mv[4];
            int ev[4];
            q_sigma_of<WIDE, T>(A, gbase, v, act4, mv, ev);
            Sum<T> acc[4];
            int pc[4] = {0, 0, 0, 0};
            if (nact > A.sparse) q_bwd_scan<WIDE, T, LT>(A, d, gbase, lv, act4, mv, ev, A.row[v], A.row[v + 1], wib, WARPS,
                                                     q_col(A, A.row[v] + 32LL * wib, A.row[v + 1]), acc, pc);
            else q_bwd_edges<WIDE, T, LT>(A, d, gbase, lv, act4, mv, ev, A.row[v], A.row[v + 1], wib, WARPS, acc, pc);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                h_s[wib][4 * t + j] = acc[j].s;
                h_c[wib][4 * t + j] = acc[j].c;
                h_pc[wib][4 * t + j] = pc[j];
            }
            __syncthreads();
            if (wib == 0) {
                for (int w = 1; w < WARPS; w++) {
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        acc[j].merge(h_s[w][4 * t + j], h_c[w][4 * t + j]);
                        pc[j] += h_pc[w][4 * t + j];
                    }
                }
                q_bwd_finish<WIDE, T, SB>(A, g, gbase, v, act4, mv, ev, acc, pc, refsem);
            }
            __syncthreads();
        }
        const unsigned long long e = A.foff[d + 1];
        for (;;) {
            int take;
            const unsigned long long base = q_fetch(A, e, take);
            if (base >= e) break;
            const unsigned long long my = base + t;
            const bool mine = t < take && my < e;
            const uint32_t ment = mine ? A.fq[my] : 0u;
            const long long m0 = mine ? A.row[ment >> 5] : 0, m1 = mine ? A.row[(ment >> 5) + 1] : 0;
            const int cntE = (int)min((unsigned long long)take, e - base);
            for (int k = 0; k < cntE; k++) {
                const uint32_t ent = __shfl_sync(FULL, ment, k);
                const long long r0 = __shfl_sync(FULL, m0, k), r1 = __shfl_sync(FULL, m1, k);
                const int v = (int)(ent >> 5), g = (int)(ent & 31u);
                const size_t gbase = (size_t)g * (size_t)A.n;
                const LT* lv = reinterpret_cast<const LT*>(A.lvl) + (gbase << 7);
                const unsigned act4 = Quad<LT>::load(lv + ((size_t)v << 7), t).eq(d);
                const int xm0 = q_col(A, r0, r1);   // the first chunk's columns, loaded with the level row
                const int nact = __reduce_add_sync(FULL, __popc(act4));
                if (nact == 0) continue;
                T mv[4];
                int ev[4];
                q_sigma_of<WIDE, T>(A, gbase, v, act4, mv, ev);
                Sum<T> acc[4];
                int pc[4] = {0, 0, 0, 0};
                if (nact > A.sparse) q_bwd_scan<WIDE, T, LT>(A, d, gbase, lv, act4, mv, ev, r0, r1, 0, 1, xm0, acc, pc);
                else q_bwd_edges<WIDE, T, LT>(A, d, gbase, lv, act4, mv, ev, r0, r1, 0, 1, acc, pc);
                q_bwd_finish<WIDE, T, SB>(A, g, gbase, v, act4, mv, ev, acc, pc, refsem);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&A.ctl->blocks, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            A.ctl->blocks = 0;
            if (d >= 1) {
                A.ctl->level = d - 1;
                A.ctl->next = A.foff[d - 1];
                A.ctl->hnext = A.hoff[d - 1];
            }
        }
    }
}


// ---- one lane per task (group width 1) ---------------------------------------
// Deep graphs whose sampled sources lie far apart (grids, meshes, roads) give a
// lane group about one active lane per task, so per-group tasks read a whole
// level row to find it.  With group width 1 the lane state is lane-major
// (level / path count / rho [lane][v]), a frontier entry is one (vertex, lane)
// pair packed v << 10 | lane (n < 2^22), and discovery is a 16-bit
// compare-and-swap on the neighbour's level, so each (vertex, lane) enters the
// queue exactly once per batch and no claim array is needed.  Neighbours that
// are close in id (v +- 1 on a grid) share the cache line of v's own entry.
// The sweep writes each lane's BC contribution into the lane's path-count slot,
// which nothing reads after it; lane_bc_reduce_kernel then sums the slots over
// lanes in lane order, so results stay deterministic.
constexpr int S_LANE_BITS = 10;
constexpr uint16_t S_INF = 0xFFFFu;

template <int MODE, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) expand_s_kernel(KArgs A) {
    constexpr int WARPS = NT / 32;
    constexpr int U = LIGHT_U;
    __shared__ unsigned long long cc_sh[MODE == 0 ? 1024 : 1];
    __shared__ uint32_t stg[WARPS][STG];
    if (MODE == 0) {
        for (int i = threadIdx.x; i < A.ng; i += blockDim.x) cc_sh[i] = 0ULL;
        __syncthreads();
    }
    const int done = *(volatile int*)&A.ctl->done;
    const int d = *(volatile int*)&A.ctl->level;
    const int t = threadIdx.x & 31, wib = threadIdx.x >> 5;
    Stage S{stg[wib], 0};
    unsigned long long vis = 0;
    if (!done) {
        const uint16_t dprev = (uint16_t)(d - 1), dnext = (uint16_t)(d + 1), dl = (uint16_t)d;
        uint16_t* lv = reinterpret_cast<uint16_t*>(A.lvl);
        const unsigned long long e = A.foff[d + 1];
        bool first = true;
        for (;;) {
            const unsigned long long base = warp_fetch(A, d, first);
            if (base >= e) break;
            const bool act = base + t < e;
            const uint32_t ent = act ? A.fq[base + t] : 0u;
            const int v = (int)(ent >> S_LANE_BITS), a = (int)(ent & ((1u << S_LANE_BITS) - 1u));
            // neighbours from the padded table (no row-offset round trip) or from the CSR
            const long long r0 = (act && !A.ell_q) ? A.row[v] : 0, r1 = (act && !A.ell_q) ? A.row[v + 1] : 0;
            const size_t la = (size_t)a * (size_t)A.n;
            if (act) vis += (unsigned long long)(r1 - r0);
            if (MODE == 0 && act) {
                const long long c = (A.w ? (long long)d * (long long)A.w[v] : (long long)d) + (A.ff ? A.ff[v] : 0LL);
                atomicAdd(&cc_sh[a], (unsigned long long)c);
            }
            const int maxs = A.ell_q ? A.ell_q : __reduce_max_sync(FULL, (int)((r1 - r0 + U - 1) / U));
            long long j = r0;
            uint64_t acc = 0;
            bool of = false;
            int we = WEMPTY;
            double ws = 0.0;
            for (int it = 0; it < maxs; it++) {
                int x[U];
                uint16_t L[U];
                if (A.ell_q) {
                    const int4 nb = act ? A.ell[(size_t)v * A.ell_q + it] : make_int4(-1, -1, -1, -1);
                    x[0] = nb.x; x[1] = nb.y; x[2] = nb.z; x[3] = nb.w;
#pragma unroll
                    for (int u = 0; u < U; u++) vis += x[u] >= 0;
                } else {
#pragma unroll
                    for (int u = 0; u < U; u++) x[u] = (j + u < r1) ? A.col[j + u] : -1;
                }
#pragma unroll
                for (int u = 0; u < U; u++) L[u] = x[u] >= 0 ? lv[la + (size_t)x[u]] : dl;   // dl: neither case below
                // path-count loads, then the discovery compare-and-swaps, then the sums:
                // the swaps' round trip overlaps the loads' instead of following it
                uint64_t sv[U];
#pragma unroll
                for (int u = 0; u < U; u++)
                    sv[u] = (MODE != 0 && d > 0 && L[u] == dprev) ? A.sig[la + (size_t)x[u]] : 0ULL;
                bool has[U];
#pragma unroll
                for (int u = 0; u < U; u++)
                    has[u] = L[u] == S_INF && atomicCAS(lv + la + (size_t)x[u], S_INF, dnext) == S_INF;
                if (MODE != 0 && d > 0) {
#pragma unroll
                    for (int u = 0; u < U; u++) {
                        if (L[u] != dprev) continue;
                        if (MODE == 1) {
                            const uint64_t na = acc + sv[u];
                            of |= (na < acc);
                            acc = na;
                        } else {
                            wadd(ws, we, sv[u]);
                        }
                    }
                }
                j = min(j + U, r1);
#pragma unroll
                for (int u = 0; u < U; u++)
                    warp_append(A, S, has[u], false, ((uint32_t)x[u] << S_LANE_BITS) | (uint32_t)a);
            }
            if (act && MODE != 0 && d > 0) {
                if (MODE == 2) acc = wpack(ws, we, of);
                A.sig[la + (size_t)v] = acc;
                if (of) {
                    atomicOr(&A.ovf[a >> 5], 1u << (a & 31));
                    A.ctl->any_ovf = 1;
                }
            }
        }
    }
    stage_flush(A, S);
    add_visits(A, vis);
    if (MODE == 0) {
        __syncthreads();
        for (int i = threadIdx.x; i < A.ng; i += blockDim.x)
            if (cc_sh[i]) atomicAdd(&A.cc[i], cc_sh[i]);
    }
    fwd_last_block(A, d, done, Lv<uint16_t>::MAXD);
}

template <bool WIDE, typename T, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) backward_s_kernel(KArgs A) {
    constexpr int U = LIGHT_U;
    const int d = *(volatile int*)&A.ctl->level;
    const int t = threadIdx.x & 31;
    const bool refsem = (A.semantics == GBC_BC_REFERENCE);
    if (d >= 1) {
        const uint16_t dprev = (uint16_t)(d - 1), dnext = (uint16_t)(d + 1), dl = (uint16_t)d;
        const uint16_t* lv = reinterpret_cast<const uint16_t*>(A.lvl);
        const uint64_t* rw = reinterpret_cast<const uint64_t*>(A.rho);
        const unsigned long long e = A.foff[d + 1];
        bool first = true;
        for (;;) {
            const unsigned long long base = warp_fetch(A, d, first);
            if (base >= e) break;
            if (base + t < e) {   // the last fetch of a level may leave threads without an entry
                const uint32_t ent = A.fq[base + t];
                const int v = (int)(ent >> S_LANE_BITS), a = (int)(ent & ((1u << S_LANE_BITS) - 1u));
                // neighbours from the padded table (no row-offset round trip) or from the CSR
                const long long r0 = A.ell_q ? 0 : A.row[v], r1 = A.ell_q ? (long long)U * A.ell_q : A.row[v + 1];
                const size_t la = (size_t)a * (size_t)A.n, vi = la + (size_t)v;
                const uint64_t sw = A.sig[vi];
                T mv = T(0);
                int ev = 0;
                if (WIDE) { mv = wmant<T>(sw); ev = wexp(sw); }
                Sum<T> acc;
                int pc = 0;
                for (long long j = r0; j < r1; j += U) {
                    int x[U];
                    uint16_t L[U];
                    if (A.ell_q) {
                        const int4 nb = A.ell[(size_t)v * A.ell_q + (int)(j / U)];
                        x[0] = nb.x; x[1] = nb.y; x[2] = nb.z; x[3] = nb.w;
                    } else {
#pragma unroll
                        for (int u = 0; u < U; u++) x[u] = j + u < r1 ? A.col[j + u] : -1;
                    }
#pragma unroll
                    for (int u = 0; u < U; u++) L[u] = x[u] >= 0 ? lv[la + (size_t)x[u]] : dl;
                    uint64_t rv[U];
#pragma unroll
                    for (int u = 0; u < U; u++) {
                        rv[u] = 0;
                        if (L[u] == dnext) {
                            if (WIDE || sizeof(T) == 8) rv[u] = rw[la + (size_t)x[u]];
                            else rv[u] = __float_as_uint(reinterpret_cast<const float*>(A.rho)[la + (size_t)x[u]]);
                        }
                    }
#pragma unroll
                    for (int u = 0; u < U; u++) {
                        if (L[u] == dnext) {
                            if (WIDE) acc.add(wterm<T>(mv, ev, rv[u]));
                            else if (sizeof(T) == 8) acc.add((T)__longlong_as_double((long long)rv[u]));
                            else acc.add((T)__uint_as_float((unsigned)rv[u]));
                        } else if (L[u] == dprev) {
                            pc++;
                        }
                    }
                }
                const T tw = A.w ? (T)A.w[v] : T(1);
                T delta;
                if (WIDE) {
                    delta = acc.value();
                    bool of = false;
                    reinterpret_cast<uint64_t*>(A.rho)[vi] = wpack((T)((tw + delta) / mv), -ev, of);
                } else {
                    const T sv = (T)sw;
                    delta = sv * acc.value();
                    reinterpret_cast<T*>(A.rho)[vi] = (tw + delta) / sv;
                }
                // the lane's contribution replaces its path count, which nothing reads after this
                const double contrib = (double)delta * (double)A.srcw[a] * (refsem ? (double)pc : 1.0);
                A.sig[vi] = (uint64_t)__double_as_longlong(contrib);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&A.ctl->blocks, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            A.ctl->blocks = 0;
            if (d >= 1) {
                A.ctl->level = d - 1;
                A.ctl->next = A.foff[d - 1];
                A.ctl->hnext = A.hoff[d - 1];
            }
        }
    }
}


// 128-lane entry points of one level width; path-count widths 4 and 2 bytes
// exist for the exact forward and the non-wide sweeps only.
template <typename LT, int NT>
void fill_q(LevelKernels& K, int lv) {
    for (int m = 0; m < 3; m++)
        for (int w = 0; w < 3; w++) K.expand_q[lv][m][w] = nullptr;
    K.expand_q[lv][0][0] = expand_q_kernel<0, LT, NT, 8>;
    K.expand_q[lv][1][0] = expand_q_kernel<1, LT, NT, 8>;
    K.expand_q[lv][1][1] = expand_q_kernel<1, LT, NT, 4>;
    K.expand_q[lv][1][2] = expand_q_kernel<1, LT, NT, 2>;
    K.expand_q[lv][2][0] = expand_q_kernel<2, LT, NT, 8>;
    for (int v = 0; v < 4; v++)
        for (int w = 0; w < 3; w++) K.backward_q[lv][v][w] = nullptr;
    K.backward_q[lv][0][0] = backward_q_kernel<false, float, LT, NT, 8>;
    K.backward_q[lv][0][1] = backward_q_kernel<false, float, LT, NT, 4>;
    K.backward_q[lv][0][2] = backward_q_kernel<false, float, LT, NT, 2>;
    K.backward_q[lv][1][0] = backward_q_kernel<false, double, LT, NT, 8>;
    K.backward_q[lv][1][1] = backward_q_kernel<false, double, LT, NT, 4>;
    K.backward_q[lv][1][2] = backward_q_kernel<false, double, LT, NT, 2>;
    K.backward_q[lv][2][0] = backward_q_kernel<true, float, LT, NT, 8>;
    K.backward_q[lv][3][0] = backward_q_kernel<true, double, LT, NT, 8>;
}

// Entry points of every level kernel for NT-thread CTAs.
template <int NT>
void fill_level_kernels(LevelKernels& K) {
    K.expand_s[0] = expand_s_kernel<0, NT>;
    K.expand_s[1] = expand_s_kernel<1, NT>;
    K.expand_s[2] = expand_s_kernel<2, NT>;
    K.backward_s[0] = backward_s_kernel<false, float, NT>;
    K.backward_s[1] = backward_s_kernel<false, double, NT>;
    K.backward_s[2] = backward_s_kernel<true, float, NT>;
    K.backward_s[3] = backward_s_kernel<true, double, NT>;
    K.expand[0][0] = expand_kernel<0, uint8_t, NT>;
    K.expand[0][1] = expand_kernel<1, uint8_t, NT>;
    K.expand[0][2] = expand_kernel<2, uint8_t, NT>;
    K.expand[1][0] = expand_kernel<0, uint16_t, NT>;
    K.expand[1][1] = expand_kernel<1, uint16_t, NT>;
    K.expand[1][2] = expand_kernel<2, uint16_t, NT>;
    K.backward[0][0] = backward_kernel<false, float, uint8_t, NT>;
    K.backward[0][1] = backward_kernel<false, double, uint8_t, NT>;
    K.backward[0][2] = backward_kernel<true, float, uint8_t, NT>;
    K.backward[0][3] = backward_kernel<true, double, uint8_t, NT>;
    K.backward[1][0] = backward_kernel<false, float, uint16_t, NT>;
    K.backward[1][1] = backward_kernel<false, double, uint16_t, NT>;
    K.backward[1][2] = backward_kernel<true, float, uint16_t, NT>;
    K.backward[1][3] = backward_kernel<true, double, uint16_t, NT>;
    fill_q<uint8_t, NT>(K, 0);
    fill_q<uint16_t, NT>(K, 1);
}

}  // namespace

}  // namespace gbc
