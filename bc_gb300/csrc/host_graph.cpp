// Host-side graph utilities of libgbc: error state, RNG, CSR construction,
// components, the edge-list reader and the synthetic generators.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <thread>

#include "gbc_internal.h"

namespace gbc {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}
const char* last_error() { return g_err; }

// ---------------------------------------------------------------- RNG ----
static inline uint64_t splitmix64(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

Rng::Rng(uint64_t seed, uint64_t stream) {
    uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull);
    for (int i = 0; i < 4; i++) s[i] = splitmix64(x);
}
uint64_t Rng::next() {  // xoshiro256**
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
}
double Rng::uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
uint64_t Rng::below(uint64_t bound) {  // Lemire's nearly-divisionless method
    if (bound == 0) return 0;
    __uint128_t m = (__uint128_t)next() * bound;
    uint64_t l = (uint64_t)m;
    if (l < bound) {
        uint64_t t = (0 - bound) % bound;
        while (l < t) { m = (__uint128_t)next() * bound; l = (uint64_t)m; }
    }
    return (uint64_t)(m >> 64);
}

static int n_threads() {
    unsigned h = std::thread::hardware_concurrency();
    return h == 0 ? 4 : (int)std::min(h, 64u);
}

template <class F>
static void parallel_for(int64_t n, F f) {
    int T = n_threads();
    if (n < 65536) T = 1;
    std::vector<std::thread> th;
    for (int t = 0; t < T; t++) {
        int64_t a = n * t / T, b = n * (t + 1) / T;
        if (T == 1) { f(a, b); break; }
        th.emplace_back([=] { f(a, b); });
    }
    for (auto& x : th) x.join();
}

// --------------------------------------------------------- CSR build ----
// First index in [0, count) where bad(i) holds, or count; chunks are scanned
// in parallel and the smallest hit wins, so the answer does not depend on the
// thread count.
template <class F>
static int64_t first_bad(int64_t count, F bad) {
    std::atomic<int64_t> best(count);
    parallel_for(count, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++) {
            if (i >= best.load(std::memory_order_relaxed)) return;
            if (bad(i)) {
                int64_t cur = best.load(std::memory_order_relaxed);
                while (i < cur && !best.compare_exchange_weak(cur, i, std::memory_order_relaxed)) {
                }
                return;
            }
        }
    });
    return best.load();
}

gbc_status validate_csr_header(const int64_t* row, const int32_t* col, int32_t n) {
    if (n <= 0 || !row || (row[n] > 0 && !col)) { set_error("invalid CSR arguments (n=%d)", n); return GBC_ERR_ARG; }
    if (row[0] != 0) { set_error("row[0] must be 0"); return GBC_ERR_ARG; }
    if (row[n] < 0 || row[n] >= ((int64_t)1 << 31)) return validate_csr(row, col, n);
    return GBC_OK;
}

gbc_status validate_csr(const int64_t* row, const int32_t* col, int32_t n) {
    if (n <= 0 || !row || (row[n] > 0 && !col)) { set_error("invalid CSR arguments (n=%d)", n); return GBC_ERR_ARG; }
    if (row[0] != 0) { set_error("row[0] must be 0"); return GBC_ERR_ARG; }
    const int64_t dv = first_bad(n, [&](int64_t v) { return row[v + 1] < row[v]; });
    if (dv < n) { set_error("row offsets decrease at %lld", (long long)dv); return GBC_ERR_ARG; }
    int64_t m = row[n];
    if (m >= ((int64_t)1 << 31)) { set_error("more than 2^31-1 directed edges (%lld)", (long long)m); return GBC_ERR_ARG; }
    const int64_t be = first_bad(m, [&](int64_t e) { return (uint32_t)col[e] >= (uint32_t)n; });
    if (be < m) { set_error("col[%lld]=%d out of range", (long long)be, col[be]); return GBC_ERR_ARG; }
    return GBC_OK;
}

void csr_from_edges(int32_t n, const std::vector<int32_t>& u, const std::vector<int32_t>& v, HostCSR& out) {
    const int64_t E = (int64_t)u.size();
    std::vector<std::atomic<int64_t>> deg(n);
    for (int32_t i = 0; i < n; i++) deg[i].store(0, std::memory_order_relaxed);
    parallel_for(E, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++)
            if (u[i] != v[i]) {
                deg[u[i]].fetch_add(1, std::memory_order_relaxed);
                deg[v[i]].fetch_add(1, std::memory_order_relaxed);
            }
    });
    std::vector<int64_t> row(n + 1);
    row[0] = 0;
    for (int32_t i = 0; i < n; i++) row[i + 1] = row[i] + deg[i].load(std::memory_order_relaxed);
    std::vector<int32_t> col(row[n]);
    std::vector<std::atomic<int64_t>> fill(n);
    for (int32_t i = 0; i < n; i++) fill[i].store(row[i], std::memory_order_relaxed);
    parallel_for(E, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++)
            if (u[i] != v[i]) {
                col[fill[u[i]].fetch_add(1, std::memory_order_relaxed)] = v[i];
                col[fill[v[i]].fetch_add(1, std::memory_order_relaxed)] = u[i];
            }
    });
    // sort + unique each row
    std::vector<int64_t> newdeg(n);
    parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t x = a; x < b; x++) {
            int32_t* p = col.data() + row[x];
            int32_t* q = col.data() + row[x + 1];
            std::sort(p, q);
            newdeg[x] = std::unique(p, q) - p;
        }
    });
    out.n = n;
    out.row.assign(n + 1, 0);
    for (int32_t i = 0; i < n; i++) out.row[i + 1] = out.row[i] + newdeg[i];
    out.col.resize(out.row[n]);
    parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t x = a; x < b; x++)
            std::memcpy(out.col.data() + out.row[x], col.data() + row[x], sizeof(int32_t) * newdeg[x]);
    });
}

int32_t components(const HostCSR& g, std::vector<int32_t>& comp, std::vector<int64_t>& sizes) {
    comp.assign(g.n, -1);
    sizes.clear();
    std::vector<int32_t> q(g.n);
    int32_t nc = 0;
    for (int32_t r = 0; r < g.n; r++) {
        if (comp[r] >= 0) continue;
        int64_t head = 0, tail = 0;
        q[tail++] = r;
        comp[r] = nc;
        while (head < tail) {
            int32_t x = q[head++];
            for (int64_t e = g.row[x]; e < g.row[x + 1]; e++) {
                int32_t y = g.col[e];
                if (comp[y] < 0) { comp[y] = nc; q[tail++] = y; }
            }
        }
        sizes.push_back(tail);
        nc++;
    }
    return nc;
}

int64_t edges_of_sources(const HostCSR& g, const std::vector<int32_t>& comp, const std::vector<int64_t>& comp_edges,
                         const int32_t* src, int32_t k) {
    (void)g;
    int64_t s = 0;
    for (int32_t i = 0; i < k; i++) s += comp_edges[comp[src[i]]];
    return s;
}

gbc_status export_csr(const HostCSR& g, int64_t** row, int32_t** col) {
    *row = (int64_t*)malloc(sizeof(int64_t) * (g.n + 1));
    *col = (int32_t*)malloc(sizeof(int32_t) * std::max<int64_t>(g.m(), 1));
    if (!*row || !*col) { free(*row); free(*col); set_error("host allocation failed"); return GBC_ERR_NOMEM; }
    std::memcpy(*row, g.row.data(), sizeof(int64_t) * (g.n + 1));
    if (g.m()) std::memcpy(*col, g.col.data(), sizeof(int32_t) * g.m());
    return GBC_OK;
}

}  // namespace gbc

using namespace gbc;

extern "C" {

const char* gbc_last_error(void) { return gbc::last_error(); }
void gbc_free(void* p) { free(p); }

// Barabasi-Albert preferential attachment: a star on m+1 vertices, then each
// new vertex joins m distinct targets drawn uniformly from the list holding
// every vertex once per unit of degree.
gbc_status gbc_gen_ba(int32_t n, int32_t m, uint64_t seed, int64_t** row, int32_t** col) {
    if (m < 1 || n <= m) { set_error("BA needs 1 <= m < n"); return GBC_ERR_ARG; }
    Rng rng(seed, 1);
    std::vector<int32_t> eu, ev, rep;
    eu.reserve((size_t)n * m);
    ev.reserve((size_t)n * m);
    rep.reserve((size_t)2 * n * m);
    for (int32_t i = 1; i <= m; i++) { eu.push_back(0); ev.push_back(i); rep.push_back(0); rep.push_back(i); }
    std::vector<int32_t> targets(m);
    for (int32_t s = m + 1; s < n; s++) {
        int32_t cnt = 0;
        while (cnt < m) {
            int32_t t = rep[rng.below(rep.size())];
            bool dup = false;
            for (int32_t j = 0; j < cnt; j++) dup |= (targets[j] == t);
            if (!dup) targets[cnt++] = t;
        }
        for (int32_t j = 0; j < m; j++) {
            eu.push_back(s); ev.push_back(targets[j]);
            rep.push_back(targets[j]); rep.push_back(s);
        }
    }
    HostCSR g;
    csr_from_edges(n, eu, ev, g);
    return export_csr(g, row, col);
}

// R-MAT (Chakrabarti et al. 2004): every edge picks one quadrant per level
// with probabilities a, b, c, 1-a-b-c; symmetrised, self-loops and duplicate
// edges dropped; optional seeded vertex relabelling (Graph500 convention).
gbc_status gbc_gen_rmat(int32_t scale, int32_t ef, double a, double b, double c, uint64_t seed, int32_t permute,
                        int64_t** row, int32_t** col, int32_t* n_out) {
    if (scale < 1 || scale > 30 || ef < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) {
        set_error("bad R-MAT parameters"); return GBC_ERR_ARG;
    }
    const int32_t n = (int32_t)1 << scale;
    const int64_t E = (int64_t)ef * n;
    std::vector<int32_t> eu(E), ev(E);
    const int64_t chunk = 1 << 16;
    const int64_t nchunks = (E + chunk - 1) / chunk;
    std::atomic<int64_t> next{0};
    auto work = [&] {
        for (;;) {
            int64_t ci = next.fetch_add(1);
            if (ci >= nchunks) break;
            Rng r(seed, 1000 + (uint64_t)ci);
            int64_t lo = ci * chunk, hi = std::min(E, lo + chunk);
            for (int64_t i = lo; i < hi; i++) {
                uint32_t x = 0, y = 0;
                for (int32_t l = 0; l < scale; l++) {
                    double p = r.uniform();
                    uint32_t bx = 0, by = 0;
                    if (p < a) { }
                    else if (p < a + b) by = 1;
                    else if (p < a + b + c) bx = 1;
                    else { bx = 1; by = 1; }
                    x = (x << 1) | bx;
                    y = (y << 1) | by;
                }
                eu[i] = (int32_t)x;
                ev[i] = (int32_t)y;
            }
        }
    };
    {
        std::vector<std::thread> th;
        for (int t = 0; t < n_threads(); t++) th.emplace_back(work);
        for (auto& t : th) t.join();
    }
    if (permute) {
        std::vector<int32_t> perm(n);
        for (int32_t i = 0; i < n; i++) perm[i] = i;
        Rng pr(seed, 7);
        for (int32_t i = n - 1; i > 0; i--) std::swap(perm[i], perm[pr.below((uint64_t)i + 1)]);
        parallel_for(E, [&](int64_t lo, int64_t hi) {
            for (int64_t i = lo; i < hi; i++) { eu[i] = perm[eu[i]]; ev[i] = perm[ev[i]]; }
        });
    }
    HostCSR g;
    csr_from_edges(n, eu, ev, g);
    *n_out = n;
    return export_csr(g, row, col);
}

// 4-neighbour grid with a uniformly chosen set of round(remove_frac * E)
// edges removed; optionally only the largest component, relabelled in
// row-major order.
gbc_status gbc_gen_grid(int32_t rows, int32_t cols, double remove_frac, uint64_t seed, int32_t largest_only,
                        int64_t** row, int32_t** col, int32_t* n_out) {
    if (rows < 1 || cols < 1 || (int64_t)rows * cols >= ((int64_t)1 << 31) || remove_frac < 0 || remove_frac >= 1) {
        set_error("bad grid parameters"); return GBC_ERR_ARG;
    }
    const int64_t nh = (int64_t)rows * (cols - 1), nv = (int64_t)cols * (rows - 1), E = nh + nv;
    std::vector<uint8_t> removed(E, 0);
    int64_t R = (int64_t)std::llround(remove_frac * (double)E);
    {
        std::vector<int64_t> idx(E);
        for (int64_t i = 0; i < E; i++) idx[i] = i;
        Rng r(seed, 3);
        for (int64_t i = 0; i < R; i++) {
            int64_t j = i + (int64_t)r.below((uint64_t)(E - i));
            std::swap(idx[i], idx[j]);
            removed[idx[i]] = 1;
        }
    }
    const int32_t n = rows * cols;
    std::vector<int32_t> eu, ev;
    eu.reserve(E - R); ev.reserve(E - R);
    for (int64_t i = 0; i < E; i++) {
        if (removed[i]) continue;
        int32_t x, y;
        if (i < nh) { int32_t r = (int32_t)(i / (cols - 1)), cc = (int32_t)(i % (cols - 1)); x = r * cols + cc; y = x + 1; }
        else { int64_t j = i - nh; int32_t r = (int32_t)(j / cols), cc = (int32_t)(j % cols); x = r * cols + cc; y = x + cols; }
        eu.push_back(x); ev.push_back(y);
    }
    HostCSR g;
    csr_from_edges(n, eu, ev, g);
    if (largest_only) {
        std::vector<int32_t> comp;
        std::vector<int64_t> sizes;
        components(g, comp, sizes);
        int32_t best = (int32_t)(std::max_element(sizes.begin(), sizes.end()) - sizes.begin());
        std::vector<int32_t> nid(n, -1);
        int32_t k = 0;
        for (int32_t v = 0; v < n; v++) if (comp[v] == best) nid[v] = k++;
        HostCSR h;
        h.n = k;
        h.row.assign(k + 1, 0);
        for (int32_t v = 0; v < n; v++) if (nid[v] >= 0) h.row[nid[v] + 1] = g.row[v + 1] - g.row[v];
        for (int32_t i = 0; i < k; i++) h.row[i + 1] += h.row[i];
        h.col.resize(h.row[k]);
        for (int32_t v = 0; v < n; v++) {
            if (nid[v] < 0) continue;
            int64_t o = h.row[nid[v]];
            for (int64_t e = g.row[v]; e < g.row[v + 1]; e++) h.col[o++] = nid[g.col[e]];
        }
        *n_out = k;
        return export_csr(h, row, col);
    }
    *n_out = n;
    return export_csr(g, row, col);
}

// Erdos-Renyi G(n, M) with M = round(n * avg_degree / 2) drawn pairs
// (self-loops and repeats dropped).
gbc_status gbc_gen_er(int32_t n, double avg_degree, uint64_t seed, int64_t** row, int32_t** col) {
    if (n < 2 || avg_degree < 0) { set_error("bad ER parameters"); return GBC_ERR_ARG; }
    int64_t M = (int64_t)std::llround((double)n * avg_degree / 2.0);
    std::vector<int32_t> eu(M), ev(M);
    Rng r(seed, 5);
    for (int64_t i = 0; i < M; i++) { eu[i] = (int32_t)r.below(n); ev[i] = (int32_t)r.below(n); }
    HostCSR g;
    csr_from_edges(n, eu, ev, g);
    return export_csr(g, row, col);
}

gbc_status gbc_add_pendants(const int64_t* row, const int32_t* col, int32_t n, int32_t trees, int32_t max_depth,
                            uint64_t seed, int64_t** row_out, int32_t** col_out, int32_t* n_out) {
    gbc_status st = validate_csr(row, col, n);
    if (st != GBC_OK) return st;
    if (trees < 0 || max_depth < 1) { set_error("bad pendant parameters"); return GBC_ERR_ARG; }
    std::vector<int32_t> eu, ev;
    eu.reserve(row[n] / 2 + (int64_t)trees * max_depth);
    ev.reserve(row[n] / 2 + (int64_t)trees * max_depth);
    for (int32_t x = 0; x < n; x++)
        for (int64_t e = row[x]; e < row[x + 1]; e++)
            if (x < col[e]) { eu.push_back(x); ev.push_back(col[e]); }
    Rng r(seed, 11);
    int32_t next = n;
    for (int32_t t = 0; t < trees; t++) {
        int32_t host = (int32_t)r.below(n);
        int32_t depth = 1 + (int32_t)r.below(max_depth);
        int32_t prev = host;
        for (int32_t d = 0; d < depth; d++) { eu.push_back(prev); ev.push_back(next); prev = next++; }
    }
    HostCSR g;
    csr_from_edges(next, eu, ev, g);
    *n_out = next;
    return export_csr(g, row_out, col_out);
}

// Cycles of min_len..max_len vertices (uniform), each through one uniformly
// chosen vertex of the input and len - 1 new vertices: every chosen vertex
// becomes an articulation point and every cycle a block of its own.
gbc_status gbc_add_cycles(const int64_t* row, const int32_t* col, int32_t n, int32_t cycles, int32_t min_len,
                          int32_t max_len, uint64_t seed, int64_t** row_out, int32_t** col_out, int32_t* n_out) {
    gbc_status st = validate_csr(row, col, n);
    if (st != GBC_OK) return st;
    if (cycles < 0 || min_len < 3 || max_len < min_len) { set_error("bad cycle parameters"); return GBC_ERR_ARG; }
    if ((int64_t)n + (int64_t)cycles * (max_len - 1) >= INT32_MAX) { set_error("too many vertices"); return GBC_ERR_ARG; }
    std::vector<int32_t> eu, ev;
    eu.reserve(row[n] / 2 + (int64_t)cycles * max_len);
    ev.reserve(row[n] / 2 + (int64_t)cycles * max_len);
    for (int32_t x = 0; x < n; x++)
        for (int64_t e = row[x]; e < row[x + 1]; e++)
            if (x < col[e]) { eu.push_back(x); ev.push_back(col[e]); }
    Rng r(seed, 13);
    int32_t next = n;
    for (int32_t c = 0; c < cycles; c++) {
        const int32_t host = (int32_t)r.below(n);
        const int32_t len = min_len + (int32_t)r.below(max_len - min_len + 1);
        int32_t prev = host;
        for (int32_t i = 1; i < len; i++) { eu.push_back(prev); ev.push_back(next); prev = next++; }
        eu.push_back(prev);
        ev.push_back(host);
    }
    HostCSR g;
    csr_from_edges(next, eu, ev, g);
    *n_out = next;
    return export_csr(g, row_out, col_out);
}

// "start end" header, then one "%f" line per vertex of values rounded to FP32
// (the reference prints its float BC array this way).
gbc_status gbc_write_scores(const char* path, const double* values, int32_t start, int32_t end, int32_t append) {
    if (!path || !values || start < 0 || end < start - 1) { set_error("bad arguments"); return GBC_ERR_ARG; }
    FILE* f = fopen(path, append ? "a" : "w");
    if (!f) { set_error("cannot open %s", path); return GBC_ERR_ARG; }
    bool ok = fprintf(f, "%d %d\n", start, end) > 0;
    for (int32_t v = start; v <= end && ok; v++) ok = fprintf(f, "%f\n", (double)(float)values[v]) > 0;
    ok = (fclose(f) == 0) && ok;
    if (!ok) { set_error("write to %s failed", path); return GBC_ERR_ARG; }
    return GBC_OK;
}

// Text edge list, as Lib/AdjList/AdjList.c:13-150 reads it: header "n m",
// then m lines "u v"; 0-based when any endpoint is 0, else slot 0 is a
// phantom vertex.  Both directions kept in file order, then each list is
// ordered by neighbour degree ascending (stable).
gbc_status gbc_read_edgelist(const char* path, int64_t** row_out, int32_t** col_out, int32_t* n_out,
                             int32_t* start_out) {
    FILE* f = fopen(path, "r");
    if (!f) { set_error("cannot open %s", path); return GBC_ERR_ARG; }
    char line[4096];
    long n = -1, m = -1;
    if (!fgets(line, sizeof line, f) || sscanf(line, "%ld %ld", &n, &m) != 2 || n <= 0 || m < 0) {
        fclose(f); set_error("bad header in %s", path); return GBC_ERR_ARG;
    }
    std::vector<int32_t> eu, ev;
    eu.reserve(m); ev.reserve(m);
    bool zero = false;
    while ((long)eu.size() < m && fgets(line, sizeof line, f)) {
        long a, b;
        if (sscanf(line, "%ld %ld", &a, &b) != 2) continue;
        eu.push_back((int32_t)a); ev.push_back((int32_t)b);
        zero |= (a == 0 || b == 0);
    }
    fclose(f);
    if ((long)eu.size() != m) { set_error("%s: expected %ld edges, read %zu", path, m, eu.size()); return GBC_ERR_ARG; }
    const int32_t N = zero ? (int32_t)n : (int32_t)(n + 1);
    std::vector<int64_t> deg(N + 1, 0);
    for (long i = 0; i < m; i++) {
        if (eu[i] < 0 || eu[i] >= N || ev[i] < 0 || ev[i] >= N) { set_error("%s: vertex id out of range", path); return GBC_ERR_ARG; }
        deg[eu[i]]++; deg[ev[i]]++;
    }
    HostCSR g;
    g.n = N;
    g.row.assign(N + 1, 0);
    for (int32_t v = 0; v < N; v++) g.row[v + 1] = g.row[v] + deg[v];
    g.col.resize(g.row[N]);
    std::vector<int64_t> fill(g.row.begin(), g.row.end() - 1);
    for (long i = 0; i < m; i++) { g.col[fill[eu[i]]++] = ev[i]; g.col[fill[ev[i]]++] = eu[i]; }
    for (int32_t v = 0; v < N; v++) {
        if (deg[v] <= 1) continue;
        std::stable_sort(g.col.begin() + g.row[v], g.col.begin() + g.row[v + 1],
                         [&](int32_t x, int32_t y) { return deg[x] < deg[y]; });
    }
    *n_out = N;
    *start_out = zero ? 0 : 1;
    return export_csr(g, row_out, col_out);
}

}  // extern "C"
