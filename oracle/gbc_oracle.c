/*
 * gbc_oracle.c -- CPU restatement of the XPPGX/BC centrality path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg.  The product library never links or calls
 * it.  Every routine cites the reference file:line it restates; arithmetic is
 * widened (uint64 sigma with overflow flags, FP64 delta/BC, int64 sums).
 */
#define _GNU_SOURCE
#include "gbc_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void orc_free(void* p) { free(p); }

/* ------------------------------------------------------------------------ */
/* Edge-list reader: header "n m", then m lines "u v" parsed with strtok/atoi
 * (Lib/FileReader/FileReader.c:9-20, Lib/AdjList/AdjList.c:13-96).  The graph
 * is 0-based when any endpoint is 0 (AdjList.c:39,84); otherwise slot 0 is a
 * phantom vertex.  Both directions of every edge are kept, in file order,
 * then each list is ordered by neighbour degree ascending (AdjList.c:98-131;
 * the reference's quicksort is not stable, ties here keep file order).       */
int orc_load_edgelist(const char* path, int32_t* N_out, int64_t* M_out,
                      int32_t* start_out, int64_t** row_out, int32_t** col_out) {
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    char line[4096];
    if (!fgets(line, sizeof line, f)) { fclose(f); return -2; }
    char* tok = strtok(line, " \t\r\n");
    if (!tok) { fclose(f); return -2; }
    long n = atol(tok);
    tok = strtok(NULL, " \t\r\n");
    if (!tok) { fclose(f); return -2; }
    long m = atol(tok);
    if (n <= 0 || m < 0) { fclose(f); return -2; }
    int32_t* eu = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m ? m : 1));
    int32_t* ev = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m ? m : 1));
    int zero_based = 0;
    long got = 0;
    while (got < m && fgets(line, sizeof line, f)) {
        char* a = strtok(line, " \t\r\n");
        if (!a) continue;
        char* b = strtok(NULL, " \t\r\n");
        if (!b) continue;
        eu[got] = atoi(a);
        ev[got] = atoi(b);
        if (eu[got] == 0 || ev[got] == 0) zero_based = 1;
        got++;
    }
    fclose(f);
    if (got != m) { free(eu); free(ev); return -3; }
    int32_t N = zero_based ? (int32_t)n : (int32_t)(n + 1);
    for (long i = 0; i < m; i++)
        if (eu[i] < 0 || eu[i] >= N || ev[i] < 0 || ev[i] >= N) { free(eu); free(ev); return -4; }
    int64_t* deg = (int64_t*)calloc((size_t)N + 1, sizeof(int64_t));
    for (long i = 0; i < m; i++) { deg[eu[i]]++; deg[ev[i]]++; }
    int64_t* row = (int64_t*)malloc(sizeof(int64_t) * ((size_t)N + 1));
    row[0] = 0;
    for (int32_t v = 0; v < N; v++) row[v + 1] = row[v] + deg[v];
    int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * m ? 2 * m : 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * ((size_t)N + 1));
    memcpy(fill, row, sizeof(int64_t) * ((size_t)N + 1));
    for (long i = 0; i < m; i++) {
        col[fill[eu[i]]++] = ev[i];
        col[fill[ev[i]]++] = eu[i];
    }
    /* stable insertion/merge order by degree: per list, a simple stable sort */
    int32_t* tmp = NULL;
    size_t tmpcap = 0;
    for (int32_t v = 0; v < N; v++) {
        int64_t a = row[v], b = row[v + 1], len = b - a;
        if (len <= 1 || deg[v] == 1) continue;
        if ((size_t)len > tmpcap) { tmpcap = (size_t)len; tmp = (int32_t*)realloc(tmp, sizeof(int32_t) * tmpcap); }
        /* bottom-up merge sort keyed by deg[] (stable) */
        int32_t* src = col + a;
        int32_t* dst = tmp;
        for (int64_t width = 1; width < len; width *= 2) {
            for (int64_t i = 0; i < len; i += 2 * width) {
                int64_t lo = i, mid = i + width < len ? i + width : len;
                int64_t hi = i + 2 * width < len ? i + 2 * width : len;
                int64_t p = lo, q = mid, o = lo;
                while (p < mid && q < hi) dst[o++] = (deg[src[q]] < deg[src[p]]) ? src[q++] : src[p++];
                while (p < mid) dst[o++] = src[p++];
                while (q < hi) dst[o++] = src[q++];
            }
            int32_t* t = src; src = dst; dst = t;
        }
        if (src != col + a) memcpy(col + a, src, sizeof(int32_t) * (size_t)len);
    }
    free(tmp);
    free(fill);
    free(deg);
    free(eu);
    free(ev);
    *N_out = N;
    *M_out = 2 * (int64_t)m;
    *start_out = zero_based ? 0 : 1;
    *row_out = row;
    *col_out = col;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Forward BFS with exact path counts (Seq_Brandes/Brandes.c:274-298).
 * sigma[w] accumulates sigma[v] over every DAG edge v->w; a sum that leaves
 * uint64 sets the sticky flag of w (and of everything downstream of it).   */
int orc_sssp(int32_t N, const int64_t* row, const int32_t* col, int32_t s,
             int32_t* dist, uint64_t* sigma, uint8_t* ovf, int32_t* npred) {
    if (s < 0 || s >= N) return -1;
    int32_t* q = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    for (int32_t v = 0; v < N; v++) { dist[v] = -1; sigma[v] = 0; ovf[v] = 0; if (npred) npred[v] = 0; }
    int64_t head = 0, tail = 0;
    q[tail++] = s;
    dist[s] = 0;
    sigma[s] = 1;
    while (head < tail) {
        int32_t v = q[head++];
        for (int64_t e = row[v]; e < row[v + 1]; e++) {
            int32_t w = col[e];
            if (dist[w] < 0) { dist[w] = dist[v] + 1; q[tail++] = w; }
            if (dist[w] == dist[v] + 1) {
                uint64_t r;
                if (__builtin_add_overflow(sigma[w], sigma[v], &r) || ovf[v]) ovf[w] = 1;
                sigma[w] = r;
                if (npred) npred[w]++;
            }
        }
    }
    free(q);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Brandes BC for a range of sources (Seq_Brandes/Brandes.c:249-327). */
typedef struct {
    int32_t N;
    const int64_t* row;
    const int32_t* col;
    const int32_t* src;
    int32_t k0, k1;
    int semantics, scaled;
    double* bc;
    int64_t n_ovf;
} bc_job;

static void* bc_worker(void* arg) {
    bc_job* J = (bc_job*)arg;
    int32_t N = J->N;
    const int64_t* row = J->row;
    const int32_t* col = J->col;
    int32_t* dist = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t* q = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t* npred = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    uint64_t* sig = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)N);
    uint8_t* ovf = (uint8_t*)malloc((size_t)N);
    double* sigf = (double*)malloc(sizeof(double) * (size_t)N); /* scaled counts */
    double* delta = (double*)malloc(sizeof(double) * (size_t)N);
    int* shift = (int*)malloc(sizeof(int) * ((size_t)N + 2));
    for (int32_t v = 0; v < N; v++) dist[v] = -1;
    for (int32_t i = J->k0; i < J->k1; i++) {
        int32_t s = J->src[i];
        int64_t head = 0, tail = 0;
        q[tail++] = s;
        dist[s] = 0;
        sig[s] = 1; ovf[s] = 0; sigf[s] = 1.0; npred[s] = 0;
        shift[0] = 0;
        /* level-synchronous forward: the queue holds levels contiguously */
        int32_t level = 0;
        int64_t lvl_begin = 0;
        while (lvl_begin < tail) {
            int64_t lvl_end = tail;
            for (int64_t h = lvl_begin; h < lvl_end; h++) {
                int32_t v = q[h];
                for (int64_t e = row[v]; e < row[v + 1]; e++) {
                    int32_t w = col[e];
                    if (dist[w] < 0) {
                        dist[w] = level + 1; q[tail++] = w;
                        sig[w] = 0; ovf[w] = 0; sigf[w] = 0.0; npred[w] = 0;
                    }
                    if (dist[w] == level + 1) {
                        uint64_t r;
                        if (__builtin_add_overflow(sig[w], sig[v], &r) || ovf[v]) ovf[w] = 1;
                        sig[w] = r;
                        sigf[w] += sigf[v];
                        npred[w]++;
                    }
                }
            }
            /* normalise the new level's scaled counts by a power of two */
            if (J->scaled && tail > lvl_end) {
                double mx = 0.0;
                for (int64_t h = lvl_end; h < tail; h++) if (sigf[q[h]] > mx) mx = sigf[q[h]];
                int e2 = 0;
                frexp(mx, &e2);
                shift[level + 1] = e2;
                for (int64_t h = lvl_end; h < tail; h++) sigf[q[h]] = ldexp(sigf[q[h]], -e2);
            }
            lvl_begin = lvl_end;
            level++;
        }
        /* backward sweep (Brandes.c:317-327), deepest vertices first */
        for (int64_t h = tail - 1; h >= 0; h--) delta[q[h]] = 0.0;
        for (int64_t h = tail - 1; h >= 0; h--) {
            int32_t v = q[h];
            if (ovf[v]) J->n_ovf++;
            if (v == s) continue;
            /* pull formulation: delta(v) = sum over successors w of
             * sigma(v)/sigma(w) * (1 + delta(w)) -- identical sums to the
             * reference's push over predecessor lists. */
            double acc = 0.0;
            for (int64_t e = row[v]; e < row[v + 1]; e++) {
                int32_t w = col[e];
                if (dist[w] == dist[v] + 1) {
                    if (J->scaled) acc += (1.0 + delta[w]) / sigf[w];
                    else acc += (1.0 + delta[w]) / (double)sig[w];
                }
            }
            double dv;
            if (J->scaled) dv = sigf[v] * ldexp(acc, -shift[dist[v] + 1]);
            else dv = (double)sig[v] * acc;
            delta[v] = dv;
            double mult = (J->semantics == ORC_BC_REFERENCE) ? (double)npred[v] : 1.0;
            J->bc[v] += dv * mult;
        }
        for (int64_t h = 0; h < tail; h++) dist[q[h]] = -1;
    }
    free(dist); free(q); free(npred); free(sig); free(ovf); free(sigf); free(delta); free(shift);
    return NULL;
}

int orc_bc(int32_t N, const int64_t* row, const int32_t* col, const int32_t* src,
           int32_t k, int semantics, int scaled, int nthreads, double* bc, int64_t* n_ovf) {
    for (int32_t i = 0; i < k; i++) if (src[i] < 0 || src[i] >= N) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > k) nthreads = k > 0 ? k : 1;
    bc_job* jobs = (bc_job*)calloc((size_t)nthreads, sizeof(bc_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        jobs[t].N = N; jobs[t].row = row; jobs[t].col = col; jobs[t].src = src;
        jobs[t].k0 = (int32_t)((int64_t)k * t / nthreads);
        jobs[t].k1 = (int32_t)((int64_t)k * (t + 1) / nthreads);
        jobs[t].semantics = semantics; jobs[t].scaled = scaled;
        jobs[t].bc = (t == 0) ? bc : (double*)calloc((size_t)N, sizeof(double));
        jobs[t].n_ovf = 0;
        if (nthreads == 1) bc_worker(&jobs[t]);
        else pthread_create(&th[t], NULL, bc_worker, &jobs[t]);
    }
    int64_t tot = 0;
    for (int t = 0; t < nthreads; t++) {
        if (nthreads > 1) pthread_join(th[t], NULL);
        tot += jobs[t].n_ovf;
    }
    for (int t = 1; t < nthreads; t++) {
        for (int32_t v = 0; v < N; v++) bc[v] += jobs[t].bc[v];
        free(jobs[t].bc);
    }
    if (n_ovf) *n_ovf = tot;
    free(jobs); free(th);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Closeness distance sums (Seq_CC/CC.cpp:37-117; weighted form CC.cpp:
 * 1828-1843).                                                               */
typedef struct {
    int32_t N;
    const int64_t* row;
    const int32_t* col;
    const int32_t* src;
    int32_t k0, k1;
    const int64_t* w;
    const int64_t* ff;
    int64_t* cc;
} cc_job;

static void* cc_worker(void* arg) {
    cc_job* J = (cc_job*)arg;
    int32_t* dist = (int32_t*)malloc(sizeof(int32_t) * (size_t)J->N);
    int32_t* q = (int32_t*)malloc(sizeof(int32_t) * (size_t)J->N);
    for (int32_t v = 0; v < J->N; v++) dist[v] = -1;
    for (int32_t i = J->k0; i < J->k1; i++) {
        int32_t s = J->src[i];
        int64_t head = 0, tail = 0, sum = 0;
        q[tail++] = s;
        dist[s] = 0;
        while (head < tail) {
            int32_t v = q[head++];
            for (int64_t e = J->row[v]; e < J->row[v + 1]; e++) {
                int32_t u = J->col[e];
                if (dist[u] < 0) {
                    dist[u] = dist[v] + 1;
                    q[tail++] = u;
                    if (J->w) sum += J->ff[u] + (int64_t)dist[u] * J->w[u];
                    else sum += dist[u];
                }
            }
        }
        if (J->w) sum += J->ff[s];
        J->cc[i] = sum;
        for (int64_t h = 0; h < tail; h++) dist[q[h]] = -1;
    }
    free(dist); free(q);
    return NULL;
}

int orc_cc(int32_t N, const int64_t* row, const int32_t* col, const int32_t* src,
           int32_t k, const int64_t* w, const int64_t* ff, int nthreads, int64_t* cc) {
    for (int32_t i = 0; i < k; i++) if (src[i] < 0 || src[i] >= N) return -1;
    if ((w == NULL) != (ff == NULL)) return -2;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > k) nthreads = k > 0 ? k : 1;
    cc_job* jobs = (cc_job*)calloc((size_t)nthreads, sizeof(cc_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        cc_job* J = &jobs[t];
        J->N = N; J->row = row; J->col = col; J->src = src; J->w = w; J->ff = ff; J->cc = cc;
        J->k0 = (int32_t)((int64_t)k * t / nthreads);
        J->k1 = (int32_t)((int64_t)k * (t + 1) / nthreads);
        if (nthreads == 1) cc_worker(J);
        else pthread_create(&th[t], NULL, cc_worker, J);
    }
    if (nthreads > 1) for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(jobs); free(th);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Shared-BFS closeness (Seq_CC/CC.cpp:1779-2030, unreduced graph, unit
 * weights).  One BFS from s computes dist, the shared-bit index SI (which of
 * up to 32 mapped neighbours n_i lie on a shortest s->v path; CC.cpp:1903-
 * 1915) and the relation bits R (CC.cpp:1916-1921 for same-level edges,
 * CC.cpp:1937-1951 for propagation down the DAG).  Then, per mapped
 * neighbour (CC.cpp:1980-2003):
 *     d(n_i, v) = d(s, v) - 1            if SI_i(v)
 *               = d(s, v) + 1 - R_i(v)   otherwise.                          */
int64_t orc_cc_shared(int32_t N, const int64_t* row, const int32_t* col,
                      const int32_t* order, int32_t norder, int64_t* cc) {
    int32_t* dist = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t* q = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    uint32_t* SI = (uint32_t*)calloc((size_t)N, sizeof(uint32_t));
    uint32_t* R = (uint32_t*)calloc((size_t)N, sizeof(uint32_t));
    uint8_t* done = (uint8_t*)calloc((size_t)N, 1);
    int32_t mapped[32];
    int64_t runs = 0;
    for (int32_t v = 0; v < N; v++) dist[v] = -1;
    for (int32_t oi = 0; oi < norder; oi++) {
        int32_t s = order[oi];
        if (s < 0 || s >= N || done[s]) continue;
        done[s] = 1;
        runs++;
        int nm = 0;
        for (int64_t e = row[s]; e < row[s + 1] && nm < 32; e++) {
            int32_t u = col[e];
            if (!done[u]) { int dup = 0; for (int j = 0; j < nm; j++) dup |= (mapped[j] == u); if (!dup) mapped[nm++] = u; }
        }
        int share = nm >= 3;  /* CC.cpp:1825 */
        if (share) for (int j = 0; j < nm; j++) SI[mapped[j]] = 1u << j;
        int64_t head = 0, tail = 0, sum = 0;
        q[tail++] = s;
        dist[s] = 0;
        while (head < tail) {
            int32_t v = q[head++];
            for (int64_t e = row[v]; e < row[v + 1]; e++) {
                int32_t u = col[e];
                if (dist[u] < 0) {
                    dist[u] = dist[v] + 1; q[tail++] = u; sum += dist[u];
                    if (share) SI[u] |= SI[v];
                } else if (share && dist[u] == dist[v] + 1) {
                    SI[u] |= SI[v];
                } else if (share && dist[u] == dist[v]) {
                    R[v] |= SI[u] & ~SI[v];
                }
            }
        }
        cc[s] = sum;
        if (share) {
            for (int64_t h = 0; h < tail; h++) {
                int32_t v = q[h];
                for (int64_t e = row[v]; e < row[v + 1]; e++) {
                    int32_t u = col[e];
                    if (dist[u] == dist[v] + 1) R[u] |= R[v];
                }
            }
            for (int j = 0; j < nm; j++) {
                uint32_t bit = 1u << j;
                int64_t acc = 0;
                for (int64_t h = 0; h < tail; h++) {
                    int32_t v = q[h];
                    int64_t d = (SI[v] & bit) ? dist[v] - 1 : dist[v] + 1 - ((R[v] & bit) ? 1 : 0);
                    acc += d;
                }
                cc[mapped[j]] = acc;
                done[mapped[j]] = 1;
            }
        }
        for (int64_t h = 0; h < tail; h++) { int32_t v = q[h]; dist[v] = -1; SI[v] = 0; R[v] = 0; }
    }
    free(dist); free(q); free(SI); free(R); free(done);
    return runs;
}

/* ------------------------------------------------------------------------ */
/* Degree-1 folding (Lib/D1Process/D1Process.c:32-73). */
int orc_d1_fold(int32_t N, const int64_t* row, const int32_t* col, int32_t start,
                int64_t* represent, int64_t* ff, int32_t* parent, int64_t* live_lo,
                int32_t* col_out, int32_t* fold_order, int32_t* n_folded, int32_t* n_hub) {
    int64_t M = row[N];
    memcpy(col_out, col, sizeof(int32_t) * (size_t)M);
    int64_t* degv = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int32_t* q = (int32_t*)malloc(sizeof(int32_t) * ((size_t)N + 1));
    uint8_t* folded = (uint8_t*)calloc((size_t)N, 1);
    uint8_t* hub = (uint8_t*)calloc((size_t)N, 1);
    int64_t head = 0, tail = 0;
    for (int32_t v = 0; v < N; v++) {
        represent[v] = 1; ff[v] = 0; parent[v] = -1;
        live_lo[v] = row[v];
        degv[v] = row[v + 1] - row[v];
        if (v >= start && degv[v] == 1) q[tail++] = v;   /* AdjList.c:105 */
    }
    int32_t nf = 0;
    while (head < tail) {
        int32_t d1 = q[head++];
        if (degv[d1] != 1) continue;   /* tree root: last vertex of a tree component */
        int32_t p = col_out[live_lo[d1]];
        folded[d1] = 1;
        parent[d1] = p;
        hub[p] = 1;
        represent[p] += represent[d1];                 /* D1Process.c:43 */
        ff[p] += represent[d1] + ff[d1];               /* D1Process.c:46 */
        for (int64_t e = live_lo[p]; e < row[p + 1]; e++) {  /* D1Process.c:52-58 */
            if (col_out[e] == d1) {
                int32_t t = col_out[e]; col_out[e] = col_out[live_lo[p]]; col_out[live_lo[p]] = t;
                break;
            }
        }
        live_lo[p]++;                                   /* D1Process.c:63 */
        degv[d1] = 0;
        degv[p]--;
        if (degv[p] == 1) q[tail++] = p;               /* D1Process.c:67-69 */
        fold_order[nf++] = d1;
    }
    int32_t nh = 0;
    for (int32_t v = start; v < N; v++) if (hub[v] && !folded[v]) nh++;
    *n_folded = nf;
    *n_hub = nh;
    free(degv); free(q); free(folded); free(hub);
    return 0;
}

int32_t orc_components(int32_t N, const int64_t* row, const int32_t* col, int32_t* comp, int32_t* size_out) {
    int32_t* q = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    for (int32_t v = 0; v < N; v++) comp[v] = -1;
    int32_t nc = 0;
    for (int32_t r = 0; r < N; r++) {
        if (comp[r] >= 0) continue;
        int64_t head = 0, tail = 0;
        q[tail++] = r; comp[r] = nc;
        while (head < tail) {
            int32_t v = q[head++];
            for (int64_t e = row[v]; e < row[v + 1]; e++) {
                int32_t u = col[e];
                if (comp[u] < 0) { comp[u] = nc; q[tail++] = u; }
            }
        }
        if (size_out) for (int64_t h = 0; h < tail; h++) size_out[q[h]] = (int32_t)tail;
        nc++;
    }
    free(q);
    return nc;
}

/* Closeness through D1 folding (Seq_CC/CC.cpp:418-499). */
int orc_d1_cc(int32_t N, const int64_t* row, const int32_t* col, int32_t start,
              int fix_components, int64_t* cc) {
    int64_t M = row[N];
    int64_t* rep = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int64_t* ff = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int32_t* par = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int64_t* lo = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int32_t* col2 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(M ? M : 1));
    int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t nf = 0, nh = 0;
    orc_d1_fold(N, row, col, start, rep, ff, par, lo, col2, order, &nf, &nh);
    uint8_t* folded = (uint8_t*)calloc((size_t)N, 1);
    for (int32_t i = 0; i < nf; i++) folded[order[i]] = 1;
    /* weighted BFS over live ranges [lo[v], row[v+1]) (CC.cpp:436-474) */
    int32_t* dist = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t* q = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    for (int32_t v = 0; v < N; v++) { dist[v] = -1; cc[v] = 0; }
    for (int32_t s = start; s < N; s++) {
        if (folded[s]) continue;
        int64_t head = 0, tail = 0, sum = ff[s];
        q[tail++] = s; dist[s] = 0;
        while (head < tail) {
            int32_t v = q[head++];
            for (int64_t e = lo[v]; e < row[v + 1]; e++) {
                int32_t u = col2[e];
                if (dist[u] < 0) { dist[u] = dist[v] + 1; q[tail++] = u; sum += ff[u] + (int64_t)dist[u] * rep[u]; }
            }
        }
        cc[s] = sum;
        for (int64_t h = 0; h < tail; h++) dist[q[h]] = -1;
    }
    int32_t* csize = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t* comp = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    orc_components(N, row, col, comp, csize);
    int64_t total = N - start;  /* csr->totalNodeNumber */
    for (int32_t i = nf - 1; i >= 0; i--) {    /* CC.cpp:2037-2049 */
        int32_t d1 = order[i];
        int64_t Nn = fix_components ? csize[d1] : total;
        cc[d1] = cc[par[d1]] + Nn - 2 * rep[d1];
    }
    free(rep); free(ff); free(par); free(lo); free(col2); free(order); free(folded);
    free(dist); free(q); free(csize); free(comp);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Articulation points of the folded graph by iterative Tarjan (the
 * reference's AP_detection, Lib/AP_Process/AP_Process.c:6-140, computes the
 * same set with depth/low values over an explicit DFS stack).              */
static int32_t ap_core(int32_t N, const int64_t* row, const int64_t* lo, const int32_t* col2,
                       const uint8_t* folded, int32_t start, uint8_t* is_ap) {
    int32_t* disc = (int32_t*)calloc((size_t)N, sizeof(int32_t));
    int32_t* low = (int32_t*)calloc((size_t)N, sizeof(int32_t));
    int32_t* par = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t* stk = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int64_t* it = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int32_t* nchild = (int32_t*)calloc((size_t)N, sizeof(int32_t));
    int32_t timer = 0, count = 0;
    for (int32_t v = 0; v < N; v++) is_ap[v] = 0;
    for (int32_t r = start; r < N; r++) {
        if (folded[r] || disc[r]) continue;
        int32_t sp = 0;
        stk[sp++] = r; par[r] = -1; disc[r] = low[r] = ++timer; it[r] = lo[r];
        while (sp > 0) {
            int32_t v = stk[sp - 1];
            if (it[v] < row[v + 1]) {
                int32_t u = col2[it[v]++];
                if (!disc[u]) {
                    par[u] = v; disc[u] = low[u] = ++timer; it[u] = lo[u];
                    nchild[v]++;
                    stk[sp++] = u;
                } else if (u != par[v] && disc[u] < low[v]) {
                    low[v] = disc[u];
                }
            } else {
                sp--;
                int32_t p = par[v];
                if (p >= 0) {
                    if (low[v] < low[p]) low[p] = low[v];
                    if (par[p] >= 0 && low[v] >= disc[p]) is_ap[p] = 1;
                }
            }
        }
        if (nchild[r] > 1) is_ap[r] = 1;
    }
    for (int32_t v = 0; v < N; v++) count += is_ap[v];
    free(disc); free(low); free(par); free(stk); free(it); free(nchild);
    return count;
}

int32_t orc_articulation_points(int32_t N, const int64_t* row, const int32_t* col,
                                int32_t start, uint8_t* is_ap) {
    int64_t M = row[N];
    int64_t* rep = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int64_t* ff = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int32_t* par = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int64_t* lo = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int32_t* col2 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(M ? M : 1));
    int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t nf = 0, nh = 0;
    orc_d1_fold(N, row, col, start, rep, ff, par, lo, col2, order, &nf, &nh);
    uint8_t* folded = (uint8_t*)calloc((size_t)N, 1);
    for (int32_t i = 0; i < nf; i++) folded[order[i]] = 1;
    int32_t c = ap_core(N, row, lo, col2, folded, start, is_ap);
    free(rep); free(ff); free(par); free(lo); free(col2); free(order); free(folded);
    return c;
}

/* Per-AP parts (Lib/AP_Process/AP_Process.c:289-345 assigns part ids by BFS
 * that does not cross the AP; :383-466 sums each part's reach and ff from a
 * multi-source BFS seeded with the AP's neighbours in that part at distance
 * 1; :741 sets CC[ap] = total_ff + ff[ap]).                                  */
int32_t orc_ap_cc(int32_t N, const int64_t* row, const int32_t* col, int32_t start, int64_t* cc_ap) {
    int64_t M = row[N];
    int64_t* rep = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int64_t* ff = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int32_t* par = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int64_t* lo = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int32_t* col2 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(M ? M : 1));
    int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t nf = 0, nh = 0;
    orc_d1_fold(N, row, col, start, rep, ff, par, lo, col2, order, &nf, &nh);
    uint8_t* folded = (uint8_t*)calloc((size_t)N, 1);
    for (int32_t i = 0; i < nf; i++) folded[order[i]] = 1;
    uint8_t* is_ap = (uint8_t*)malloc((size_t)N);
    int32_t c = ap_core(N, row, lo, col2, folded, start, is_ap);
    int32_t* part = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t* dist = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    int32_t* q = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
    for (int32_t v = 0; v < N; v++) { part[v] = -1; dist[v] = -1; }
    for (int32_t a = start; a < N; a++) {
        if (!is_ap[a]) continue;
        /* part ids: BFS from each unlabelled live neighbour, never entering a */
        int32_t np = 0;
        int64_t touched = 0;
        for (int64_t e = lo[a]; e < row[a + 1]; e++) {
            int32_t x = col2[e];
            if (part[x] >= 0) continue;
            int64_t head = touched, tail = touched;
            q[tail++] = x; part[x] = np;
            while (head < tail) {
                int32_t v = q[head++];
                for (int64_t f = lo[v]; f < row[v + 1]; f++) {
                    int32_t u = col2[f];
                    if (u != a && part[u] < 0) { part[u] = np; q[tail++] = u; }
                }
            }
            touched = tail;
            np++;
        }
        /* per part: multi-source BFS seeded at distance 1 */
        int64_t total_ff = 0;
        dist[a] = 0;
        for (int32_t p = 0; p < np; p++) {
            int64_t head = 0, tail = 0, pff = 0;
            for (int64_t e = lo[a]; e < row[a + 1]; e++) {
                int32_t x = col2[e];
                if (part[x] == p && dist[x] < 0) { dist[x] = 1; q[tail++] = x; pff += ff[x] + rep[x]; }
            }
            while (head < tail) {
                int32_t v = q[head++];
                for (int64_t f = lo[v]; f < row[v + 1]; f++) {
                    int32_t u = col2[f];
                    if (dist[u] < 0) { dist[u] = dist[v] + 1; q[tail++] = u; pff += ff[u] + (int64_t)dist[u] * rep[u]; }
                }
            }
            total_ff += pff;
            for (int64_t h = 0; h < tail; h++) { dist[q[h]] = -1; }
        }
        dist[a] = -1;
        cc_ap[a] = total_ff + ff[a];
        /* clear part labels of this AP's component */
        for (int32_t v = 0; v < N; v++) part[v] = -1;
    }
    free(rep); free(ff); free(par); free(lo); free(col2); free(order); free(folded);
    free(is_ap); free(part); free(dist); free(q);
    return c;
}

/* ------------------------------------------------------------------------ */
/* Seeded R-MAT generator, so the bench's CPU legs build their graph without
 * the product library.  It restates gbc_gen_rmat of libgbc bit for bit: a
 * splitmix64-seeded xoshiro256** stream per block of 65,536 edges (stream
 * 1000 + block), one uniform per level choosing a quadrant (a, b, c, rest),
 * a Fisher-Yates relabelling (stream 7, Lemire's bounded draw), then the
 * symmetric CSR without self-loops or repeated edges, rows ascending.
 * tests/test_oracle.py checks the two generators give identical arrays.     */
typedef struct { uint64_t s[4]; } orc_rng;

static uint64_t orc_splitmix(uint64_t* x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static void orc_rng_init(orc_rng* r, uint64_t seed, uint64_t stream) {
    uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull);
    for (int i = 0; i < 4; i++) r->s[i] = orc_splitmix(&x);
}
static inline uint64_t orc_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t orc_next(orc_rng* r) {
    uint64_t* s = r->s;
    const uint64_t out = orc_rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t;
    s[3] = orc_rotl(s[3], 45);
    return out;
}
static double orc_uniform(orc_rng* r) { return (double)(orc_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static uint64_t orc_below(orc_rng* r, uint64_t bound) {
    if (bound == 0) return 0;
    unsigned __int128 m = (unsigned __int128)orc_next(r) * bound;
    uint64_t l = (uint64_t)m;
    if (l < bound) {
        const uint64_t t = (0 - bound) % bound;
        while (l < t) { m = (unsigned __int128)orc_next(r) * bound; l = (uint64_t)m; }
    }
    return (uint64_t)(m >> 64);
}

typedef struct {
    int32_t scale, nthreads, tid;
    double a, b, c;
    uint64_t seed;
    int64_t E;
    int32_t *eu, *ev;
    const int32_t* perm;
    int64_t* row;
    int32_t* col;
    int64_t* fill;
    int64_t* newdeg;
    int32_t n;
    int phase;
} rmat_job;

static int cmp_i32(const void* x, const void* y) {
    const int32_t a = *(const int32_t*)x, b = *(const int32_t*)y;
    return (a > b) - (a < b);
}

static void* rmat_worker(void* arg) {
    rmat_job* J = (rmat_job*)arg;
    const int64_t chunk = 1 << 16;
    if (J->phase == 0) {   /* edges, block ci on thread ci % nthreads */
        const int64_t nchunks = (J->E + chunk - 1) / chunk;
        for (int64_t ci = J->tid; ci < nchunks; ci += J->nthreads) {
            orc_rng r;
            orc_rng_init(&r, J->seed, 1000 + (uint64_t)ci);
            const int64_t hi = J->E < (ci + 1) * chunk ? J->E : (ci + 1) * chunk;
            for (int64_t i = ci * chunk; i < hi; i++) {
                uint32_t x = 0, y = 0;
                for (int32_t l = 0; l < J->scale; l++) {
                    const double p = orc_uniform(&r);
                    uint32_t bx = 0, by = 0;
                    if (p < J->a) {
                    } else if (p < J->a + J->b) {
                        by = 1;
                    } else if (p < J->a + J->b + J->c) {
                        bx = 1;
                    } else {
                        bx = 1;
                        by = 1;
                    }
                    x = (x << 1) | bx;
                    y = (y << 1) | by;
                }
                J->eu[i] = J->perm ? J->perm[x] : (int32_t)x;
                J->ev[i] = J->perm ? J->perm[y] : (int32_t)y;
            }
        }
    } else {   /* sort + unique the rows of vertices tid, tid + nthreads, ... */
        for (int32_t x = J->tid; x < J->n; x += J->nthreads) {
            int32_t* p = J->col + J->row[x];
            const int64_t len = J->row[x + 1] - J->row[x];
            qsort(p, (size_t)len, sizeof(int32_t), cmp_i32);
            int64_t k = 0;
            for (int64_t i = 0; i < len; i++)
                if (k == 0 || p[i] != p[k - 1]) p[k++] = p[i];
            J->newdeg[x] = k;
        }
    }
    return NULL;
}

int orc_gen_rmat(int32_t scale, int32_t ef, double a, double b, double c, uint64_t seed, int permute, int nthreads,
                 int32_t* n_out, int64_t** row_out, int32_t** col_out) {
    if (scale < 1 || scale > 30 || ef < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    const int32_t n = (int32_t)1 << scale;
    const int64_t E = (int64_t)ef * n;
    int32_t* eu = (int32_t*)malloc(sizeof(int32_t) * (size_t)E);
    int32_t* ev = (int32_t*)malloc(sizeof(int32_t) * (size_t)E);
    int32_t* perm = NULL;
    if (!eu || !ev) { free(eu); free(ev); return -2; }
    if (permute) {
        perm = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
        if (!perm) { free(eu); free(ev); return -2; }
        for (int32_t i = 0; i < n; i++) perm[i] = i;
        orc_rng pr;
        orc_rng_init(&pr, seed, 7);
        for (int32_t i = n - 1; i > 0; i--) {
            const int32_t j = (int32_t)orc_below(&pr, (uint64_t)i + 1);
            const int32_t t = perm[i];
            perm[i] = perm[j];
            perm[j] = t;
        }
    }
    rmat_job* jobs = (rmat_job*)calloc((size_t)nthreads, sizeof(rmat_job));
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) {
        rmat_job J = {scale, nthreads, t, a, b, c, seed, E, eu, ev, perm, NULL, NULL, NULL, NULL, n, 0};
        jobs[t] = J;
        pthread_create(&th[t], NULL, rmat_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(perm);
    /* both directions of every non-loop edge, then sorted unique rows */
    int64_t* row = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    for (int64_t i = 0; i < E; i++)
        if (eu[i] != ev[i]) { row[eu[i] + 1]++; row[ev[i] + 1]++; }
    for (int32_t i = 0; i < n; i++) row[i + 1] += row[i];
    int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(row[n] ? row[n] : 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    memcpy(fill, row, sizeof(int64_t) * (size_t)n);
    for (int64_t i = 0; i < E; i++)
        if (eu[i] != ev[i]) { col[fill[eu[i]]++] = ev[i]; col[fill[ev[i]]++] = eu[i]; }
    free(fill);
    free(eu);
    free(ev);
    int64_t* newdeg = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    for (int t = 0; t < nthreads; t++) {
        jobs[t].phase = 1;
        jobs[t].row = row;
        jobs[t].col = col;
        jobs[t].newdeg = newdeg;
        pthread_create(&th[t], NULL, rmat_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(jobs);
    free(th);
    int64_t* orow = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
    orow[0] = 0;
    for (int32_t i = 0; i < n; i++) orow[i + 1] = orow[i] + newdeg[i];
    int32_t* ocol = (int32_t*)malloc(sizeof(int32_t) * (size_t)(orow[n] ? orow[n] : 1));
    for (int32_t i = 0; i < n; i++) memcpy(ocol + orow[i], col + row[i], sizeof(int32_t) * (size_t)newdeg[i]);
    free(newdeg);
    free(row);
    free(col);
    *n_out = n;
    *row_out = orow;
    *col_out = ocol;
    return 0;
}
