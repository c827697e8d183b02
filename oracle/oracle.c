/*
 * oracle.c -- CPU oracle for the EEGraph push-kernel path (declarations and scope in oracle.h).
 * TEST INFRASTRUCTURE ONLY. Plain C written for clarity; the FP64 PageRank solvers and the input
 * generators also run on several threads (OpenMP) so that full-size checks finish in seconds.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ text parsing (src/graph.cpp:35-105) */

static int is_sp(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }
static int is_dg(char c) { return c >= '0' && c <= '9'; }

/* `istream >> unsigned`: skip blanks, optional sign, digits; returns 1 on success. */
static int tok_u32(const char** pp, const char* e, uint32_t* out) {
    const char* p = *pp;
    while (p < e && is_sp(*p)) ++p;
    int neg = 0;
    if (p < e && (*p == '+' || *p == '-')) {
        neg = *p == '-';
        ++p;
    }
    if (p >= e || !is_dg(*p)) {
        *out = 0;
        return 0;
    }
    uint64_t v = 0;
    int over = 0;
    while (p < e && is_dg(*p)) {
        if (!over) {
            v = v * 10 + (uint64_t)(*p - '0');
            if (v > 0xFFFFFFFFull) over = 1;
        }
        ++p;
    }
    *pp = p;
    if (over) {
        *out = 0xFFFFFFFFu;
        return 0;
    }
    *out = neg ? (uint32_t)(0u - (uint32_t)v) : (uint32_t)v;
    return 1;
}

typedef struct {
    uint64_t m;
    uint32_t max;
    int zero;
    int weighted;
    uint32_t *s, *d, *w;
} parse_state;

static int parse_file(const char* path, parse_state* st) {
    FILE* f = fopen(path, "rb");
    if (!f) return -1;
    size_t cap = 1 << 16, len = 0;
    char* line = (char*)malloc(cap);
    int c;
    for (;;) {
        len = 0;
        while ((c = fgetc(f)) != EOF && c != '\n') {
            if (len + 1 >= cap) {
                cap *= 2;
                line = (char*)realloc(line, cap);
            }
            line[len++] = (char)c;
        }
        if (c == EOF && len == 0) break;
        line[len] = 0;
        if (len > 0 && is_dg(line[0])) { /* src/graph.cpp:66-67: skip lines not starting with a digit */
            const char* p = line;
            const char* e = line + len;
            uint32_t s = 0, d = 0, w = 1;
            int ok = tok_u32(&p, e, &s);
            if (ok) ok = tok_u32(&p, e, &d);
            else d = 0;
            if (st->weighted) {
                uint32_t t = 1;
                w = (ok && tok_u32(&p, e, &t)) ? t : 1u;
            }
            if (st->s) {
                st->s[st->m] = s;
                st->d[st->m] = d;
                if (st->w) st->w[st->m] = w;
            }
            if (s == 0 || d == 0) st->zero = 1;
            if (s > st->max) st->max = s;
            if (d > st->max) st->max = d;
            st->m++;
        }
        if (c == EOF) break;
    }
    free(line);
    fclose(f);
    return 0;
}

int orc_parse_count(const char* path, uint64_t* num_edges, uint32_t* num_nodes, int* has_zero_id) {
    parse_state st;
    memset(&st, 0, sizeof(st));
    if (parse_file(path, &st) != 0) return -1;
    *num_edges = st.m;
    *has_zero_id = st.zero;
    *num_nodes = st.zero ? st.max + 1 : st.max; /* src/graph.cpp:102-105 */
    return 0;
}

int orc_parse_fill(const char* path, int weighted, uint32_t* src, uint32_t* dst, uint32_t* w) {
    parse_state st;
    memset(&st, 0, sizeof(st));
    st.weighted = weighted;
    st.s = src;
    st.d = dst;
    st.w = weighted ? w : NULL;
    return parse_file(path, &st);
}

/* ------------------------------------------------------------------ virtual graph (src/virtual_graph.cpp:36-112) */

static uint32_t ceil_div(uint32_t a, uint32_t b) { return a % b == 0 ? a / b : a / b + 1; }

uint64_t orc_num_parts(uint32_t n, uint64_t m, const uint32_t* src, uint32_t K) {
    uint32_t* deg = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    for (uint64_t e = 0; e < m; ++e) deg[src[e]]++;
    uint64_t p = 0;
    for (uint32_t v = 0; v < n; ++v) p += ceil_div(deg[v], K);
    free(deg);
    return p;
}

void orc_virtual_graph(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w,
                       uint32_t K, uint32_t* nodePointer, uint32_t* edgeList, uint32_t* partNodePointer) {
    uint32_t* deg = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    uint32_t* cnt = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t)); /* zeroed (the reference's is not, :66) */
    for (uint64_t e = 0; e < m; ++e) deg[src[e]]++;
    uint64_t counter = 0;
    for (uint32_t v = 0; v < n; ++v) {
        nodePointer[v] = (uint32_t)counter;
        edgeList[counter] = deg[v];
        counter += 2 * (uint64_t)deg[v] + 1;
    }
    for (uint64_t e = 0; e < m; ++e) { /* no `location >= num_edges` drop (src/virtual_graph.cpp:86-88) */
        const uint32_t s = src[e];
        const uint64_t loc = (uint64_t)nodePointer[s] + 1 + 2 * (uint64_t)cnt[s];
        edgeList[loc] = dst[e];
        edgeList[loc + 1] = w ? w[e] : 1u;
        cnt[s]++;
    }
    uint64_t p = 0;
    for (uint32_t v = 0; v < n; ++v) {
        const uint32_t np = ceil_div(deg[v], K);
        for (uint32_t j = 0; j < np; ++j, ++p) {
            partNodePointer[2 * p] = v;
            partNodePointer[2 * p + 1] = j;
        }
    }
    free(deg);
    free(cnt);
}

void orc_init_values(int algo, uint32_t n, uint32_t source, uint32_t* dist) {
    for (uint32_t v = 0; v < n; ++v) {
        if (algo == ORC_CC) dist[v] = v;                                  /* src/eegraph.cu:546 */
        else if (algo == ORC_SSWP) dist[v] = v == source ? ORC_INF : 0u;  /* src/eegraph.cu:1551-1559 */
        else dist[v] = v == source ? 0u : ORC_INF;                        /* src/eegraph.cu:41-49 */
    }
}

/* one relaxation of edge slot `end` from a vertex holding `sw`; returns 1 when dist improved */
static int relax(int algo, int wrap, uint32_t sw, uint32_t t, uint32_t w8, uint32_t* dist) {
    uint32_t fd;
    if (algo == ORC_SSWP) {
        fd = sw < w8 ? sw : w8;
        if (fd > dist[t]) {
            dist[t] = fd;
            return 1;
        }
        return 0;
    }
    const uint32_t add = algo == ORC_BFS ? 1u : w8;
    if (wrap) {
        fd = sw + add; /* uint32 arithmetic as in the reference */
    } else {
        if ((algo == ORC_BFS || algo == ORC_SSSP) && sw == ORC_INF) return 0;
        const uint64_t s = (uint64_t)sw + add;
        fd = s >= ORC_INF ? ORC_INF : (uint32_t)s;
    }
    if (fd < dist[t]) {
        dist[t] = fd;
        return 1;
    }
    return 0;
}

static int unreached(int algo, uint32_t d) {
    if (algo == ORC_BFS || algo == ORC_SSSP) return d == ORC_INF;
    if (algo == ORC_SSWP) return d == 0;
    return 0;
}

/* the body shared by seq_cpu and the frontier rounds: part (id, part) with the strided slot order
 * j + i*ceil(deg/K) of the reference kernels (src/sssp.cu:377-399) */
static int expand_part(int algo, int wrap, uint32_t id, uint32_t part, const uint32_t* nodePointer,
                       const uint32_t* edgeList, uint32_t K, uint32_t* dist, uint8_t* mark) {
    const uint32_t sw = dist[id];
    const uint32_t tp = nodePointer[id];
    const uint32_t degree = edgeList[tp];
    const uint32_t np = ceil_div(degree, K);
    const uint64_t ofs = (uint64_t)tp + 2 * (uint64_t)part + 1;
    int changed = 0;
    for (uint32_t i = 0; i < K; ++i) {
        if ((uint64_t)part + (uint64_t)i * np >= degree) break;
        const uint64_t end = ofs + (uint64_t)i * np * 2;
        const uint32_t t = edgeList[end];
        if (relax(algo, wrap, sw, t, edgeList[end + 1], dist)) {
            changed = 1;
            if (mark) mark[t] = 1;
        }
    }
    return changed;
}

int64_t orc_seq_sweep(int algo, uint32_t n, uint64_t num_parts, const uint32_t* nodePointer, const uint32_t* edgeList,
                      const uint32_t* partNodePointer, uint32_t K, int wrap, uint64_t max_sweeps, uint32_t* dist) {
    (void)n;
    int64_t sweeps = 0;
    int finished;
    do {
        if (max_sweeps && (uint64_t)sweeps >= max_sweeps) return -1;
        finished = 1;
        ++sweeps;
        for (uint64_t p = 0; p < num_parts; ++p) {
            const uint32_t id = partNodePointer[2 * p], part = partNodePointer[2 * p + 1];
            if (!wrap && unreached(algo, dist[id])) continue;
            if (expand_part(algo, wrap, id, part, nodePointer, edgeList, K, dist, NULL)) finished = 0;
        }
    } while (!finished);
    return sweeps;
}

int64_t orc_frontier_sweep(int algo, uint32_t n, uint64_t num_parts, const uint32_t* nodePointer,
                           const uint32_t* edgeList, const uint32_t* partNodePointer, uint32_t K, int seed_all,
                           uint32_t source, uint32_t* dist) {
    uint8_t* l1 = (uint8_t*)calloc(n ? n : 1, 1);
    uint8_t* l2 = (uint8_t*)calloc(n ? n : 1, 1);
    if (seed_all) memset(l1, 1, n);
    else l1[source] = 1;
    int64_t rounds = 0;
    int finished;
    do {
        finished = 1;
        ++rounds;
        for (uint64_t p = 0; p < num_parts; ++p) {
            const uint32_t id = partNodePointer[2 * p], part = partNodePointer[2 * p + 1];
            if (!l1[id] || unreached(algo, dist[id])) continue;
            if (expand_part(algo, 0, id, part, nodePointer, edgeList, K, dist, l2)) finished = 0;
        }
        uint8_t* t = l1;
        l1 = l2;
        l2 = t;
        memset(l2, 0, n);
    } while (!finished);
    free(l1);
    free(l2);
    return rounds;
}

/* ------------------------------------------------------------------ independent oracles */

typedef struct {
    uint64_t* off;
    uint32_t* col;
    uint32_t* w;
} csr;

static csr make_csr(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w) {
    csr c;
    c.off = (uint64_t*)calloc((size_t)n + 1, sizeof(uint64_t));
    c.col = (uint32_t*)malloc((m ? m : 1) * sizeof(uint32_t));
    c.w = (uint32_t*)malloc((m ? m : 1) * sizeof(uint32_t));
    for (uint64_t e = 0; e < m; ++e) c.off[src[e] + 1]++;
    for (uint32_t v = 0; v < n; ++v) c.off[v + 1] += c.off[v];
    uint64_t* pos = (uint64_t*)malloc(((size_t)n + 1) * sizeof(uint64_t));
    memcpy(pos, c.off, ((size_t)n + 1) * sizeof(uint64_t));
    for (uint64_t e = 0; e < m; ++e) {
        const uint64_t at = pos[src[e]]++;
        c.col[at] = dst[e];
        c.w[at] = w ? w[e] : 1u;
    }
    free(pos);
    return c;
}

static void free_csr(csr* c) {
    free(c->off);
    free(c->col);
    free(c->w);
}

void orc_bfs(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, uint32_t source, uint32_t* dist) {
    csr c = make_csr(n, m, src, dst, NULL);
    uint32_t* q = (uint32_t*)malloc((n ? n : 1) * sizeof(uint32_t));
    for (uint32_t v = 0; v < n; ++v) dist[v] = ORC_INF;
    uint64_t h = 0, t = 0;
    dist[source] = 0;
    q[t++] = source;
    while (h < t) {
        const uint32_t u = q[h++];
        for (uint64_t e = c.off[u]; e < c.off[u + 1]; ++e) {
            const uint32_t v = c.col[e];
            if (dist[v] == ORC_INF) {
                dist[v] = dist[u] + 1;
                q[t++] = v;
            }
        }
    }
    free(q);
    free_csr(&c);
}

/* binary heap of (key, vertex); min-heap, or max-heap when maxh */
typedef struct {
    uint64_t* k;
    uint32_t* v;
    uint64_t n, cap;
    int maxh;
} heap;

static int hless(const heap* h, uint64_t a, uint64_t b) { return h->maxh ? h->k[a] > h->k[b] : h->k[a] < h->k[b]; }
static void hswap(heap* h, uint64_t a, uint64_t b) {
    uint64_t tk = h->k[a];
    h->k[a] = h->k[b];
    h->k[b] = tk;
    uint32_t tv = h->v[a];
    h->v[a] = h->v[b];
    h->v[b] = tv;
}
static void hpush(heap* h, uint64_t key, uint32_t v) {
    if (h->n == h->cap) {
        h->cap = h->cap ? 2 * h->cap : 1024;
        h->k = (uint64_t*)realloc(h->k, h->cap * sizeof(uint64_t));
        h->v = (uint32_t*)realloc(h->v, h->cap * sizeof(uint32_t));
    }
    uint64_t i = h->n++;
    h->k[i] = key;
    h->v[i] = v;
    while (i > 0 && hless(h, i, (i - 1) / 2)) {
        hswap(h, i, (i - 1) / 2);
        i = (i - 1) / 2;
    }
}
static void hpop(heap* h, uint64_t* key, uint32_t* v) {
    *key = h->k[0];
    *v = h->v[0];
    h->n--;
    h->k[0] = h->k[h->n];
    h->v[0] = h->v[h->n];
    uint64_t i = 0;
    for (;;) {
        uint64_t l = 2 * i + 1, r = l + 1, b = i;
        if (l < h->n && hless(h, l, b)) b = l;
        if (r < h->n && hless(h, r, b)) b = r;
        if (b == i) break;
        hswap(h, i, b);
        i = b;
    }
}

/* multi-source Dijkstra: dist holds the initial keys; every vertex with a key < INF starts queued */
static void dijkstra_from(const csr* c, uint32_t n, uint32_t* dist) {
    heap h;
    memset(&h, 0, sizeof(h));
    for (uint32_t v = 0; v < n; ++v)
        if (dist[v] != ORC_INF) hpush(&h, dist[v], v);
    while (h.n) {
        uint64_t d;
        uint32_t u;
        hpop(&h, &d, &u);
        if (d != dist[u]) continue;
        for (uint64_t e = c->off[u]; e < c->off[u + 1]; ++e) {
            const uint32_t t = c->col[e];
            uint64_t nd = d + c->w[e];
            if (nd > ORC_INF) nd = ORC_INF;
            if (nd < dist[t]) {
                dist[t] = (uint32_t)nd;
                hpush(&h, nd, t);
            }
        }
    }
    free(h.k);
    free(h.v);
}

void orc_dijkstra(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w,
                  uint32_t source, uint32_t* dist) {
    csr c = make_csr(n, m, src, dst, w);
    for (uint32_t v = 0; v < n; ++v) dist[v] = ORC_INF;
    dist[source] = 0;
    dijkstra_from(&c, n, dist);
    free_csr(&c);
}

void orc_cc_labels(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w, uint32_t* out) {
    csr c = make_csr(n, m, src, dst, w);
    for (uint32_t v = 0; v < n; ++v) out[v] = v;
    dijkstra_from(&c, n, out);
    free_csr(&c);
}

void orc_widest(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w,
                uint32_t source, uint32_t* out) {
    csr c = make_csr(n, m, src, dst, w);
    for (uint32_t v = 0; v < n; ++v) out[v] = 0;
    out[source] = ORC_INF;
    heap h;
    memset(&h, 0, sizeof(h));
    h.maxh = 1;
    hpush(&h, ORC_INF, source);
    while (h.n) {
        uint64_t d;
        uint32_t u;
        hpop(&h, &d, &u);
        if (d != out[u] || d == 0) continue;
        for (uint64_t e = c.off[u]; e < c.off[u + 1]; ++e) {
            const uint32_t t = c.col[e];
            const uint32_t nd = (uint32_t)d < c.w[e] ? (uint32_t)d : c.w[e];
            if (nd > out[t]) {
                out[t] = nd;
                hpush(&h, nd, t);
            }
        }
    }
    free(h.k);
    free(h.v);
    free_csr(&c);
}

/* Edges grouped by one endpoint (`key` = dst for a pull over in-edges, src for a pull over out-edges),
 * stable: within a group the edges keep their input order, so a pull that adds them in group order
 * adds them in the same order as a sequential scatter over the edge list would (same FP64 results). */
typedef struct {
    uint64_t* off; /* n + 1 */
    uint64_t* eid; /* m: input edge index */
} groups;

static groups group_by(uint32_t n, uint64_t m, const uint32_t* key) {
    groups g;
    g.off = (uint64_t*)calloc((size_t)n + 1, sizeof(uint64_t));
    g.eid = (uint64_t*)malloc((m ? m : 1) * sizeof(uint64_t));
    for (uint64_t e = 0; e < m; ++e) g.off[key[e] + 1]++;
    for (uint32_t v = 0; v < n; ++v) g.off[v + 1] += g.off[v];
    uint64_t* pos = (uint64_t*)malloc(((size_t)n + 1) * sizeof(uint64_t));
    memcpy(pos, g.off, ((size_t)n + 1) * sizeof(uint64_t));
    for (uint64_t e = 0; e < m; ++e) g.eid[pos[key[e]]++] = e;
    free(pos);
    return g;
}

static void free_groups(groups* g) {
    free(g->off);
    free(g->eid);
}

/* Sums over fixed blocks of ORC_BLOCK vertices, added block by block: the same result for any thread count. */
#define ORC_BLOCK 4096u

int64_t orc_pagerank(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, double damping, double tol,
                     uint64_t max_iter, double* x) {
    return orc_pagerank_mt(n, m, src, dst, damping, tol, max_iter, 1, x);
}

void orc_in_csr(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, uint64_t* off, uint32_t* isrc,
                uint32_t* outdeg) {
    memset(off, 0, ((size_t)n + 1) * sizeof(uint64_t));
    memset(outdeg, 0, (size_t)n * sizeof(uint32_t));
    for (uint64_t e = 0; e < m; ++e) {
        off[dst[e] + 1]++;
        outdeg[src[e]]++;
    }
    for (uint32_t v = 0; v < n; ++v) off[v + 1] += off[v];
    uint64_t* pos = (uint64_t*)malloc(((size_t)n + 1) * sizeof(uint64_t));
    memcpy(pos, off, ((size_t)n + 1) * sizeof(uint64_t));
    for (uint64_t e = 0; e < m; ++e) isrc[pos[dst[e]]++] = src[e]; /* stable: input order per target */
    free(pos);
}

int64_t orc_pagerank_pull(uint32_t n, const uint64_t* off, const uint32_t* isrc, const uint32_t* outdeg,
                          double damping, double tol, uint64_t max_iter, int threads, double* x) {
    if (threads < 1) threads = 1;
    double* c = (double*)malloc((n ? n : 1) * sizeof(double));
    const uint32_t nb = (n + ORC_BLOCK - 1) / ORC_BLOCK;
    double* bdiff = (double*)calloc(nb ? nb : 1, sizeof(double));
    double* bnorm = (double*)calloc(nb ? nb : 1, sizeof(double));
    for (uint32_t v = 0; v < n; ++v) x[v] = 1.0 - damping;
    int64_t it = 0;
    while ((uint64_t)it < max_iter) {
        ++it;
        int64_t v0;
#pragma omp parallel for num_threads(threads) schedule(static)
        for (v0 = 0; v0 < (int64_t)n; ++v0) c[v0] = outdeg[v0] ? x[v0] / (double)outdeg[v0] : 0.0;
        int64_t b;
        /* x_new[v] depends on c only, so x is updated in place block by block */
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
        for (b = 0; b < (int64_t)nb; ++b) {
            double diff = 0.0, norm = 0.0;
            const uint32_t lo = (uint32_t)b * ORC_BLOCK;
            const uint32_t hi = lo + ORC_BLOCK < n ? lo + ORC_BLOCK : n;
            for (uint32_t v = lo; v < hi; ++v) {
                double y = 0.0;
                for (uint64_t i = off[v]; i < off[v + 1]; ++i) y += c[isrc[i]];
                const double nx = (1.0 - damping) + damping * y;
                diff += nx > x[v] ? nx - x[v] : x[v] - nx;
                norm += nx;
                x[v] = nx;
            }
            bdiff[b] = diff;
            bnorm[b] = norm;
        }
        double diff = 0.0, norm = 0.0;
        for (uint32_t k = 0; k < nb; ++k) {
            diff += bdiff[k];
            norm += bnorm[k];
        }
        if (diff <= tol * norm) break;
    }
    free(c);
    free(bdiff);
    free(bnorm);
    return it;
}

int64_t orc_pagerank_mt(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, double damping, double tol,
                        uint64_t max_iter, int threads, double* x) {
    uint64_t* off = (uint64_t*)malloc(((size_t)n + 1) * sizeof(uint64_t));
    uint32_t* isrc = (uint32_t*)malloc((m ? m : 1) * sizeof(uint32_t));
    uint32_t* deg = (uint32_t*)malloc((n ? n : 1) * sizeof(uint32_t));
    orc_in_csr(n, m, src, dst, off, isrc, deg);
    const int64_t it = orc_pagerank_pull(n, off, isrc, deg, damping, tol, max_iter, threads, x);
    free(off);
    free(isrc);
    free(deg);
    return it;
}

static double* orc_out_sums(uint32_t n, uint64_t m, const uint32_t* src, const double* w) {
    double* s = (double*)calloc(n ? n : 1, sizeof(double));
    for (uint64_t e = 0; e < m; ++e) s[src[e]] += w[e];
    return s;
}

int64_t orc_ppr_solve(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const double* w, uint32_t C,
                      const double* b, double scale_b, int transpose, double damping, double tol, uint64_t max_iter,
                      double* y) {
    return orc_ppr_solve_mt(n, m, src, dst, w, C, b, scale_b, transpose, damping, tol, max_iter, 1, y);
}

int64_t orc_ppr_solve_mt(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const double* w,
                         uint32_t C, const double* b, double scale_b, int transpose, double damping, double tol,
                         uint64_t max_iter, int threads, double* y) {
    if (threads < 1) threads = 1;
    const size_t N = (size_t)n * C;
    double* s = orc_out_sums(n, m, src, w);
    double* z = (double*)malloc((N ? N : 1) * sizeof(double));
    const uint32_t nb = (n + ORC_BLOCK - 1) / ORC_BLOCK;
    double* bdiff = (double*)calloc(nb ? nb : 1, sizeof(double));
    double* bnorm = (double*)calloc(nb ? nb : 1, sizeof(double));
    /* forward: v gathers the rows of its in-neighbours u; adjoint: u gathers the rows of its out-neighbours v */
    const uint32_t* to_key = transpose ? src : dst;
    const uint32_t* from_key = transpose ? dst : src;
    groups g = group_by(n, m, to_key);
    uint32_t* from = (uint32_t*)malloc((m ? m : 1) * sizeof(uint32_t));
    double* a = (double*)malloc((m ? m : 1) * sizeof(double));
    for (uint64_t i = 0; i < m; ++i) {
        const uint64_t e = g.eid[i];
        from[i] = from_key[e];
        a[i] = s[src[e]] == 0.0 ? 0.0 : damping * (w[e] / s[src[e]]);
    }
    for (size_t i = 0; i < N; ++i) y[i] = scale_b * b[i];
    int64_t it = 0;
    int converged = 0;
    while ((uint64_t)it < max_iter) {
        ++it;
        int64_t bk;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
        for (bk = 0; bk < (int64_t)nb; ++bk) {
            const uint32_t lo = (uint32_t)bk * ORC_BLOCK;
            const uint32_t hi = lo + ORC_BLOCK < n ? lo + ORC_BLOCK : n;
            for (uint32_t v = lo; v < hi; ++v) {
                double* zr = z + (size_t)v * C;
                for (uint32_t k = 0; k < C; ++k) zr[k] = scale_b * b[(size_t)v * C + k];
                for (uint64_t i = g.off[v]; i < g.off[v + 1]; ++i) {
                    if (a[i] == 0.0 && s[transpose ? v : from[i]] == 0.0) continue; /* source without out-weight */
                    const double* yr = y + (size_t)from[i] * C;
                    for (uint32_t k = 0; k < C; ++k) zr[k] += a[i] * yr[k];
                }
            }
        }
#pragma omp parallel for num_threads(threads) schedule(static)
        for (bk = 0; bk < (int64_t)nb; ++bk) {
            const size_t lo = (size_t)bk * ORC_BLOCK * C;
            const size_t hi = lo + (size_t)ORC_BLOCK * C < N ? lo + (size_t)ORC_BLOCK * C : N;
            double diff = 0.0, norm = 0.0;
            for (size_t i = lo; i < hi; ++i) {
                diff += fabs(z[i] - y[i]);
                norm += fabs(z[i]);
                y[i] = z[i];
            }
            bdiff[bk] = diff;
            bnorm[bk] = norm;
        }
        double diff = 0.0, norm = 0.0;
        for (uint32_t k = 0; k < nb; ++k) {
            diff += bdiff[k];
            norm += bnorm[k];
        }
        if (damping / (1.0 - damping) * diff <= tol * norm) {
            converged = 1;
            break;
        }
    }
    free(z);
    free(s);
    free(a);
    free(from);
    free(bdiff);
    free(bnorm);
    free_groups(&g);
    return converged ? it : -1;
}

void orc_ppr_grads(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const double* w, uint32_t C,
                   const double* X, const double* L, double damping, double* gWn, double* gw, double* gT) {
    double* s = orc_out_sums(n, m, src, w);
    double* g = (double*)malloc((m ? m : 1) * sizeof(double));
    double* r = (double*)calloc(n ? n : 1, sizeof(double));
    for (uint64_t e = 0; e < m; ++e) {
        const double* xr = X + (size_t)src[e] * C;
        const double* lr = L + (size_t)dst[e] * C;
        double dot = 0.0;
        for (uint32_t k = 0; k < C; ++k) dot += xr[k] * lr[k];
        g[e] = damping * dot;
        if (s[src[e]] != 0.0) r[src[e]] += g[e] * (w[e] / s[src[e]]);
    }
    for (uint64_t e = 0; e < m; ++e) {
        if (gWn) gWn[e] = g[e];
        if (gw) gw[e] = s[src[e]] != 0.0 ? (g[e] - r[src[e]]) / s[src[e]] : 0.0;
    }
    if (gT)
        for (size_t i = 0; i < (size_t)n * C; ++i) gT[i] = (1.0 - damping) * L[i];
    free(r);
    free(g);
    free(s);
}

/* ------------------------------------------------------------------ synthetic inputs
 * The seeded R-MAT and grid generators of the benchmark inputs, restated so that CPU-only code (the
 * reference arm of the benchmark, oracle-side tests) makes the same graphs without loading the product
 * library; tests check both give identical arrays. Counter-based: edge e depends only on (seed, e). */

static uint64_t orc_mix64(uint64_t z) { /* SplitMix64 finaliser (Steele, Lea, Flood 2014) */
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t orc_hash2(uint64_t a, uint64_t b) { return orc_mix64(a ^ orc_mix64(b + 0x632BE59BD9B4E019ull)); }

int orc_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed, uint32_t wmin,
                 uint32_t wmax, int threads, uint32_t* src, uint32_t* dst, uint32_t* weight) {
    if (!src || !dst || scale == 0 || scale > 31 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0 ||
        (weight && wmax < wmin))
        return -1;
    if (threads < 1) threads = 1;
    const uint64_t m = (uint64_t)edge_factor << scale;
    const double two32 = 4294967296.0;
    const uint64_t tA = (uint64_t)floor(a * two32);
    const uint64_t tAB = (uint64_t)floor((a + b) * two32);
    const uint64_t tABC = (uint64_t)floor((a + b + c) * two32);
    const uint64_t range = (uint64_t)wmax - wmin + 1u;
    int64_t e;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (e = 0; e < (int64_t)m; ++e) {
        const uint64_t s0 = orc_hash2(seed, (uint64_t)e);
        uint32_t u = 0, v = 0;
        uint64_t r = 0;
        for (uint32_t l = 0; l < scale; ++l) { /* one quadrant choice per level, two per 64-bit draw */
            if ((l & 1u) == 0) r = orc_mix64(s0 + 0x9E3779B97F4A7C15ull * (l / 2 + 1));
            const uint64_t x = (l & 1u) ? (r >> 32) : (r & 0xFFFFFFFFull);
            const uint32_t bit = 1u << (scale - 1 - l);
            if (x < tA) {
            } else if (x < tAB) {
                v |= bit;
            } else if (x < tABC) {
                u |= bit;
            } else {
                u |= bit;
                v |= bit;
            }
        }
        src[e] = u;
        dst[e] = v;
        if (weight) weight[e] = wmin + (uint32_t)(orc_mix64(s0 ^ 0xA5A5A5A55A5A5A5Aull) % range);
    }
    return 0;
}

/* grid edge i: horizontal (r,c)-(r,c+1) for i < S(S-1), vertical (r,c)-(r+1,c) up to E = 2S(S-1), then shortcuts */
static void grid_endpoints(uint64_t S, uint64_t E, uint64_t N, uint64_t seed, uint64_t i, uint32_t* u, uint32_t* v) {
    if (i < S * (S - 1)) {
        const uint64_t r = i / (S - 1), c = i % (S - 1);
        *u = (uint32_t)(r * S + c);
        *v = (uint32_t)(r * S + c + 1);
    } else if (i < E) {
        const uint64_t j = i - S * (S - 1);
        const uint64_t r = j / S, c = j % S;
        *u = (uint32_t)(r * S + c);
        *v = (uint32_t)((r + 1) * S + c);
    } else {
        const uint64_t j = i - E;
        *u = (uint32_t)(orc_hash2(seed ^ 0x5CA1AB1Eull, 2 * j) % N);
        *v = (uint32_t)(orc_hash2(seed ^ 0x5CA1AB1Eull, 2 * j + 1) % N);
    }
}

int orc_gen_grid(uint32_t side, double p_delete, double shortcut_frac, uint64_t seed, uint32_t wmin, uint32_t wmax,
                 int threads, uint64_t* num_arcs, uint32_t* src, uint32_t* dst, uint32_t* weight) {
    if (!num_arcs || side < 2 || (uint64_t)side * side > 0xFFFFFFFFull || p_delete < 0 || p_delete > 1 ||
        shortcut_frac < 0 || wmax < wmin)
        return -1;
    if (threads < 1) threads = 1;
    const uint64_t S = side, N = S * S, E = 2 * S * (S - 1);
    const uint64_t nshort = (uint64_t)llround(shortcut_frac * (double)E);
    const uint64_t thr = p_delete >= 1.0 ? ~0ull : (uint64_t)(p_delete * 18446744073709551616.0);
    const uint64_t range = (uint64_t)wmax - wmin + 1u;
    const uint64_t total = E + nshort, B = 1u << 16, nb = (total + B - 1) / B;
    uint64_t* cnt = (uint64_t*)calloc(nb + 1, sizeof(uint64_t));
    int64_t bk;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (bk = 0; bk < (int64_t)nb; ++bk) {
        uint64_t k = 0;
        const uint64_t hi = ((uint64_t)bk + 1) * B < total ? ((uint64_t)bk + 1) * B : total;
        for (uint64_t i = (uint64_t)bk * B; i < hi; ++i)
            k += (i >= E || p_delete <= 0 || orc_mix64(orc_hash2(seed, i)) >= thr) ? 1 : 0;
        cnt[bk + 1] = k;
    }
    for (uint64_t k = 0; k < nb; ++k) cnt[k + 1] += cnt[k];
    *num_arcs = 2 * cnt[nb];
    if (src && dst) {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (bk = 0; bk < (int64_t)nb; ++bk) {
            uint64_t o = 2 * cnt[bk];
            const uint64_t hi = ((uint64_t)bk + 1) * B < total ? ((uint64_t)bk + 1) * B : total;
            for (uint64_t i = (uint64_t)bk * B; i < hi; ++i) {
                if (!(i >= E || p_delete <= 0 || orc_mix64(orc_hash2(seed, i)) >= thr)) continue;
                uint32_t u, v;
                grid_endpoints(S, E, N, seed, i, &u, &v);
                const uint32_t w = wmin + (uint32_t)(orc_hash2(seed ^ 0x77EE77EEull, i) % range);
                src[o] = u;
                dst[o] = v;
                src[o + 1] = v;
                dst[o + 1] = u;
                if (weight) weight[o] = weight[o + 1] = w;
                o += 2;
            }
        }
    }
    free(cnt);
    return 0;
}

void orc_symmetrize(uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w, uint32_t* so,
                    uint32_t* d_o, uint32_t* wo) {
    for (uint64_t e = 0; e < m; ++e) { /* the input arcs, then every arc reversed with its weight */
        so[e] = src[e];
        d_o[e] = dst[e];
        so[m + e] = dst[e];
        d_o[m + e] = src[e];
        if (wo) wo[e] = wo[m + e] = w[e];
    }
}
