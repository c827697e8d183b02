/*
 * oracle.c -- CPU oracle for the EEGraph push-kernel path (declarations and scope in oracle.h).
 * TEST INFRASTRUCTURE ONLY. Plain C, single-threaded, written for clarity, not speed.
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

int64_t orc_pagerank(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, double damping, double tol,
                     uint64_t max_iter, double* x) {
    uint32_t* deg = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    double* y = (double*)malloc((n ? n : 1) * sizeof(double));
    double* c = (double*)malloc((n ? n : 1) * sizeof(double));
    for (uint64_t e = 0; e < m; ++e) deg[src[e]]++;
    for (uint32_t v = 0; v < n; ++v) x[v] = 1.0 - damping;
    int64_t it = 0;
    while ((uint64_t)it < max_iter) {
        ++it;
        for (uint32_t v = 0; v < n; ++v) {
            y[v] = 0.0;
            c[v] = deg[v] ? x[v] / (double)deg[v] : 0.0;
        }
        for (uint64_t e = 0; e < m; ++e) y[dst[e]] += c[src[e]];
        double diff = 0.0, norm = 0.0;
        for (uint32_t v = 0; v < n; ++v) {
            const double nx = (1.0 - damping) + damping * y[v];
            diff += nx > x[v] ? nx - x[v] : x[v] - nx;
            norm += nx;
            x[v] = nx;
        }
        if (diff <= tol * norm) break;
    }
    free(deg);
    free(y);
    free(c);
    return it;
}

/* ------------------------------------------------------------------ personalised PageRank (FP64) */
static double* orc_out_sums(uint32_t n, uint64_t m, const uint32_t* src, const double* w) {
    double* s = (double*)calloc(n ? n : 1, sizeof(double));
    for (uint64_t e = 0; e < m; ++e) s[src[e]] += w[e];
    return s;
}

int64_t orc_ppr_solve(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const double* w, uint32_t C,
                      const double* b, double scale_b, int transpose, double damping, double tol, uint64_t max_iter,
                      double* y) {
    const size_t N = (size_t)n * C;
    double* s = orc_out_sums(n, m, src, w);
    double* z = (double*)malloc((N ? N : 1) * sizeof(double));
    for (size_t i = 0; i < N; ++i) y[i] = scale_b * b[i];
    int64_t it = 0;
    int converged = 0;
    while ((uint64_t)it < max_iter) {
        ++it;
        for (size_t i = 0; i < N; ++i) z[i] = scale_b * b[i];
        for (uint64_t e = 0; e < m; ++e) {
            const uint32_t u = src[e], v = dst[e];
            if (s[u] == 0.0) continue;
            const double a = damping * (w[e] / s[u]);
            /* forward pushes u's row into v; the adjoint pulls v's row into u */
            const uint32_t from = transpose ? v : u, to = transpose ? u : v;
            const double* yr = y + (size_t)from * C;
            double* zr = z + (size_t)to * C;
            for (uint32_t k = 0; k < C; ++k) zr[k] += a * yr[k];
        }
        double diff = 0.0, norm = 0.0;
        for (size_t i = 0; i < N; ++i) {
            diff += fabs(z[i] - y[i]);
            norm += fabs(z[i]);
            y[i] = z[i];
        }
        if (damping / (1.0 - damping) * diff <= tol * norm) {
            converged = 1;
            break;
        }
    }
    free(z);
    free(s);
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
