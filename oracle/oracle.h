/*
 * oracle.h -- CPU oracle for the EEGraph push-kernel path. TEST INFRASTRUCTURE ONLY: tests, the
 * smoke check and the bench's CPU baseline call it as the checker; the product never links it.
 *
 * Restates, in plain C, the reference's host-side algorithms (rwatling/EEGraph paths):
 *   orc_parse_*          Graph::ReadGraph text rules             src/graph.cpp:35-105
 *   orc_virtual_graph    VirtualGraph::MakeGraph layout           src/virtual_graph.cpp:36-112 (lossless)
 *   orc_seq_sweep        {bfs,sssp,sswp,cc}::seq_cpu(VirtualGraph) src/bfs.cu:275-320, src/sssp.cu:357-404,
 *                                                                 src/sswp.cu:273-320, src/cc.cu:329-376
 *   orc_frontier_sweep   the *_push_dd kernels run sequentially   src/sssp.cu:192-299, host loop
 *                                                                 src/eegraph.cu:89-211
 *   orc_dijkstra / orc_bfs / orc_widest / orc_pagerank: independent textbook algorithms that pin the
 *   fixed points (Dijkstra 1959; breadth-first search; max-min Dijkstra; power iteration in FP64).
 *   orc_ppr_*: FP64 personalised PageRank on row-normalised edge weights, its adjoint solve and the
 *   gradients (a project-added form: the reference has no counterpart, so these pin the GPU kernels
 *   by mathematics -- finite differences and the duality c^T x = (1-d) t^T lambda are checked in tests).
 * Parity pinned against the reference itself: oracle/_ref (built from the reference sources) and the
 * golden vectors in tests/golden/ that it produced.
 */
#ifndef EEG_ORACLE_H
#define EEG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_INF 4294967294u

enum { ORC_BFS = 0, ORC_SSSP = 1, ORC_SSWP = 2, ORC_CC = 3 };

/* text edge-list parse, two calls: counts first, then fill (arrays of num_edges) */
int orc_parse_count(const char* path, uint64_t* num_edges, uint32_t* num_nodes, int* has_zero_id);
int orc_parse_fill(const char* path, int weighted, uint32_t* src, uint32_t* dst, uint32_t* w);

/* number of parts = sum_v ceil(outdeg(v)/K) over 0-based edges */
uint64_t orc_num_parts(uint32_t n, uint64_t m, const uint32_t* src, uint32_t K);
/* reference layout (lossless): nodePointer[n], edgeList[2m+n], partNodePointer[2*numParts] */
void orc_virtual_graph(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w,
                       uint32_t K, uint32_t* nodePointer, uint32_t* edgeList, uint32_t* partNodePointer);

/* initial values per the reference drivers: BFS/SSSP src=0 else INF; SSWP src=INF else 0; CC v */
void orc_init_values(int algo, uint32_t n, uint32_t source, uint32_t* dist);

/* Topology-driven sweeps over parts in order (the reference's seq_cpu). wrap != 0 keeps uint32 wrap
 * of INF+w exactly as the reference; wrap == 0 skips unreached sources (the parity contract).
 * dist must hold the initial values. Returns the number of sweeps, or -1 if max_sweeps is hit. */
int64_t orc_seq_sweep(int algo, uint32_t n, uint64_t num_parts, const uint32_t* nodePointer, const uint32_t* edgeList,
                      const uint32_t* partNodePointer, uint32_t K, int wrap, uint64_t max_sweeps, uint32_t* dist);

/* Data-driven rounds (sync_push_dd / async_push_dd semantics), sequential: label1 = active set
 * (all vertices when seed_all, else {source}), in-place relaxation, improved targets -> label2. */
int64_t orc_frontier_sweep(int algo, uint32_t n, uint64_t num_parts, const uint32_t* nodePointer,
                           const uint32_t* edgeList, const uint32_t* partNodePointer, uint32_t K, int seed_all,
                           uint32_t source, uint32_t* dist);

/* independent oracles over a 0-based edge list */
void orc_bfs(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, uint32_t source, uint32_t* dist);
void orc_dijkstra(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w,
                  uint32_t source, uint32_t* dist);
void orc_widest(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w,
                uint32_t source, uint32_t* out);
/* min-plus label fixed point label(v) = min(v, min_u label(u)+w(u,v)), all vertices seeded
 * (multi-source Dijkstra with source distances = ids) */
void orc_cc_labels(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w, uint32_t* out);

/* FP64 PageRank: x = (1-d) + d * A^T D^-1 x (dangling mass dropped), power iteration until
 * ||x_{k+1}-x_k||_1 <= tol * ||x||_1. Returns iterations. */
int64_t orc_pagerank(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, double damping, double tol,
                     uint64_t max_iter, double* x);

/* Personalised PageRank on row-normalised weights W_e = w_e / s_src(e), s_u = sum of w over u's
 * out-edges (W = 0 where s_u == 0). C columns, row-major n x C arrays.
 *   forward : X = (1-d) T + d W^T X        (x_v = (1-d) t_v + d sum_{e: u->v} W_e x_u)
 *   adjoint : L = G + d W L                (l_u = g_u + d sum_{e: u->v} W_e l_v), G = dLoss/dX
 * Jacobi in FP64 until d/(1-d) * ||Y_{k+1}-Y_k||_1 <= tol * ||Y_{k+1}||_1 (all columns together).
 * Returns the sweeps taken, or -1 when max_iter was reached first. */
int64_t orc_ppr_solve(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const double* w, uint32_t C,
                      const double* b, double scale_b, int transpose, double damping, double tol, uint64_t max_iter,
                      double* y);
/* Gradients from X and L: gWn_e = d <X_src(e), L_dst(e)> (w.r.t. the normalised weight),
 * gw_e = (gWn_e - sum_{e' out of src(e)} gWn_e' W_e') / s_src(e) (w.r.t. the raw weight; 0 where s == 0),
 * gT = (1-d) L. Any output may be NULL. */
void orc_ppr_grads(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const double* w, uint32_t C,
                   const double* X, const double* L, double damping, double* gWn, double* gw, double* gT);

/* Threaded forms of the two FP64 solvers (OpenMP where the oracle was built with it; the same result
 * for every thread count: fixed sum orders). The plain forms above are these with one thread. */
int64_t orc_pagerank_mt(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, double damping, double tol,
                        uint64_t max_iter, int threads, double* x);
/* PageRank in two steps: the in-edge CSR (sources grouped by target in input order, off[n+1]) and
 * out-degrees once, then the pull sweeps on it (orc_pagerank_mt is the two in a row). */
void orc_in_csr(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, uint64_t* off, uint32_t* isrc,
                uint32_t* outdeg);
int64_t orc_pagerank_pull(uint32_t n, const uint64_t* off, const uint32_t* isrc, const uint32_t* outdeg,
                          double damping, double tol, uint64_t max_iter, int threads, double* x);
int64_t orc_ppr_solve_mt(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const double* w,
                         uint32_t C, const double* b, double scale_b, int transpose, double damping, double tol,
                         uint64_t max_iter, int threads, double* y);

/* Seeded synthetic inputs (the benchmark's R-MAT and road-like grid), identical to the product
 * library's generators so CPU-only callers need not load it. Grid: call with src == NULL for the arc
 * count first. Return 0, or -1 on invalid parameters. */
int orc_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed, uint32_t wmin,
                 uint32_t wmax, int threads, uint32_t* src, uint32_t* dst, uint32_t* weight);
int orc_gen_grid(uint32_t side, double p_delete, double shortcut_frac, uint64_t seed, uint32_t wmin, uint32_t wmax,
                 int threads, uint64_t* num_arcs, uint32_t* src, uint32_t* dst, uint32_t* weight);
void orc_symmetrize(uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w, uint32_t* so,
                    uint32_t* d_o, uint32_t* wo);

#ifdef __cplusplus
}
#endif

#endif
