/*
 * eegraph_c.h -- C ABI of the GB300-native EEGraph push-kernel library.
 *
 * Every entry point takes plain pointers and sizes, returns an eeg_status and never calls exit().
 * The C++ facade (include/eegraph.hpp) and the per-algorithm executables are built on top of it.
 *
 * Reference interfaces each group replaces (paths inside rwatling/EEGraph):
 *   loader            Graph::Graph / Graph::ReadGraph              src/graph.cpp:3-113, include/graph.hpp:28-50
 *   virtual graph     VirtualGraph::VirtualGraph / MakeGraph       src/virtual_graph.cpp:3-112, include/virtual_graph.hpp:8-26
 *                     UMVirtualGraph (managed-memory twin)          src/um_virtual_graph.cu:36-111
 *   runs              eegraph_{bfs,sssp,sswp,cc,pr}[_um]            include/eegraph.cuh:21-39, src/eegraph.cu
 *                     (+ the host do/while loop around the kernels src/eegraph.cu:89-211)
 *   kernels           {bfs,sssp,sswp,cc,pr}::{sync,async}_push_{td,dd} src/{bfs,sssp,sswp,cc,pr}.cu
 *                     clearLabel/mixLabels/moveUpLabels/sumLabels   src/gpu_utils.cu:3-34 (fused)
 *   energy            nvmlClass                                     include/nvmlClass.cuh:77-356
 *   errors            gpuErrorcheck -> exit(code)                   include/gpu_error_check.cuh:8-16
 */
#ifndef EEGRAPH_C_H
#define EEGRAPH_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define EEG_API __attribute__((visibility("default")))
#else
#define EEG_API
#endif

/* ------------------------------------------------------------------ status / enums */

typedef enum eeg_status {
    EEG_OK = 0,
    EEG_ERR_INVALID = 1,      /* bad argument (null pointer, source out of range, unknown algo ...) */
    EEG_ERR_IO = 2,           /* file missing / unreadable / unrecognised extension                 */
    EEG_ERR_CUDA = 3,         /* a CUDA runtime call failed (message in eeg_last_error())            */
    EEG_ERR_NOMEM = 4,        /* device or host allocation failed                                    */
    EEG_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up (grid barrier)                   */
    EEG_ERR_ITER_CAP = 6,     /* the iteration cap was reached before the fixed point                */
    EEG_ERR_UNSUPPORTED = 7,  /* combination not available (e.g. K not in {4,8,16})                  */
    EEG_ERR_NO_DEVICE = 8,    /* no CUDA device visible                                              */
    EEG_ERR_ENERGY = 9        /* NVML could not be started: energy unavailable                       */
} eeg_status;

/* Algorithms of the reference (one executable / eegraph_<algo> each). */
typedef enum eeg_algo {
    EEG_BFS = 0,
    EEG_SSSP = 1,
    EEG_SSWP = 2,
    EEG_CC = 3,  /* the reference's min-plus label propagation: label(v)=min(v, min_u label(u)+w(u,v)) */
    EEG_PR = 4
} eeg_algo;

/* Same numbering as the reference's `enum Variant` (include/globals.hpp:36-41). */
typedef enum eeg_variant {
    EEG_ASYNC_PUSH_TD = 0,
    EEG_ASYNC_PUSH_DD = 1,
    EEG_SYNC_PUSH_TD = 2,
    EEG_SYNC_PUSH_DD = 3
} eeg_variant;

/* Reference constants (include/globals.hpp:30-32). */
#define EEG_DIST_INFINITY 4294967294u /* UINT_MAX - 1 */
#define EEG_DEFAULT_K 8u              /* Part_Size */

/* ------------------------------------------------------------------ errors / device */

/* Human-readable text for a status code (static storage). */
EEG_API const char* eeg_status_string(eeg_status s);
/* Detail of the last error raised on the calling thread (thread-local, "" if none). */
EEG_API const char* eeg_last_error(void);
/* Library version string. */
EEG_API const char* eeg_version(void);
/* Number of visible CUDA devices (0 when none); never fails. */
EEG_API int eeg_device_count(void);
/* Select the device used by the calling thread (reference: --device -> cudaSetDevice). */
EEG_API eeg_status eeg_set_device(int device);
/* Managed (unified) memory for the --um path (reference: cudaMallocManaged in src/um_graph.cu). */
EEG_API eeg_status eeg_managed_alloc(size_t bytes, void** out);
EEG_API void eeg_managed_free(void* p);

/* ------------------------------------------------------------------ host edge list (Graph) */

/* Host edge list produced by the loader or from caller arrays. Replaces `Graph`
 * (include/graph.hpp:28-50). Ids are stored as read; has_zero_id tells whether the file is
 * 0-based (otherwise the virtual-graph build shifts every id down by one, as
 * VirtualGraph::VirtualGraph does at src/virtual_graph.cpp:5-12). */
typedef struct eeg_graph eeg_graph;

typedef struct eeg_graph_view {
    uint32_t num_nodes;      /* max id (+1 when an id 0 exists) -- src/graph.cpp:102-105 */
    uint64_t num_edges;
    int has_zero_id;
    int is_weighted;
    const uint32_t* src;     /* num_edges source ids (as read) */
    const uint32_t* dst;     /* num_edges destination ids (as read) */
    const uint32_t* weight;  /* num_edges weights (1 when the column is absent); NULL if unweighted */
} eeg_graph_view;

/* Parse a text edge list (.edges .el .wel .txt .edgelist) with the rules of
 * Graph::ReadGraph (src/graph.cpp:35-105): lines whose first character is not a digit are
 * skipped, the third column is the weight (1 when absent), extra columns are ignored. Binary
 * .bcsr/.bwcsr files (Subway's CSR format) are read too. n_threads<=0 picks the hardware count. */
EEG_API eeg_status eeg_graph_load(const char* path, int weighted, int n_threads, eeg_graph** out);
/* Wrap caller arrays (copied). ids are taken as 0-based; weight may be NULL (all 1). */
EEG_API eeg_status eeg_graph_from_arrays(uint32_t num_nodes, uint64_t num_edges, const uint32_t* src,
                                         const uint32_t* dst, const uint32_t* weight, eeg_graph** out);
EEG_API eeg_status eeg_graph_view_get(const eeg_graph* g, eeg_graph_view* out);
/* Ids after the reference's 1-based -> 0-based normalisation (what the kernels see). */
EEG_API eeg_status eeg_graph_normalized_ids(const eeg_graph* g, uint32_t* src_out, uint32_t* dst_out);
EEG_API void eeg_graph_destroy(eeg_graph* g);

/* Write a binary CSR file in Subway's .bcsr (unweighted) / .bwcsr (weighted) layout. */
EEG_API eeg_status eeg_graph_save_bcsr(const eeg_graph* g, const char* path);

/* ------------------------------------------------------------------ synthetic inputs */

/* R-MAT edge generator (Graph500 quadrant recursion, counter-based RNG: deterministic,
 * independent of thread count). Writes m = edge_factor << scale edges into caller arrays;
 * weights uniform in [wmin, wmax] (weight may be NULL). Ids are 0-based, not permuted;
 * duplicates and self-loops are kept. */
EEG_API eeg_status eeg_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                                uint64_t seed, uint32_t wmin, uint32_t wmax, uint32_t* src, uint32_t* dst,
                                uint32_t* weight);
/* 2-D grid road-like graph: side x side vertices, 4-neighbour undirected (both arcs stored),
 * each undirected edge deleted with probability p_delete, plus round(shortcut_frac * #grid edges)
 * random undirected long-range shortcuts; weights uniform in [wmin, wmax].
 * Call with src == NULL to obtain the arc count in *num_arcs first. */
EEG_API eeg_status eeg_gen_grid(uint32_t side, double p_delete, double shortcut_frac, uint64_t seed,
                                uint32_t wmin, uint32_t wmax, uint64_t* num_arcs, uint32_t* src,
                                uint32_t* dst, uint32_t* weight);
/* Symmetrise an arc list: out = in + reversed(in) (2*m arcs, caller arrays). */
EEG_API eeg_status eeg_symmetrize(uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w,
                                  uint32_t* src_out, uint32_t* dst_out, uint32_t* w_out);

/* ------------------------------------------------------------------ device virtual graph */

/* K-bounded virtual graph resident in HBM (replaces VirtualGraph / UMVirtualGraph).
 * Layout: vertex v owns parts vstart[v] .. vstart[v+1]-1, part p holds up to K consecutive
 * out-edges of vowner[p] in vcol[p*K .. p*K+K) (unused slots = 0xFFFFFFFF) and their weights
 * in vw[]. Lossless: every edge is kept (the reference drops edges, src/virtual_graph.cpp:86-88). */
typedef struct eeg_vgraph eeg_vgraph;

enum {
    EEG_VG_REVERSE = 1u << 0,   /* also build the in-edge (transposed) virtual graph (PageRank pull) */
    EEG_VG_MANAGED = 1u << 1,   /* allocate in managed memory (the --um path) */
    EEG_VG_INPUT_DEVICE = 1u << 2, /* src/dst/weight pointers are device (or managed) pointers */
    EEG_VG_SHIFT_ONE = 1u << 3, /* subtract 1 from every id while building (1-based input) */
    EEG_VG_EDGE_IDS = 1u << 4,  /* keep each slot's input edge index (per-edge results in input order;
                                   needed by eeg_ppr_create) */
    EEG_VG_SYMMETRIC = 1u << 5, /* the caller guarantees an undirected edge list (every arc's reverse is
                                   present with the same weight): the forward graph doubles as the
                                   transposed one, so PageRank runs without a second build. Ignored with
                                   REVERSE; not usable by eeg_ppr_create (needs the transposed edge ids). */
    EEG_VG_SYMMETRIZE = 1u << 6, /* insert every input edge in both directions: the arcs are the input
                                   followed by its reverse, as eeg_symmetrize lays them out (so the graph
                                   is the one built from eeg_symmetrize's output), without that host-side
                                   copy. Implies EEG_VG_SYMMETRIC. num_edges counts input edges; the graph
                                   has twice as many arcs, and with EEG_VG_EDGE_IDS the reverse of input
                                   edge e has index num_edges + e. */
    EEG_VG_REVERSE_ONLY = 1u << 7 /* build only what PageRank reads: the transposed graph and the
                                   out-degrees (implies EEG_VG_REVERSE). The forward parts are not
                                   built, so the traversals, eeg_batch_create, eeg_ppr_create and
                                   eeg_vgraph_download refuse such a graph (EEG_ERR_INVALID). */
};

typedef struct eeg_vgraph_info {
    uint32_t num_nodes;
    uint64_t num_edges;
    uint32_t K;
    uint64_t num_parts;        /* sum_v ceil(outdeg(v)/K) -- numParts of the reference */
    uint64_t num_rparts;       /* parts of the transposed graph (0 when not built) */
    uint32_t max_out_degree;
    uint32_t max_degree_vertex; /* lowest id with the largest out-degree */
    uint64_t device_bytes;     /* HBM held by the graph */
    float build_ms;            /* device time of the last build (CUDA events) */
} eeg_vgraph_info;

/* Build from a host edge list. The build runs on the GPU (degree histogram, part-count
 * scan, scatter into the part-major layout, owner table by max-scan). `stream` is a
 * cudaStream_t (NULL = legacy default stream). */
EEG_API eeg_status eeg_vgraph_build(const eeg_graph* g, uint32_t K, uint32_t flags, void* stream, eeg_vgraph** out);
/* Build from raw arrays (host or, with EEG_VG_INPUT_DEVICE, device pointers); weight may be NULL. */
EEG_API eeg_status eeg_vgraph_build_arrays(uint32_t num_nodes, uint64_t num_edges, const uint32_t* src,
                                           const uint32_t* dst, const uint32_t* weight, uint32_t K,
                                           uint32_t flags, void* stream, eeg_vgraph** out);
EEG_API eeg_status eeg_vgraph_get_info(const eeg_vgraph* vg, eeg_vgraph_info* out);
/* Copy the device arrays back (any pointer may be NULL to skip it). Sizes: vstart n+1,
 * vowner num_parts, vcol/vw num_parts*K, outdeg n. */
EEG_API eeg_status eeg_vgraph_download(const eeg_vgraph* vg, uint32_t* vstart, uint32_t* vowner, uint32_t* vcol,
                                       uint32_t* vw, uint32_t* outdeg);
/* Export the reference's host layout (src/virtual_graph.cpp:36-112, but lossless):
 * nodePointer[n], edgeList[2m+n] = per vertex [deg, (t0,w0), (t1,w1) ...],
 * partNodePointer[2*numParts] = {node, part} pairs. Any pointer may be NULL. */
EEG_API eeg_status eeg_vgraph_export_reference_layout(const eeg_vgraph* vg, uint32_t* nodePointer,
                                                      uint32_t* edgeList, uint32_t* partNodePointer);
EEG_API void eeg_vgraph_destroy(eeg_vgraph* vg);

/* ------------------------------------------------------------------ runs */

typedef struct eeg_options {
    uint32_t max_iterations;  /* 0 = default cap (n+2 for traversals, 10000 for PageRank) */
    float pr_tolerance;       /* PageRank stop: bound on ||x - x*||_1 / ||x||_1 (0 = 1e-7) */
    float pr_damping;         /* 0 = 0.85 (src/pr.cu:43) */
    float pr_accuracy;        /* DD PageRank activation threshold on |delta| (0 = derived from tolerance) */
    uint32_t block_size;      /* 0 = 512 threads per CTA */
    uint32_t blocks_per_sm;   /* 0 = as many as occupancy allows */
    uint32_t record_activity; /* 1: store active-vertex counts per iteration (reference --activity) */
    uint32_t timeout_ms;      /* bound on any device-side wait (0 = 10000 ms) */
    uint32_t host_loop;       /* traversals: 1 = one launch per round with a host round trip in between,
                                 as the reference's do { H2D flag; launch; sync; D2H flag } while loop
                                 (src/eegraph.cu:89-211) -- for comparison; 0 = one persistent launch */
    uint32_t pr_hot_limit;    /* PageRank: at most this many of the highest out-degree vertices have their
                                 contributions staged in shared memory each sweep (0 = 32768; 1 = none) */
    uint32_t delta;           /* SSSP / SSWP with SYNC_PUSH_DD: bucketed rounds of this key width -- a vertex
                                 whose distance (SSSP) or INF - width (SSWP) is not below the current
                                 threshold waits until the frontier runs empty (0 = plain rounds). Same
                                 results; far fewer rescans on high-diameter graphs. */
    uint32_t cc_components;   /* CC: 1 = connected components, relaxing with weight 0 instead of the edge
                                 weight, so label(v) = the smallest id in v's component when every vertex
                                 is seeded (ASYNC_* and SYNC_PUSH_TD) -- an extension, not the reference's
                                 min-plus labels (0, the default) */
    uint32_t timeout_us;      /* bound on any device-side wait in microseconds; when nonzero it replaces
                                 timeout_ms (sub-millisecond limits). A wait that runs out makes every CTA
                                 leave and the call return EEG_ERR_TIMEOUT; the handle stays usable. */
    uint32_t bfs_push_only;   /* BFS (SYNC_PUSH_DD): 1 = push rounds only; 0 = pull (bottom-up) rounds while the
                                 frontier is large, when the graph has its transposed parts (EEG_VG_REVERSE);
                                 the same levels either way */
    uint32_t reserved[2];
} eeg_options;

typedef struct eeg_result {
    float kernel_ms;            /* CUDA-event time of the device work (init + persistent loop) */
    uint32_t iterations;        /* rounds of the persistent loop (PageRank: sweeps) */
    uint64_t reached_vertices;  /* n_r: vertices with a final value != initial "unreached" value */
    uint64_t reached_edges;     /* m_r: out-edges of reached vertices (Graph500 TEPS count) */
    uint64_t parts_processed;   /* virtual nodes expanded over the whole run */
    uint64_t edges_scanned;     /* edge slots read over the whole run (redundant work included) */
    uint64_t updates;           /* successful atomic improvements */
    double algorithmic_bytes;   /* work-minimal byte count (12 n_r + (12|8) m_r; PR: sweeps*(12n+8m)) */
    double gteps;               /* m_r / kernel time (PR: sweeps * m / time) */
    double pr_residual;         /* PageRank: last ||x_{k+1}-x_k||_1 (FP64) */
    double pr_l1_norm;          /* PageRank: ||x||_1 (FP64) */
    uint32_t num_activity;      /* entries written to activity[] */
    uint32_t launches;          /* kernels this call launched (persistent kernel + set-up/statistics) */
    uint32_t partitions;        /* streamed runs (eeg_stream_run): partitions gathered over all rounds */
    uint32_t pull_rounds;       /* BFS: rounds that pulled over the transposed parts (the rest pushed) */
    uint32_t reserved[4];
} eeg_result;

/* Default options (all zero fields -> defaults). */
EEG_API void eeg_options_init(eeg_options* o);

/* One run of `algo` / `variant` on a device virtual graph.
 *  source      start vertex (ignored by PageRank; by CC except for SYNC_PUSH_DD, which seeds only it
 *              -- src/eegraph.cu:548-553)
 *  out         caller-owned result array of num_nodes entries: uint32 for BFS/SSSP/SSWP/CC,
 *              float for PageRank; host memory unless out_on_device != 0
 *  activity    optional (may be NULL) host array of `activity_cap` uint32 receiving the number of
 *              active vertices per iteration (the reference's --activity sumLabels vector)
 * Results: BFS hop levels, SSSP Dijkstra distances, SSWP widest-path values, CC min-plus labels,
 * unreached = EEG_DIST_INFINITY (SSWP: 0, source = EEG_DIST_INFINITY). Every variant and K gives the
 * same integer array. */
EEG_API eeg_status eeg_run(eeg_vgraph* vg, eeg_algo algo, eeg_variant variant, uint32_t source,
                           const eeg_options* opts, void* out, int out_on_device, uint32_t* activity,
                           uint32_t activity_cap, void* stream, eeg_result* res);

/* ------------------------------------------------------------------ batched queries */

/* Many BFS/SSSP/SSWP queries over many device virtual graphs in ONE launch. No counterpart in the
 * reference, which runs each query as a separate eegraph_<algo> call (src/main.cu:74-281).
 * A persistent kernel made of thread-block clusters takes queries from a device work queue (largest
 * graphs first) and runs each traversal on one cluster (rounds separated by the hardware cluster
 * barrier); the launch is captured once in a CUDA graph and replayed by eeg_batch_run. Results equal
 * eeg_run's for the same (graph, algorithm, source). Graphs must stay alive while the batch is used. */
typedef struct eeg_batch eeg_batch;
typedef struct eeg_query {
    uint32_t graph;    /* index into the graphs given to eeg_batch_create */
    uint32_t algo;     /* EEG_BFS, EEG_SSSP or EEG_SSWP */
    uint32_t source;
    uint32_t reserved;
} eeg_query;
EEG_API eeg_status eeg_batch_create(eeg_vgraph* const* graphs, uint32_t num_graphs, eeg_batch** out);
/* Set the queries; *out_words receives the output size: query i writes num_nodes(graph_i) uint32 values
 * at eeg_batch_query_offset(i) (queries laid out in the given order). cluster_size: CTAs per query
 * (1, 2, 4 or 8; 0 = 4). */
EEG_API eeg_status eeg_batch_set_queries(eeg_batch* b, const eeg_query* queries, uint32_t num_queries,
                                         uint32_t cluster_size, unsigned long long* out_words);
EEG_API eeg_status eeg_batch_query_offset(const eeg_batch* b, uint32_t query, unsigned long long* offset);
/* Run every query (device output arena `out`); ordered after `stream`; *ms = device time of the launch. */
EEG_API eeg_status eeg_batch_run(eeg_batch* b, uint32_t* out, void* stream, float* ms);
/* Rounds each query took (num_queries entries, query order). */
EEG_API eeg_status eeg_batch_rounds(const eeg_batch* b, uint32_t* rounds);
/* Per query (query order) of the last run: device start and end time (ns, global timer) and the
 * index of the cluster that ran it (~0 for a whole-grid query) -- 3 values per query. */
EEG_API eeg_status eeg_batch_query_times(const eeg_batch* b, unsigned long long* times);
/* The first `count` queries in size order (largest graphs first) run one after another on the whole
 * grid before the rest are spread over the clusters (0 = none; the default). That phase waits at a
 * grid-wide barrier, so it needs every CTA of the launch resident at once: with kernels of other
 * streams holding SMs, some CTAs may not start, the wait gives up after 1 s, and eeg_batch_run then
 * runs the batch once more with every query on the clusters (correct results, slower; *ms covers
 * that second launch). Give the batch the device to itself when using this phase. */
EEG_API eeg_status eeg_batch_set_grid_queries(eeg_batch* b, uint32_t count);
EEG_API eeg_status eeg_batch_get_config(const eeg_batch* b, uint32_t* cluster_size, uint32_t* grid_queries);
/* Autotuner: time the batch with 1, 2, 4 and 8 CTAs per query, each with 0, 1, 2, 4 ... 64 whole-grid
 * queries, and keep the fastest pair (eeg_batch_get_config reports it). */
EEG_API eeg_status eeg_batch_autotune(eeg_batch* b, uint32_t* out, uint32_t* chosen_cluster_size, float* best_ms);
EEG_API void eeg_batch_destroy(eeg_batch* b);

/* Autotuner for the part size: builds the graph with K = 4, 8 and 16, times BFS and SSSP from the
 * highest-out-degree vertex (median of `reps`), and returns the fastest K; ms_per_k (may be NULL)
 * receives the three times. Results are cached per (num_nodes, num_edges, max out-degree). Host arrays. */
EEG_API eeg_status eeg_autotune_k(uint32_t num_nodes, uint64_t num_edges, const uint32_t* src, const uint32_t* dst,
                                  const uint32_t* weight, uint32_t reps, uint32_t* best_k, float* ms_per_k);

/* Autotuner per graph and algorithm (no counterpart in the reference): for K in {4, 8, 16} and every
 * variant whose fixed point equals the default's -- all four for BFS, SSSP, SSWP and PageRank; for CC
 * all but SYNC_PUSH_DD, whose source-seeded fixed point differs -- build the graph (PageRank: its
 * transposed graph only), run from the highest-out-degree vertex, one warm-up then `reps` runs, and
 * keep the median kernel time. ms_table[k_index * 4 + variant] (k_index 0, 1, 2 for K = 4, 8, 16) holds
 * the medians, -1 where a variant is not tried. Then, for the chosen (K, variant), the number of
 * resident CTAs per SM: 1 or 2 for the traversal kernels (384 or 512 threads each, so 384-1024 threads
 * per SM) and the data-driven PageRank kernel (512 threads), 1 for the pull PageRank kernel (its
 * 1024-thread CTA fills an SM); ms_per_blocks[b-1] holds the median at b CTAs per SM (-1 where not
 * possible) and blocks_per_sm the faster one -- pass it as eeg_options.blocks_per_sm. The threads per
 * CTA are fixed per kernel by its register budget (measured best), and the split of hub vertices is K
 * itself: a vertex of more than K out-edges becomes several parts, expanded by as many threads, instead
 * of being handed to a warp or a CTA past a degree threshold. Host arrays. */
typedef struct eeg_tuning {
    uint32_t K;
    eeg_variant variant;
    float ms;
    float ms_table[12];
    uint32_t blocks_per_sm;
    float ms_per_blocks[2];
} eeg_tuning;
EEG_API eeg_status eeg_autotune(uint32_t num_nodes, uint64_t num_edges, const uint32_t* src, const uint32_t* dst,
                                const uint32_t* weight, eeg_algo algo, uint32_t reps, eeg_tuning* out);

/* Allocation-free traversal run. No counterpart in the reference: it exists for callers that cannot
 * allocate device memory when they run a query -- plugins whose host application owns all GPU memory,
 * frameworks that route every allocation through their own pool, service loops where cudaMalloc's
 * possible device synchronisation is not allowed. The caller passes the virtual graph (the layout of
 * eeg_vgraph_download: vstart[n+1], vowner[P], vcol/vw[P*K]; vw may be NULL for BFS) and the output
 * dist[n], all in device memory it owns; the working memory (control block, part queues, round stamps)
 * lives in one fixed device array of EEG_NOALLOC_SCRATCH_BYTES that every GPU loading this library
 * holds until the process exits. The call allocates nothing (no cudaMalloc/cudaFree, no allocating
 * library routine). It rejects graphs whose working memory, 256 + 4*(2*P + n) bytes rounded up to
 * 256-byte blocks, exceeds the array (EEG_ERR_INVALID). The first call on a device looks up the array's
 * address (cudaGetSymbolAddress) -- make that first call before any stream capture. All calls on a device
 * share the array: calls that overlap on the GPU (unordered streams or threads) race and must be
 * serialised by the caller. Results equal eeg_run's with default eeg_options (there are none to pass:
 * CC reads the weights, the round cap is n + 2, every device wait is bounded by 10 s, no bucketed rounds);
 * *iterations (may be NULL) receives the rounds. */
#define EEG_NOALLOC_SCRATCH_BYTES (32u << 20)
EEG_API eeg_status eeg_run_noalloc(eeg_algo algo, eeg_variant variant, uint32_t num_nodes, uint64_t num_parts,
                                   uint32_t K, const uint32_t* vstart, const uint32_t* vowner, const uint32_t* vcol,
                                   const uint32_t* vw, uint32_t source, uint32_t* dist, void* stream,
                                   uint32_t* iterations);

/* ------------------------------------------------------------------ differentiable personalised PageRank */

/* Personalised PageRank with an implicit adjoint. No counterpart in the reference (its PageRank,
 * src/pr.cu:3-288, is unweighted, unpersonalised and not differentiable); it is a project-added form.
 * Model, per column k of row-major n x C arrays, with W_uv = w_uv / s_u the row-normalised raw edge
 * weights (s_u = sum of u's out-weights; a vertex with s_u == 0 has no out-flow):
 *     forward   X = (1-d) T + d W^T X            (x_v = (1-d) t_v + d sum_{u->v} W_uv x_u)
 *     adjoint   L = G + d W L                    (G = dLoss/dX)
 *     dLoss/dW_uv = d <X_u, L_v>,  dLoss/dw_uv = (dLoss/dW_uv - sum_v' dLoss/dW_uv' W_uv') / s_u,
 *     dLoss/dT = (1-d) L.
 * Both solves are Jacobi sweeps in one persistent launch each; the forward pulls over the transposed
 * graph, the adjoint over the forward graph (no atomics, no transpose at run time, no iterate storage).
 * FP32 values and accumulation; the stop test d/(1-d)*||Y_{k+1}-Y_k||_1 <= tol*||Y_{k+1}||_1 (all columns
 * together, eeg_options.pr_tolerance, default 1e-7) is reduced in FP64. C = 1 runs the single-column
 * kernels (the plain form); 2 <= C <= 64 runs the batched row kernels (rows padded to 32 columns for
 * C <= 32, else to 64). */
typedef struct eeg_ppr eeg_ppr;
/* vg must be built with EEG_VG_REVERSE | EEG_VG_EDGE_IDS and outlive the handle. */
EEG_API eeg_status eeg_ppr_create(eeg_vgraph* vg, uint32_t columns, eeg_ppr** out);
/* Raw edge weights w[num_edges] in input edge order (finite, >= 0), host or device memory. */
EEG_API eeg_status eeg_ppr_set_weights(eeg_ppr* p, const float* w, int on_device);
/* Forward solve. teleport: n x C (host, or device with in_on_device). x_out (may be NULL): n x C.
 * X is kept for the next eeg_ppr_adjoint. */
EEG_API eeg_status eeg_ppr_forward(eeg_ppr* p, const float* teleport, int in_on_device, float* x_out,
                                   int out_on_device, const eeg_options* opts, void* stream, eeg_result* res);
/* Adjoint solve for dl_dx (n x C) and the gradients, each output optional (NULL): dl_dteleport n x C,
 * dl_dw[num_edges] and dl_dwn[num_edges] (w.r.t. the raw and the normalised weights, input edge order).
 * accumulate != 0 adds the edge gradients to those of earlier adjoint calls on this handle (so a loop of
 * single-column calls returns the sum over columns); dl_dteleport is never accumulated. */
EEG_API eeg_status eeg_ppr_adjoint(eeg_ppr* p, const float* dl_dx, int in_on_device, float* dl_dteleport,
                                   float* dl_dw, float* dl_dwn, int out_on_device, int accumulate,
                                   const eeg_options* opts, void* stream, eeg_result* res);
EEG_API void eeg_ppr_destroy(eeg_ppr* p);

/* ------------------------------------------------------------------ graphs larger than device memory */

/* Active-subgraph streaming, the model of the Subway code vendored in the reference
 * (Subway/shared/subgraph_generator.cu:10-97 generates each round's active subgraph,
 * Subway/shared/partitioner.cu:12-91 cuts it into partitions of at most a quarter of device memory,
 * Subway/subway/{bfs,sssp,sswp,cc}-{sync,async}.cu run the rounds). The graph's CSR stays in
 * page-locked host memory mapped into the GPU; the device keeps O(num_nodes) state plus two partition
 * buffers within `device_budget_bytes` (0 = a quarter of the free device memory, as Subway). Each round,
 * the active vertices' out-edges, in K-bounded parts, are gathered by the GPU straight from host memory
 * into one buffer while the previous partition is relaxed from the other. Results equal eeg_run's (the
 * same fixed points) for any budget. A budget below two parts of K targets, K weights and an owner
 * (2*(8K+4) bytes) is rejected (EEG_ERR_INVALID); graphs of 2^32 or more virtual parts are unsupported. */
typedef struct eeg_stream eeg_stream;
typedef struct eeg_stream_info {
    uint32_t num_nodes;
    uint64_t num_edges;
    uint32_t K;
    uint32_t partition_parts;      /* parts one partition buffer holds */
    uint64_t device_budget_bytes;  /* bytes of the two partition buffers */
    uint64_t host_bytes;           /* page-locked host bytes of the CSR */
} eeg_stream_info;
/* Build the host CSR from a loaded edge list (1-based files shifted down by one) on the current device. */
EEG_API eeg_status eeg_stream_create(const eeg_graph* g, uint32_t K, uint64_t device_budget_bytes, eeg_stream** out);
EEG_API eeg_status eeg_stream_get_info(const eeg_stream* s, eeg_stream_info* out);
/* BFS, SSSP, SSWP or CC (every vertex seeded; cc_components honoured). SYNC_* variants relax each
 * partition once per round (Subway's *-sync); ASYNC_* variants also relax a partition again, from HBM,
 * while its own vertices keep improving (Subway's *-async). max_iterations caps the rounds.
 * out: num_nodes uint32 values, host memory unless out_on_device != 0. eeg_result: iterations =
 * rounds, parts_processed = parts streamed, edges_scanned = edges relaxed, partitions = partitions
 * gathered, kernel_ms = the whole streamed run (gathers included). */
EEG_API eeg_status eeg_stream_run(eeg_stream* s, eeg_algo algo, eeg_variant variant, uint32_t source,
                                  const eeg_options* opts, uint32_t* out, int out_on_device, void* stream,
                                  eeg_result* res);
EEG_API void eeg_stream_destroy(eeg_stream* s);

/* ------------------------------------------------------------------ energy (NVML) */

/* GPU energy over a region, from NVML's total-energy counter (mJ) with a power-sampling
 * fallback. NVML is loaded at run time; without it eeg_energy_begin returns EEG_ERR_ENERGY and
 * the caller reports "energy unavailable". csv_path may be NULL (no power trace). */
typedef struct eeg_energy eeg_energy;
EEG_API eeg_status eeg_energy_begin(int device, const char* csv_path, uint32_t sample_period_us, eeg_energy** out);
EEG_API eeg_status eeg_energy_mark(eeg_energy* e);
EEG_API eeg_status eeg_energy_end(eeg_energy* e, double* joules, double* seconds, double* avg_watts);
EEG_API void eeg_energy_destroy(eeg_energy* e);

#ifdef __cplusplus
}
#endif

#endif /* EEGRAPH_C_H */
