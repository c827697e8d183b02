// internal.hpp -- handle layouts shared by the C ABI implementation and the kernel launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

// Shared-memory carveout hint for a kernel with static shared memory only: the smallest share of the
// SM's unified L1/shared storage that holds `ctas` CTAs (each also takes 1 KB the system reserves), so
// the rest stays L1.
template <typename F>
inline eeg_status prefer_l1(F kern, int ctas, int device) {
    cudaFuncAttributes fa;
    EEG_CUDA(cudaFuncGetAttributes(&fa, (const void*)kern));
    int smem_sm = 0;
    EEG_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device));
    if (smem_sm <= 0) return EEG_OK;
    const long long need = (long long)ctas * ((long long)fa.sharedSizeBytes + 1024);
    const int pct = (int)std::min<long long>(100, (need * 100 + smem_sm - 1) / smem_sm);
    EEG_CUDA(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
    return EEG_OK;
}

// Host edge list (the reference's Graph: src/graph.cpp, include/graph.hpp:28-50).
struct eeg_graph {
    uint32_t num_nodes = 0;
    uint64_t num_edges = 0;
    bool has_zero_id = false;
    bool is_weighted = false;
    std::vector<uint32_t> src, dst, weight;
};

namespace eeg {

// One K-bounded virtual graph (forward, or transposed for pull kernels) in HBM.
struct VDir {
    uint64_t P = 0;               // number of parts
    uint32_t* vstart = nullptr;   // n+1: first part of each vertex
    uint32_t* vowner = nullptr;   // P: owning vertex of each part
    uint32_t* vcol = nullptr;     // P*K: neighbour ids (NO_EDGE padding)
    uint32_t* vw = nullptr;       // P*K: weights (uint32; float bits for PageRank weights) or null
    uint32_t* veid = nullptr;     // P*K: input edge index of each slot (EEG_VG_EDGE_IDS) or null
    uint32_t* deg = nullptr;      // n: degree in this direction
};

// Control block of the traversal kernel (device memory).
struct TravCtrl {
    BarrierWords bw;
    uint32_t qparts[3];   // parts enqueued per round (rotating; TD: improvement flag)
    uint32_t qverts[3];   // vertices enqueued per round (rotating)
    uint32_t iterations;
    uint32_t done;        // the traversal reached its end (fixed point, cap or abort)
    unsigned long long parts_processed;
    unsigned long long edges_scanned;
    unsigned long long updates;
    // bucketed SSSP/SSWP rounds
    uint32_t fcnt[3];   // far-pile lengths (three piles rotate)
    uint32_t fmin[3];   // smallest key recorded in each pile
    uint32_t fcsel[2];  // per round parity: the pile receiving far claims
    uint32_t tsel[2];   // per round parity: the threshold T
    // BFS pull rounds: length of the list of vertices each pull round left unreached (rotating)
    uint32_t lcnt[3];
    uint32_t pull_rounds;
};

// Control block of the PageRank kernels.
struct PRCtrl {
    BarrierWords bw;
    double resid[3];     // ||x_{k+1}-x_k||_1 per sweep (rotating)
    double norm[3];      // ||x_{k+1}||_1 per sweep (rotating)
    uint32_t iterations;
    uint32_t pad;
    double last_resid;
    double last_norm;
    unsigned long long edges_scanned;
    unsigned long long zero_in;  // vertices without in-edges (value stays 1-d)
};

// Control block of the data-driven PageRank kernel (residual frontier).
struct PRDDCtrl {
    BarrierWords bw;
    uint32_t plen[3];    // part-queue lengths per round (rotating)
    uint32_t iterations;
    uint32_t pad;
    unsigned long long pushes;    // edge pushes over the run
    unsigned long long parts;     // parts expanded over the run
    unsigned long long consumed;  // residuals taken (vertex activations) over the run
    double resid;        // sum of the residuals left at the end (error bound: resid / (1-d))
    double norm;         // sum of the values at the end
};

struct Workspace {
    // traversal
    uint32_t* dist = nullptr;     // n
    uint32_t* q[2] = {nullptr, nullptr};  // P each
    uint32_t* stamp = nullptr;    // n
    uint32_t* pushed = nullptr;   // P: the owner value each part last pushed with (DD rounds)
    uint32_t* plist = nullptr;    // 2n: BFS pull rounds' lists of vertices left unreached (two alternate)
    uint32_t* far = nullptr;      // 4n: three far piles and the far flags (bucketed rounds)
    uint32_t* activity = nullptr; // device copy of the activity vector
    uint32_t activity_cap = 0;
    TravCtrl* tctrl = nullptr;
    // PageRank
    float* x = nullptr;           // n
    float* contrib[2] = {nullptr, nullptr};  // n each
    double* acc = nullptr;        // n (partials of vertices whose parts cross warp chunks)
    uint32_t* arrive = nullptr;   // n (chunks that delivered a partial, per vertex)
    uint32_t* pr_rank = nullptr;  // n (+ class counters): rank of each vertex by out-degree class
    uint32_t* pr_rcol = nullptr;  // transposed graph's neighbour ids as ranks (P_rev * K)
    uint2* pr_info = nullptr;     // n: (rank, out-degree) of each vertex, one load per finalisation
    PRCtrl* pctrl = nullptr;
    // data-driven PageRank (residual frontier)
    double* dd_r = nullptr;       // n: residuals
    double* dd_x = nullptr;       // n: values (FP64 accumulation; the output is written to x)
    double* dd_amt = nullptr;     // n: push amount of each vertex activated in the current round
    uint32_t* dd_pq = nullptr;    // P: part queue of the current round
    PRDDCtrl* ddctrl = nullptr;
    // misc
    unsigned long long* stats = nullptr;  // reached counters
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

}  // namespace eeg

struct eeg_vgraph {
    int device = 0;
    uint32_t n = 0;
    uint64_t m = 0;
    uint32_t K = 8;
    uint32_t flags = 0;
    bool managed = false;
    eeg::VDir fwd, rev;
    bool has_rev = false;
    bool rev_alias = false;  // EEG_VG_SYMMETRIC: rev shares fwd's arrays
    bool fwd_parts = true;   // false with EEG_VG_REVERSE_ONLY: fwd holds the out-degrees only
    bool weighted = true;
    uint32_t max_deg = 0, max_deg_vertex = 0;
    uint64_t bytes = 0;
    float build_ms = 0.f;
    eeg::Workspace ws;
};

namespace eeg {

// Bound on device-side waits from the options: timeout_us when set, else timeout_ms (default 10 s).
inline uint64_t wait_limit_ns(const eeg_options& o) {
    if (o.timeout_us) return (uint64_t)o.timeout_us * 1000ull;
    return (uint64_t)(o.timeout_ms ? o.timeout_ms : 10000u) * 1000000ull;
}

// allocation helpers (device or managed per graph)
eeg_status vg_alloc(eeg_vgraph* vg, void** p, size_t bytes);
void vg_free(eeg_vgraph* vg, void* p);

// builder (builder.cu)
eeg_status build_direction(eeg_vgraph* vg, VDir* d, const uint32_t* d_src, const uint32_t* d_dst,
                           const uint32_t* d_w, bool reverse, cudaStream_t st);
// Out-degrees (and the largest, with its vertex) without building the forward parts.
eeg_status build_out_degrees(eeg_vgraph* vg, VDir* d, const uint32_t* d_src, const uint32_t* d_dst, cudaStream_t st);

// kernels (traverse.cu / pagerank.cu)
eeg_status run_traversal(eeg_vgraph* vg, int op, eeg_variant variant, uint32_t source, const eeg_options& o,
                         cudaStream_t st, eeg_result* res, uint32_t* activity_host, uint32_t activity_cap);
eeg_status run_pagerank(eeg_vgraph* vg, eeg_variant variant, const eeg_options& o, cudaStream_t st, eeg_result* res);
eeg_status run_pagerank_dd(eeg_vgraph* vg, eeg_variant variant, const eeg_options& o, cudaStream_t st,
                           eeg_result* res);
eeg_status reached_stats(eeg_vgraph* vg, int op, const uint32_t* d_dist, cudaStream_t st, uint64_t* n_r, uint64_t* m_r);

}  // namespace eeg
