// traverse.cuh -- persistent push kernels for BFS, SSSP, SSWP and CC over the K-bounded virtual graph.
//
// Reference kernels replaced (rwatling/EEGraph):
//   bfs::{async,sync}_push_{td,dd}   src/bfs.cu:27-273     relax d+1,        atomicMin
//   sssp::{async,sync}_push_{td,dd}  src/sssp.cu:26-299    relax d+w,        atomicMin
//   sswp::{async,sync}_push_{td,dd}  src/sswp.cu:26-271    relax min(d,w),   atomicMax
//   cc::{async,sync}_push_{td,dd}    src/cc.cu:26-271      relax label+w,    atomicMin
//   clearLabel/mixLabels/moveUpLabels/sumLabels  src/gpu_utils.cu:3-34 (frontier upkeep, fused here)
//   the host do { H2D finished; launch; sync; D2H finished } while(!finished) loop, src/eegraph.cu:89-211
//
// One cooperative launch runs the whole traversal. Rounds are separated by a bounded grid barrier
// (common.cuh) instead of a host round trip. A thread expands one part (<= K out-edges of one vertex)
// with K/4 aligned 128-bit streaming loads of targets and weights.
//   TD (topology driven): every round expands every part, as the reference's *_push_td kernels do.
//      SYNC_PUSH_TD keeps the reference's odd/even partner permutation (src/bfs.cu:196-272).
//   DD (data driven): the frontier is a queue of PART ids. A vertex whose value improved is claimed
//      once per round through a round stamp. Each CTA then appends the parts of its claimed vertices
//      with one atomic reservation per CTA chunk (hub vertices are written by the whole CTA). This
//      replaces label1/label2 + clearLabel; the queue-length counters give --activity (sumLabels).
//      SYNC_PUSH_DD seeds {source}; ASYNC_PUSH_DD seeds every vertex (src/eegraph.cu:41-49).
// Values are updated in place with atomicMin/atomicMax, as in the reference; a vertex whose value is
// still "unreached" (BFS/SSSP: DIST_INFINITY, SSWP: 0) pushes nothing. That keeps SSSP free of the
// INF+w wrap of src/sssp.cu:62 (identical to the reference's SYNC_PUSH_DD results) without changing
// any other fixed point.
#pragma once
#include <algorithm>
#include <cstdio>

#include "internal.hpp"

namespace eeg {
namespace trav {

constexpr int T_TPB = 512;
constexpr int BIG_PARTS = 32;  // a claimed vertex with more parts is appended by the whole CTA
constexpr int BIG_CAP = 64;

struct TravArgs {
    uint32_t n;
    uint32_t P;
    const uint32_t* __restrict__ vstart;
    const uint32_t* __restrict__ vowner;
    const uint32_t* __restrict__ vcol;
    const uint32_t* __restrict__ vw;
    uint32_t* dist;
    uint32_t* q0;
    uint32_t* q1;
    uint32_t* stamp;
    TravCtrl* ctrl;
    uint32_t* activity;
    uint32_t activity_cap;
    uint32_t source;
    uint32_t seed_all;
    uint32_t partner;
    uint32_t max_iters;
    uint32_t pad;
    uint64_t timeout_ns;
};

template <int OP>
__device__ __forceinline__ uint32_t init_value(uint32_t v, uint32_t src) {
    if (OP == OP_CC) return v;                       // src/eegraph.cu:546
    if (OP == OP_SSWP) return v == src ? INF : 0u;   // src/eegraph.cu:1551-1559
    return v == src ? 0u : INF;                      // src/eegraph.cu:41-49, 2062-2073
}
template <int OP>
__device__ __forceinline__ bool unreached(uint32_t d) {
    if (OP == OP_BFS || OP == OP_SSSP) return d == INF;
    if (OP == OP_SSWP) return d == 0u;
    return false;
}
template <int OP>
__device__ __forceinline__ uint32_t relax_value(uint32_t d, uint32_t w) {
    if (OP == OP_BFS) return d + 1u;
    if (OP == OP_SSWP) return d < w ? d : w;
    const uint64_t s = (uint64_t)d + w;              // SSSP / CC: saturate, never wrap
    return s >= INF ? INF : (uint32_t)s;
}
template <int OP>
__device__ __forceinline__ bool better(uint32_t a, uint32_t b) {
    return OP == OP_SSWP ? a > b : a < b;
}
template <int OP>
__device__ __forceinline__ uint32_t atomic_improve(uint32_t* p, uint32_t v) {
    return OP == OP_SSWP ? atomicMax(p, v) : atomicMin(p, v);
}

struct BigEntry {
    uint32_t first, count, dst;
};

template <int OP, int K, bool TD>
__global__ void __launch_bounds__(T_TPB) k_traverse(TravArgs a) {
    constexpr int ACT_CAP = T_TPB * K;
    __shared__ uint32_t s_act[TD ? 1 : ACT_CAP];
    __shared__ uint32_t s_warp[33];
    __shared__ uint32_t s_cnt, s_base, s_nbig;
    __shared__ BigEntry s_big[TD ? 1 : BIG_CAP];

    TravCtrl* ctrl = a.ctrl;
    const uint32_t gtid = blockIdx.x * T_TPB + threadIdx.x;
    const uint32_t gthreads = gridDim.x * T_TPB;
    const uint64_t pol = l2_evict_first_policy();
    uint32_t epoch = 0;

    // ---- round 0 set-up: values, stamps, initial frontier
    for (uint32_t v = gtid; v < a.n; v += gthreads) {
        a.dist[v] = init_value<OP>(v, a.source);
        if (!TD) a.stamp[v] = 0u;
    }
    if (!TD && !a.seed_all && blockIdx.x == 0) {
        const uint32_t s0 = a.vstart[a.source], s1 = a.vstart[a.source + 1];
        for (uint32_t j = threadIdx.x; j < s1 - s0; j += T_TPB) a.q0[j] = s0 + j;
        if (threadIdx.x == 0) {
            ctrl->qparts[0] = s1 - s0;
            ctrl->qverts[0] = 1u;
        }
    }
    if (threadIdx.x == 0) {
        s_cnt = 0;
        s_nbig = 0;
    }
    unsigned long long my_parts = 0, my_edges = 0, my_updates = 0;
    uint32_t it = 0;
    if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) goto finish;

    for (;; ++it) {
        const uint32_t cur = it % 3u, nxt = (it + 1u) % 3u, old = (it + 2u) % 3u;
        const bool dense = TD || (a.seed_all && it == 0);
        if (it > 0) {
            const uint32_t produced = ld_relaxed(&ctrl->qparts[cur]);
            if (a.activity && blockIdx.x == 0 && threadIdx.x == 0 && it - 1 < a.activity_cap)
                a.activity[it - 1] = TD ? produced : ld_relaxed(&ctrl->qverts[cur]);
            if (produced == 0u) break;
        }
        uint32_t len;
        const bool swap = TD && a.partner && (it & 1u);
        if (dense) len = swap ? (a.P + (a.P & 1u)) : a.P;
        else len = ld_relaxed(&ctrl->qparts[cur]);
        if (!dense && len == 0u) break;
        if (it >= a.max_iters) {
            if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_ITER_CAP);
            break;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctrl->qparts[old] = 0u;
            ctrl->qverts[old] = 0u;
        }
        const uint32_t* __restrict__ qcur = (it & 1u) ? a.q1 : a.q0;
        uint32_t* __restrict__ qnext = (it & 1u) ? a.q0 : a.q1;
        const uint32_t tag = it + 1u;
        uint32_t changed = 0;

        for (uint32_t base = blockIdx.x * T_TPB; base < len; base += gthreads) {
            const uint32_t idx = base + threadIdx.x;
            if (idx < len) {
                uint32_t p = dense ? idx : qcur[idx];
                if (swap) p ^= 1u;
                if (p < a.P) {
                    const uint32_t v = __ldg(&a.vowner[p]);
                    const uint32_t d = __ldcg(&a.dist[v]);
                    if (!unreached<OP>(d)) {
                        ++my_parts;
                        uint32_t col[K], wt[K];
                        ld_part<K>(a.vcol + (size_t)p * K, col, pol);
                        if (OP != OP_BFS) ld_part<K>(a.vw + (size_t)p * K, wt, pol);
#pragma unroll
                        for (int i = 0; i < K; ++i) {
                            const uint32_t t = col[i];
                            if (t == NO_EDGE) break;
                            ++my_edges;
                            const uint32_t nd = relax_value<OP>(d, OP == OP_BFS ? 1u : wt[i]);
                            if (better<OP>(nd, __ldcg(&a.dist[t]))) {
                                const uint32_t prev = atomic_improve<OP>(&a.dist[t], nd);
                                if (better<OP>(nd, prev)) {
                                    ++my_updates;
                                    if (TD) {
                                        changed = 1u;
                                    } else if (__ldcg(&a.stamp[t]) != tag && atomicExch(&a.stamp[t], tag) != tag) {
                                        const uint32_t pos = atomicAdd(&s_cnt, 1u);
                                        if (pos < (uint32_t)ACT_CAP) {
                                            s_act[pos] = t;
                                        } else {  // CTA buffer full: append this vertex directly
                                            const uint32_t s0 = a.vstart[t], np = a.vstart[t + 1] - s0;
                                            const uint32_t b0 = np ? atomicAdd(&ctrl->qparts[nxt], np) : 0u;
                                            atomicAdd(&ctrl->qverts[nxt], 1u);
                                            for (uint32_t j = 0; j < np; ++j) qnext[b0 + j] = s0 + j;
                                        }
                                    }
                                }
                            }
                        }
                    }
                }
            }
            if (!TD) {
                // ---- CTA-aggregated append of the claimed vertices' parts to the next queue
                __syncthreads();
                const uint32_t A = min(s_cnt, (uint32_t)ACT_CAP);
                uint32_t mysum = 0;
                for (uint32_t i = threadIdx.x; i < A; i += T_TPB) {
                    const uint32_t t = s_act[i];
                    mysum += a.vstart[t + 1] - a.vstart[t];
                }
                uint32_t total;
                uint32_t off = block_exclusive_sum(mysum, s_warp, &total);
                if (threadIdx.x == 0) {
                    s_base = total ? atomicAdd(&ctrl->qparts[nxt], total) : 0u;
                    if (A) atomicAdd(&ctrl->qverts[nxt], A);
                    s_cnt = 0;
                    s_nbig = 0;
                }
                __syncthreads();
                uint32_t dstpos = s_base + off;
                for (uint32_t i = threadIdx.x; i < A; i += T_TPB) {
                    const uint32_t t = s_act[i];
                    const uint32_t s0 = a.vstart[t], np = a.vstart[t + 1] - s0;
                    if (np <= (uint32_t)BIG_PARTS) {
                        for (uint32_t j = 0; j < np; ++j) qnext[dstpos + j] = s0 + j;
                    } else {
                        const uint32_t b = atomicAdd(&s_nbig, 1u);
                        if (b < (uint32_t)BIG_CAP) s_big[b] = BigEntry{s0, np, dstpos};
                        else
                            for (uint32_t j = 0; j < np; ++j) qnext[dstpos + j] = s0 + j;
                    }
                    dstpos += np;
                }
                __syncthreads();
                const uint32_t nb = min(s_nbig, (uint32_t)BIG_CAP);
                for (uint32_t b = 0; b < nb; ++b) {
                    const BigEntry e = s_big[b];
                    for (uint32_t j = threadIdx.x; j < e.count; j += T_TPB) qnext[e.dst + j] = e.first + j;
                }
            }
        }
        if (TD) {
            if (__syncthreads_or(changed) && threadIdx.x == 0) atomicAdd(&ctrl->qparts[nxt], 1u);
        }
        if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) break;
    }

finish:
    // ---- statistics
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        my_parts += __shfl_down_sync(0xffffffffu, my_parts, off);
        my_edges += __shfl_down_sync(0xffffffffu, my_edges, off);
        my_updates += __shfl_down_sync(0xffffffffu, my_updates, off);
    }
    if ((threadIdx.x & 31u) == 0) {
        if (my_parts) atomicAdd(&ctrl->parts_processed, my_parts);
        if (my_edges) atomicAdd(&ctrl->edges_scanned, my_edges);
        if (my_updates) atomicAdd(&ctrl->updates, my_updates);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->iterations = it;
}

// Reached-set statistics: n_r and m_r (out-edges of reached vertices).
// Reached: BFS/SSSP value != DIST_INFINITY, SSWP value != 0 (the source holds DIST_INFINITY), CC all.
template <int OP>
__global__ void k_reached(const uint32_t* __restrict__ dist, const uint32_t* __restrict__ deg, uint32_t n,
                          unsigned long long* out) {
    unsigned long long nr = 0, mr = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t d = dist[v];
        bool r;
        if (OP == OP_CC) r = true;
        else if (OP == OP_SSWP) r = d != 0u;
        else r = d != INF;
        if (r) {
            ++nr;
            mr += deg[v];
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        nr += __shfl_down_sync(0xffffffffu, nr, off);
        mr += __shfl_down_sync(0xffffffffu, mr, off);
    }
    if ((threadIdx.x & 31u) == 0) {
        atomicAdd(&out[0], nr);
        atomicAdd(&out[1], mr);
    }
}

template <int OP, int K, bool TD>
eeg_status launch_one(const TravArgs& args, int device, uint32_t blocks_per_sm_req, cudaStream_t st) {
    auto kern = k_traverse<OP, K, TD>;
    int per_sm = 0;
    EEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T_TPB, 0));
    if (per_sm <= 0) {
        set_last_error("traversal kernel does not fit on an SM");
        return EEG_ERR_CUDA;
    }
    if (blocks_per_sm_req > 0 && (int)blocks_per_sm_req < per_sm) per_sm = (int)blocks_per_sm_req;
    uint64_t blocks = (uint64_t)per_sm * sm_count(device);
    const uint64_t work = std::max<uint64_t>(args.P, args.n);
    const uint64_t need = (work + T_TPB - 1) / T_TPB;
    if (need < blocks) blocks = std::max<uint64_t>(need, 1);
    TravArgs a = args;
    void* params[] = {(void*)&a};
    EEG_CUDA(cudaLaunchCooperativeKernel((const void*)kern, dim3((unsigned)blocks), dim3(T_TPB), params, 0, st));
    return EEG_OK;
}

template <int OP, bool TD>
eeg_status launch_k(const TravArgs& args, uint32_t K, int device, uint32_t bps, cudaStream_t st) {
    switch (K) {
        case 4: return launch_one<OP, 4, TD>(args, device, bps, st);
        case 8: return launch_one<OP, 8, TD>(args, device, bps, st);
        case 16: return launch_one<OP, 16, TD>(args, device, bps, st);
        default: set_last_error("K must be 4, 8 or 16"); return EEG_ERR_UNSUPPORTED;
    }
}

// Launch the traversal of one operator; each is defined in its own translation unit traverse_<op>.cu.
eeg_status launch_bfs(const TravArgs& args, bool td, uint32_t K, int device, uint32_t bps, cudaStream_t st);
eeg_status launch_sssp(const TravArgs& args, bool td, uint32_t K, int device, uint32_t bps, cudaStream_t st);
eeg_status launch_sswp(const TravArgs& args, bool td, uint32_t K, int device, uint32_t bps, cudaStream_t st);
eeg_status launch_cc(const TravArgs& args, bool td, uint32_t K, int device, uint32_t bps, cudaStream_t st);

}  // namespace trav
}  // namespace eeg
