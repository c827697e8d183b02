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

// CTA size per operator, two CTAs per SM: 384 threads (85 registers) for BFS, whose group of atomics
// then covers a whole 8-slot part; 512 threads (64 registers) for the others. Measured with K = 8:
// BFS 0.385 against 0.395 ms on R-MAT s22 and 2.2 against 2.6 ms on the 4096^2 grid; CC 1.35 against
// 1.33 ms, SSSP 0.80 against 0.75 ms and SSWP 0.74 against 0.73 ms at 384 and 512 respectively.
template <int OP>
__host__ __device__ constexpr int trav_tpb() {
    return OP == OP_BFS ? 384 : 512;
}

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
    uint32_t* pushed;      // P: the owner value each part last pushed with (DD; null = every queued part expands)
    const uint32_t* rvstart;  // source-seeded BFS: the transposed graph's parts (null = push rounds only)
    const uint32_t* rvcol;
    uint32_t* plist;          // 2n: the vertices each pull round left unreached (two lists alternate)
    TravCtrl* ctrl;
    uint32_t* activity;
    uint32_t activity_cap;
    uint32_t source;
    uint32_t seed_all;
    uint32_t partner;
    uint32_t max_iters;
    uint32_t it_start;     // first round of this launch (0: also the set-up phase)
    uint64_t timeout_ns;
    uint32_t rounds_limit; // rounds this launch may run (host-loop mode: 1); 0 = until done
    uint32_t delta;        // SSSP/SSWP bucket width (bucketed kernels only)
    uint32_t* fpile;       // 3 x n far piles (bucketed kernels only)
    uint32_t* fflag;       // n far flags (1 = in a pile)
    uint32_t cc_zero;      // CC: relax with weight 0 (connected components)
};

// The weights of part p (CC in connected-components mode: zeros, nothing loaded).
template <int OP, int K>
__device__ __forceinline__ void load_weights(const TravArgs& a, uint32_t p, uint32_t (&wt)[K], uint64_t pol) {
    if (OP == OP_CC && a.cc_zero) {
#pragma unroll
        for (int i = 0; i < K; ++i) wt[i] = 0u;
    } else {
        ld_part<K>(a.vw + (size_t)p * K, wt, pol);
    }
}

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
// Slots whose atomics are issued together (value atomic + claim, 2 returned values each) under a
// 64-register budget (512-thread CTAs; the batch kernel): the most that fits without slowing the kernel
// -- measured on R-MAT s22 with K = 8, groups of 4 for BFS and SSSP (0.39 / 0.75 ms; 2: 0.40 / 0.77),
// 2 for SSWP and CC (0.73 / 1.30 ms; 4 spilled registers: 0.80 / 1.50; 1: 0.76 / 1.34).
template <int OP>
__host__ __device__ constexpr int atomic_group() {
    return (OP == OP_SSWP || OP == OP_CC) ? 2 : 4;
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

constexpr int WCAP = 256;  // per-warp append buffer (claimed vertices) before a flush to the queue
constexpr uint32_t PULL_LANE = 4;  // BFS pull rounds: parts a lane walks alone before the warp takes over

// Warp-cooperative append of the warp's claimed vertices to the next queue: one reservation per flush
// (atomicAdd of the parts total), then every claimed vertex's part ids are written; a vertex with more
// than 32 parts is written by the whole warp. Called by all 32 lanes with a warp-uniform `cnt`.
// Entries at or beyond `cap` are not written (each vertex is claimed once per round, so a round never
// produces more than `cap` = the number of parts; the reader clamps and reports an overflow).
__device__ __forceinline__ void warp_append(const uint32_t* __restrict__ vstart, uint32_t* parts_ctr,
                                            uint32_t* verts_ctr, const uint32_t* buf, uint32_t cnt, uint32_t* qnext,
                                            uint32_t lane, uint32_t cap) {
    __syncwarp();
    uint32_t sum = 0;
    for (uint32_t e = lane; e < cnt; e += 32u) {
        const uint32_t t = buf[e];
        sum += vstart[t + 1] - vstart[t];
    }
    uint32_t inc = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= (uint32_t)off) inc += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    uint32_t base = 0;
    if (lane == 0) {
        if (total) base = atomicAdd(parts_ctr, total);
        if (verts_ctr) atomicAdd(verts_ctr, cnt);
    }
    base = __shfl_sync(0xffffffffu, base, 0);
    uint32_t pos = base + inc - sum;
    const uint32_t rounds = (cnt + 31u) / 32u;
    for (uint32_t k = 0; k < rounds; ++k) {
        const uint32_t e = k * 32u + lane;
        uint32_t s0 = 0, np = 0;
        if (e < cnt) {
            const uint32_t t = buf[e];
            s0 = vstart[t];
            np = vstart[t + 1] - s0;
            if (np <= 32u)
                for (uint32_t j = 0; j < np; ++j)
                    if (pos + j < cap) qnext[pos + j] = s0 + j;
        }
        uint32_t big = __ballot_sync(0xffffffffu, np > 32u);
        while (big) {  // hub vertices: the whole warp writes their part ids
            const int l = __ffs(big) - 1;
            big &= big - 1u;
            const uint32_t bs0 = __shfl_sync(0xffffffffu, s0, l);
            const uint32_t bnp = __shfl_sync(0xffffffffu, np, l);
            const uint32_t bpos = __shfl_sync(0xffffffffu, pos, l);
            for (uint32_t j = lane; j < bnp; j += 32u)
                if (bpos + j < cap) qnext[bpos + j] = bs0 + j;
        }
        pos += np;
    }
    __syncwarp();
}

__device__ __forceinline__ void warp_flush(const TravArgs& a, const uint32_t* buf, uint32_t cnt, uint32_t* qnext,
                                           uint32_t nxt, uint32_t lane) {
    warp_append(a.vstart, &a.ctrl->qparts[nxt], &a.ctrl->qverts[nxt], buf, cnt, qnext, lane, a.P);
}

// BK (SSSP/SSWP, SYNC_PUSH_DD, delta > 0): bucketed rounds. A claimed vertex whose key (SSSP: distance,
// SSWP: INF - width; smaller is closer in both) is not below the threshold T waits in a far pile (one
// entry per vertex, marked by its flag) instead of entering the next queue. When the queue runs empty,
// a far round sets T = smallest recorded far key + delta and moves every far vertex below T back.
// The fixed point is the same; on high-diameter graphs far fewer edges are rescanned. T and the
// current pile travel in control words keyed by round parity, so every CTA (and every host-loop
// launch) reads the value the previous round settled; three piles rotate so that a pile's length is
// reset two far rounds before it is written again.
template <int OP, int K, bool TD, bool BK = false>
__global__ void __launch_bounds__(trav_tpb<OP>(), 2) k_traverse(TravArgs a) {
    constexpr int T_TPB = trav_tpb<OP>();
    __shared__ uint32_t s_buf[TD ? 1 : T_TPB / 32][TD ? 1 : WCAP];
    __shared__ uint32_t s_next[2];  // per round (alternating): next of this CTA's 32-entry chunks
    __shared__ uint32_t s_ctl[6];   // this round's control words, read once per CTA

    TravCtrl* ctrl = a.ctrl;
    const uint32_t gtid = blockIdx.x * T_TPB + threadIdx.x;
    const uint32_t gthreads = gridDim.x * T_TPB;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    uint32_t* wbuf = s_buf[TD ? 0 : threadIdx.x >> 5];
    const uint64_t pol = l2_evict_first_policy();
    uint32_t epoch = 0;

    unsigned long long my_parts = 0, my_edges = 0, my_updates = 0;
    // BFS seeded with the source only: every round's queue holds exactly the vertices at level `it`
    // (a round sets values to it+1 only, and a vertex leaves INF once, so atomicMin alone makes each claim
    // unique). Seeding every vertex (ASYNC_PUSH_DD) makes round 0 dense and in place: a vertex reached in
    // it may push again in the same round, so levels in a queue mix and claims need the stamps.
    const bool bfs_levels = OP == OP_BFS && !TD && !a.seed_all;
    // CC: a queued part that already pushed its owner's current value skips its expansion: every target
    // holds at most that value + the weight already (labels only fall), and an improvement of the owner
    // later in the round re-queues it. In the dense all-seeded round 0 most vertices are improved before
    // their own parts are reached and push the improved label, so their round-1 rescan is redundant:
    // edges scanned per reached edge 2.03 -> 1.20 and 1.33 -> 1.22 ms on R-MAT s22 (symmetrised).
    // SSSP and SSWP rescan less for it too (1.59 -> 1.21, 1.65 -> 1.19) but take the same time, and the
    // per-part values cost them 15 % more DRAM traffic, so their kernels leave the check out, as does BFS.
    const bool use_push = OP == OP_CC && !TD && !BK && a.pushed != nullptr;
    constexpr uint32_t PSENT = OP == OP_SSWP ? 0u : 0xFFFFFFFFu;  // no part ever pushes with it
    // Direction-optimising BFS (source-seeded, one persistent launch): when the frontier's parts are many
    // against the parts of the vertices not yet reached (14x), a round pulls instead of pushing -- every
    // unreached vertex reads the levels of its in-neighbours from the transposed parts, part by part, and
    // takes level it+1 at the first one found at level it (its forward parts are appended, so a push
    // round can follow); rounds push again once the frontier holds fewer than n/12 vertices. Every CTA
    // takes the same decision from the same control words. The first pull round walks every vertex and
    // lists the ones with in-edges that it left unreached; a later pull round walks the last list only
    // (a superset of the unreached vertices with in-edges, whatever rounds came between). Same levels;
    // R-MAT s22 from the hub pulls in its two large rounds, the second over 6.5 % of the vertices.
    constexpr bool BFSBU = OP == OP_BFS && !TD && !BK;
    constexpr int PVL = K <= 8 ? 4 : 2;  // vertices per lane in a pull round, their loads issued together
    const bool can_bu = BFSBU && bfs_levels && a.rvstart != nullptr && a.rounds_limit == 0;
    uint32_t seen_parts = 0;  // forward parts of the vertices reached so far
    bool bu = false;          // this round pulls
    uint32_t pj = 0;          // pull rounds so far
    uint32_t it = a.it_start;
    bool all_done = true;  // false when this launch stops only because of rounds_limit
    if (threadIdx.x == 0) s_next[0] = s_next[1] = 0u;
    __syncthreads();
    if (a.it_start == 0) {
        // ---- round 0 set-up: values, stamps, initial frontier
        for (uint32_t v = gtid; v < a.n; v += gthreads) {
            a.dist[v] = init_value<OP>(v, a.source);
            if (!TD && !bfs_levels) a.stamp[v] = 0u;
            if (BK) a.fflag[v] = 0u;
        }
        if (use_push)
            for (uint32_t q = gtid; q < a.P; q += gthreads) a.pushed[q] = PSENT;
        if (BK && blockIdx.x == 0 && threadIdx.x == 0) {
            for (int i = 0; i < 3; ++i) {
                ctrl->fcnt[i] = 0u;
                ctrl->fmin[i] = 0xFFFFFFFFu;
            }
            ctrl->fcsel[0] = 0u;  // round 0 (the source's parts) sends every claim to pile 0 (T = 0)
            ctrl->tsel[0] = 0u;
        }
        if (BFSBU && blockIdx.x == 0 && threadIdx.x == 0) ctrl->lcnt[0] = ctrl->lcnt[1] = ctrl->lcnt[2] = 0u;
        if (!TD && !a.seed_all && blockIdx.x == 0) {
            const uint32_t s0 = a.vstart[a.source], s1 = a.vstart[a.source + 1];
            for (uint32_t j = threadIdx.x; j < s1 - s0; j += T_TPB) a.q0[j] = s0 + j;
            if (threadIdx.x == 0) {
                ctrl->qparts[0] = s1 - s0;
                ctrl->qverts[0] = 1u;
            }
        }
        if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) goto finish;
    }

    for (;; ++it) {
        if (a.rounds_limit && it - a.it_start >= a.rounds_limit) {  // host-loop mode: next round, next launch
            all_done = false;
            break;
        }
        const uint32_t cur = it % 3u, nxt = (it + 1u) % 3u, old = (it + 2u) % 3u;
        const bool dense = TD || (a.seed_all && it == 0);
        // one thread per CTA reads the control words the previous round settled (not every warp of the
        // grid: those same-address reads queue at one L2 slice); the CTA takes them from shared memory
        if (threadIdx.x == 0) {
            s_ctl[0] = ld_relaxed(&ctrl->qparts[cur]);
            if (BFSBU) {
                s_ctl[5] = ld_relaxed(&ctrl->qverts[cur]);
                s_ctl[1] = ld_relaxed(&ctrl->lcnt[(pj + 2u) % 3u]);  // the last pull round's list
            }
            if (BK) {
                const uint32_t f = ld_relaxed(&ctrl->fcsel[it & 1u]);
                s_ctl[1] = f;
                s_ctl[2] = ld_relaxed(&ctrl->tsel[it & 1u]);
                s_ctl[3] = ld_relaxed(&ctrl->fcnt[f]);
                s_ctl[4] = ld_relaxed(&ctrl->fmin[f]);
            }
        }
        __syncthreads();
        uint32_t fc = 0, T = 0xFFFFFFFFu, fcount = 0;
        if (BK) {
            fc = s_ctl[1];
            T = s_ctl[2];
            fcount = s_ctl[3];
        }
        if (it > 0) {
            const uint32_t produced = s_ctl[0];
            if (a.activity && blockIdx.x == 0 && threadIdx.x == 0 && it - 1 < a.activity_cap)
                a.activity[it - 1] = TD ? produced : ld_relaxed(&ctrl->qverts[cur]);
            if (produced == 0u && fcount == 0u) break;
        }
        if (can_bu) {
            const uint32_t fparts = s_ctl[0], fverts = s_ctl[5];
            seen_parts += fparts;
            const uint32_t unreached_parts = a.P - (seen_parts < a.P ? seen_parts : a.P);
            bu = bu ? (uint64_t)fverts * 12u >= a.n : (it > 0 && (uint64_t)fparts * 14u > unreached_parts);
        }
        uint32_t len;
        const bool swap = TD && a.partner && (it & 1u);
        if (dense) len = swap ? (a.P + (a.P & 1u)) : a.P;
        else len = s_ctl[0];
        const bool frontier_empty = !dense && len == 0u;
        if (!dense && len > a.P) {  // cannot happen (one claim per vertex per round); never read past the queue
            if (blockIdx.x == 0 && threadIdx.x == 0)
                atomicCAS(&ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_OVERFLOW);
            len = a.P;
        }
        // a pull round walks every vertex, or the last pull round's list
        const uint32_t pcnt = BFSBU ? (pj > 0 && s_ctl[1] < a.n ? s_ctl[1] : a.n) : 0u;
        if (BFSBU && bu) len = (uint32_t)(((uint64_t)pcnt + 32u * PVL - 1u) / (32u * PVL) * 32u);
        bool far_round = false;
        if (frontier_empty) {
            if (!BK || fcount == 0u) break;
            if (fcount > a.n) {  // one entry per flagged vertex; never read past the pile
                if (blockIdx.x == 0 && threadIdx.x == 0)
                    atomicCAS(&ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_OVERFLOW);
                fcount = a.n;
            }
            far_round = true;
            const uint32_t fm = s_ctl[4];
            T = fm > 0xFFFFFFFFu - a.delta ? 0xFFFFFFFFu : fm + a.delta;
        }
        const uint32_t fdst = far_round ? (fc + 1u) % 3u : fc;  // pile receiving this round's far vertices
        if (it >= a.max_iters) {
            if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_ITER_CAP);
            break;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctrl->qparts[old] = 0u;
            ctrl->qverts[old] = 0u;
            if (BFSBU && bu) ctrl->lcnt[(pj + 1u) % 3u] = 0u;  // the next pull round's list
            if (BK) {  // what the next round reads; the pile two far rounds back is free again
                ctrl->fcsel[(it + 1u) & 1u] = fdst;
                ctrl->tsel[(it + 1u) & 1u] = T;
                if (far_round) {
                    ctrl->fcnt[(fc + 2u) % 3u] = 0u;
                    ctrl->fmin[(fc + 2u) % 3u] = 0xFFFFFFFFu;
                }
            }
        }
        const uint32_t* pile_src = BK ? a.fpile + (size_t)fc * a.n : nullptr;
        uint32_t* pile_dst = BK ? a.fpile + (size_t)fdst * a.n : nullptr;
        // Warp-collective: the lanes with `fl` send vertex t (key `key`) to the far pile. A vertex enters
        // the pile once (its flag); the pile's count and smallest key take one atomic per warp, not per
        // vertex (same-address atomics from every warp queue at one L2 slice).
        auto to_far = [&](bool fl, uint32_t t, uint32_t key) {
            const uint32_t fmask = __ballot_sync(0xffffffffu, fl);
            if (!fmask) return;
            const bool app = fl && atomicExch(&a.fflag[t], 1u) != 1u;
            const uint32_t amask = __ballot_sync(0xffffffffu, app);
            const uint32_t kmin = __reduce_min_sync(0xffffffffu, fl ? key : 0xFFFFFFFFu);
            const uint32_t leader = __ffs(fmask) - 1u;
            uint32_t base = 0;
            if (lane == leader) {
                if (amask) base = atomicAdd(&ctrl->fcnt[fdst], (uint32_t)__popc(amask));
                atomicMin(&ctrl->fmin[fdst], kmin);
            }
            base = __shfl_sync(0xffffffffu, base, leader);
            if (app) {
                const uint32_t pos = base + (uint32_t)__popc(amask & lanemask_lt);
                if (pos < a.n) pile_dst[pos] = t;
                else atomicCAS(&ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_OVERFLOW);
            }
        };
        // no __restrict__/const-qualified read-only path here: each queue is rewritten every other round
        const uint32_t* qcur = (it & 1u) ? a.q1 : a.q0;
        uint32_t* qnext = (it & 1u) ? a.q0 : a.q1;
        const uint32_t tag = it + 1u;
        uint32_t changed = 0;
        uint32_t wcnt = 0;  // warp-uniform fill of wbuf
        // This CTA's share of the round is the strided set of 32-entry chunks blockIdx.x + i * gridDim.x;
        // its warps draw from it through a shared counter (this round's; the other one is reset for the
        // next round, whose start is ordered by the grid barrier).
        if (threadIdx.x == 0) s_next[(it + 1u) & 1u] = 0u;
        const uint32_t items = far_round ? fcount : len;
        const uint32_t nch = (items + 31u) / 32u;
        // A pull round's chunks are vertex ranges, and a vertex id's low bits set its degree on R-MAT-like
        // graphs: with chunk b + i * grid (grid = 304 = 16 * 19) a CTA saw the same low bits in every
        // chunk, and CTAs took 115 to 360 thousand cycles over the same chunk counts (R-MAT s22). In a
        // pull round a CTA takes chunk i * grid + (b + i) mod grid of each row i instead: every chunk
        // once, every residue in every CTA.
        const bool rot = BFSBU && bu;
        const uint32_t my_chunks = rot ? (nch + gridDim.x - 1u) / gridDim.x
                                       : (nch > blockIdx.x ? (nch - blockIdx.x + gridDim.x - 1u) / gridDim.x : 0u);

        // Software-pipelined by one chunk: the next chunk is drawn and its queue entries are loaded
        // before the current chunk is expanded, so the queue load is off each part's dependent chain.
        auto draw = [&](uint32_t& pn) -> uint32_t {
            uint32_t ci = 0;
            if (lane == 0) ci = atomicAdd(&s_next[it & 1u], 1u);
            ci = __shfl_sync(0xffffffffu, ci, 0);
            pn = 0xFFFFFFFFu;
            if (ci < my_chunks) {
                uint32_t ch = blockIdx.x + ci;
                if (rot) {
                    while (ch >= gridDim.x) ch -= gridDim.x;
                    ch += ci * gridDim.x;
                } else {
                    ch = blockIdx.x + ci * gridDim.x;
                }
                const uint32_t idx = ch * 32u + lane;
                if (idx < items) {
                    pn = far_round ? pile_src[idx] : ((dense || (BFSBU && bu)) ? idx : qcur[idx]);
                    if (swap) pn ^= 1u;
                }
            }
            return ci;
        };
        uint32_t p_next;
        uint32_t ci_next = draw(p_next);
        for (;;) {
            if (ci_next >= my_chunks) break;
            const uint32_t p = p_next;
            ci_next = draw(p_next);
            if (BK && far_round) {  // far round: p is a far vertex; move it back when below T
                bool move = false, stay = false;
                uint32_t key = 0;
                if (p < a.n && atomicExch(&a.fflag[p], 0u) == 1u) {
                    const uint32_t dv = a.dist[p];
                    key = OP == OP_SSWP ? INF - dv : dv;
                    if (key < T) move = true;
                    else stay = true;
                }
                to_far(stay, p, key);
                const uint32_t mask = __ballot_sync(0xffffffffu, move);
                if (mask) {
                    const uint32_t c = __popc(mask);
                    if (wcnt + c > (uint32_t)WCAP) {
                        warp_flush(a, wbuf, wcnt, qnext, nxt, lane);
                        wcnt = 0;
                    }
                    if (move) wbuf[wcnt + __popc(mask & lanemask_lt)] = p;
                    wcnt += c;
                }
                continue;
            }
            if (BFSBU && bu) {  // pull: item p covers PVL vertices, 32 apart; each belongs to this lane alone
                bool want[PVL], claim[PVL];
                uint32_t vv[PVL], s0[PVL], np[PVL];
                const uint64_t vb = (uint64_t)(p >> 5) * (32u * PVL) + (p & 31u);
                const uint32_t* lrd = a.plist + (size_t)((pj + 1u) & 1u) * a.n;  // the last pull round's list
#pragma unroll
                for (int k = 0; k < PVL; ++k) {  // every level and part range first, then every first part
                    const uint64_t li = vb + 32u * k;
                    const bool ok = p < items && li < pcnt;
                    const uint32_t v = ok ? (pj > 0 ? lrd[li] : (uint32_t)li) : 0u;
                    want[k] = claim[k] = false;
                    vv[k] = v;
                    s0[k] = np[k] = 0u;
                    if (ok) {
                        const uint32_t dv = a.dist[v];
                        s0[k] = __ldg(&a.rvstart[v]);
                        np[k] = __ldg(&a.rvstart[v + 1]) - s0[k];
                        want[k] = dv == INF && np[k] > 0u;
                    }
                }
                {
                    uint32_t c[PVL][K];
#pragma unroll
                    for (int k = 0; k < PVL; ++k) {
                        if (want[k]) ld_part<K>(a.rvcol + (size_t)s0[k] * K, c[k], pol);
                        else
#pragma unroll
                            for (int i = 0; i < K; ++i) c[k][i] = NO_EDGE;
                    }
#pragma unroll
                    for (int k = 0; k < PVL; ++k) {
                        bool found = false;
#pragma unroll
                        for (int i = 0; i < K; ++i) {
                            if (c[k][i] != NO_EDGE) {
                                found |= a.dist[c[k][i]] == it;
                                ++my_edges;
                            }
                        }
                        if (want[k]) ++my_parts;
                        claim[k] = found;
                    }
                }
#pragma unroll
                for (int k = 0; k < PVL; ++k) {
                    // no parent in the first part: the lane walks the next ones up to PULL_LANE ...
                    const uint32_t lim = want[k] ? (np[k] < PULL_LANE ? np[k] : PULL_LANE) : 0u;
                    for (uint32_t j = 1; j < lim && !claim[k]; ++j) {
                        uint32_t c[K];
                        ld_part<K>(a.rvcol + (size_t)(s0[k] + j) * K, c, pol);
                        bool found = false;
#pragma unroll
                        for (int i = 0; i < K; ++i) {
                            if (c[i] != NO_EDGE) {
                                found |= a.dist[c[i]] == it;
                                ++my_edges;
                            }
                        }
                        ++my_parts;
                        claim[k] = found;
                    }
                    // ... and the warp walks the rest of a longer one, 32 parts at a time
                    uint32_t big = __ballot_sync(0xffffffffu, want[k] && !claim[k] && np[k] > PULL_LANE);
                    while (big) {
                        const int l = __ffs(big) - 1;
                        big &= big - 1u;
                        const uint32_t bs0 = __shfl_sync(0xffffffffu, s0[k], l);
                        const uint32_t bnp = __shfl_sync(0xffffffffu, np[k], l);
                        bool any = false;
                        for (uint32_t j0 = PULL_LANE; j0 < bnp && !any; j0 += 32u) {
                            const uint32_t j = j0 + lane;
                            bool found = false;
                            if (j < bnp) {
                                uint32_t c[K];
                                ld_part<K>(a.rvcol + (size_t)(bs0 + j) * K, c, pol);
#pragma unroll
                                for (int i = 0; i < K; ++i) {
                                    if (c[i] != NO_EDGE) {
                                        found |= a.dist[c[i]] == it;
                                        ++my_edges;
                                    }
                                }
                                ++my_parts;
                            }
                            any = __any_sync(0xffffffffu, found);
                        }
                        if ((uint32_t)l == lane) claim[k] = any;
                    }
                    if (claim[k]) {
                        a.dist[vv[k]] = it + 1u;  // no other writer: push and pull rounds never mix
                        ++my_updates;
                    }
                    const uint32_t mask = __ballot_sync(0xffffffffu, claim[k]);
                    if (mask) {
                        const uint32_t cn = __popc(mask);
                        if (wcnt + cn > (uint32_t)WCAP) {
                            warp_flush(a, wbuf, wcnt, qnext, nxt, lane);
                            wcnt = 0;
                        }
                        if (claim[k]) wbuf[wcnt + __popc(mask & lanemask_lt)] = vv[k];
                        wcnt += cn;
                    }
                }
                // the vertices left unreached go on this round's list, one reservation per chunk (buffering
                // them per warp to reserve less often made R-MAT s22's first pull round 12 % slower)
                uint32_t lm[PVL], tot = 0;
#pragma unroll
                for (int k = 0; k < PVL; ++k) {
                    lm[k] = __ballot_sync(0xffffffffu, want[k] && !claim[k]);
                    tot += __popc(lm[k]);
                }
                if (tot) {
                    uint32_t lb = 0;
                    if (lane == 0) lb = atomicAdd(&ctrl->lcnt[pj % 3u], tot);
                    lb = __shfl_sync(0xffffffffu, lb, 0);
                    uint32_t* lwr = a.plist + (size_t)(pj & 1u) * a.n;
#pragma unroll
                    for (int k = 0; k < PVL; ++k) {
                        if (want[k] && !claim[k]) {
                            const uint32_t pos = lb + __popc(lm[k] & lanemask_lt);
                            if (pos < a.n) lwr[pos] = vv[k];  // one entry per vertex: always below n
                        }
                        lb += __popc(lm[k]);
                    }
                }
                continue;
            }
            const bool valid = p < a.P;
            uint32_t col[K], wt[K];
            uint32_t d = 0;
            bool active = false;
            if (valid) {
                if (bfs_levels) {  // no owner or value load: the level is the round number
                    ld_part<K>(a.vcol + (size_t)p * K, col, pol);
                    d = it;
                    active = true;
                } else {
                    const uint32_t v = __ldg(&a.vowner[p]);
                    uint32_t pv = PSENT;
                    if (!TD) {  // DD: the part is almost surely live -- fetch its row alongside the owner's value
                        ld_part<K>(a.vcol + (size_t)p * K, col, pol);
                        if (OP != OP_BFS) load_weights<OP, K>(a, p, wt, pol);
                        if (use_push) pv = __ldcg(&a.pushed[p]);  // written in earlier rounds by any CTA
                    }
                    // plain (L1-cached) value reads: the grid barrier's acquire makes the previous round's
                    // values visible; a value improved later in this round re-enqueues its vertex anyway
                    d = a.dist[v];
                    active = !unreached<OP>(d);
                    if (use_push && active) {
                        if (d == pv) active = false;
                        else a.pushed[p] = d;
                    }
                    if (TD && active) {
                        ld_part<K>(a.vcol + (size_t)p * K, col, pol);
                        if (OP != OP_BFS) load_weights<OP, K>(a, p, wt, pol);
                    }
                }
                if (active) ++my_parts;
            }
            // all K filter reads are issued before the first atomic (the compiler may not move a load of
            // dist[] across an atomic on dist[]); a stale value only costs an atomic. Queued parts are
            // almost always live, so their filter reads do not wait for the owner's value.
            uint32_t cd[K];
            const bool fetch = (dense || use_push) ? active : valid;
#pragma unroll
            for (int i = 0; i < K; ++i) cd[i] = (fetch && col[i] != NO_EDGE) ? a.dist[col[i]] : 0u;
            // The atomics of ATB slots go out before any of their results is used: for each slot whose
            // filter read says the target improves, the value atomic and (DD, except BFS levels) the
            // claim on the target's round stamp are issued together. A won claim means the target
            // improved in this round -- by this lane, or by another after this lane's filter read (that
            // read is no older than the round's start, and values move one way only) -- so the winner
            // appends the target, whoever improved it, and a target improved in a round is appended
            // exactly once.
            // the far-pile path takes registers too; the 384-thread shape has room for a whole part
            constexpr int ATG = BK ? 2 : (trav_tpb<OP>() == 384 ? 8 : atomic_group<OP>());
            constexpr int ATB = K < ATG ? K : ATG;
#pragma unroll
            for (int i0 = 0; i0 < K; i0 += ATB) {
                uint32_t prev[ATB], ex[ATB];
                uint32_t hit = 0;  // slots whose filter passed
#pragma unroll
                for (int j = 0; j < ATB; ++j) {
                    const int i = i0 + j;
                    prev[j] = 0u;
                    ex[j] = tag;
                    if (active && col[i] != NO_EDGE) {
                        ++my_edges;
                        const uint32_t nd = relax_value<OP>(d, OP == OP_BFS ? 1u : wt[i]);
                        if (better<OP>(nd, cd[i])) {
                            hit |= 1u << j;
                            prev[j] = atomic_improve<OP>(&a.dist[col[i]], nd);
                            if (!TD && !bfs_levels) ex[j] = atomicExch(&a.stamp[col[i]], tag);
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < ATB; ++j) {
                    const int i = i0 + j;
                    bool claim = false, far = false;
                    uint32_t fkey = 0;
                    const uint32_t t = col[i];
                    if ((hit >> j) & 1u) {
                        const uint32_t nd = relax_value<OP>(d, OP == OP_BFS ? 1u : wt[i]);
                        const bool imp = better<OP>(nd, prev[j]);
                        if (imp) ++my_updates;
                        if (TD) {
                            if (imp) changed = 1u;
                        } else if (bfs_levels) {
                            claim = imp;  // atomicMin admits one first improvement
                        } else {
                            claim = ex[j] != tag;
                        }
                        if (BK && claim) {
                            const uint32_t now = imp ? nd : prev[j];  // the target's value after this atomic
                            const uint32_t key = OP == OP_SSWP ? INF - now : now;
                            if (key >= T) {  // not in this bucket: wait in the far pile
                                far = true;
                                fkey = key;
                                claim = false;
                            }
                        }
                    }
                    if (BK) to_far(far, t, fkey);
                    if (!TD) {
                        const uint32_t mask = __ballot_sync(0xffffffffu, claim);
                        if (mask) {
                            const uint32_t c = __popc(mask);
                            if (wcnt + c > (uint32_t)WCAP) {
                                warp_flush(a, wbuf, wcnt, qnext, nxt, lane);
                                wcnt = 0;
                            }
                            if (claim) wbuf[wcnt + __popc(mask & lanemask_lt)] = t;
                            wcnt += c;
                        }
                    }
                }
            }
        }
        if (TD) {
            if (__syncthreads_or(changed) && threadIdx.x == 0) atomicAdd(&ctrl->qparts[nxt], 1u);
        } else if (wcnt) {
            warp_flush(a, wbuf, wcnt, qnext, nxt, lane);
        }
        if (BFSBU && bu) ++pj;
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
    if (lane == 0) {
        if (my_parts) atomicAdd(&ctrl->parts_processed, my_parts);
        if (my_edges) atomicAdd(&ctrl->edges_scanned, my_edges);
        if (my_updates) atomicAdd(&ctrl->updates, my_updates);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctrl->iterations = it;
        ctrl->done = all_done ? 1u : 0u;
        if (BFSBU) ctrl->pull_rounds = pj;
    }
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
    constexpr bool CAN_BK = !TD && (OP == OP_SSSP || OP == OP_SSWP);
    auto kern = (CAN_BK && args.delta && !args.seed_all) ? k_traverse<OP, K, TD, CAN_BK> : k_traverse<OP, K, TD, false>;
    constexpr int T_TPB = trav_tpb<OP>();
    // The filter reads of dist[] are L1 hits in part, and L1 is what shared memory leaves: ask for the
    // smallest carveout that still holds the two CTAs per SM the kernel is built for (R-MAT s22: SSSP
    // 0.725 -> 0.706 ms, SSWP 0.726 -> 0.709, CC 1.215 -> 1.193 against the CUDA driver's default).
    EEG_TRY(prefer_l1(kern, 2, device));
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
