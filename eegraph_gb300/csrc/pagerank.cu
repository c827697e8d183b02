// pagerank.cu -- PageRank over the K-bounded virtual graph, one persistent cooperative launch.
//
// Reference: pr::{sync,async}_push_{td,dd} (src/pr.cu:3-288) with init delta=0.15, value=0
// (src/eegraph.cu:1046-1062) and damping 0.85 (src/pr.cu:43). Its fixed point is
//     x_v = (1-d) + d * sum_{u->v} x_u / outdeg(u)        (mass of dangling vertices dropped)
// The reference applies the per-vertex update once per virtual part (src/pr.cu:28-56), which
// over-counts vertices with more than K out-edges; here each vertex is updated exactly once per sweep.
//
// GB300 form: Jacobi sweeps that PULL over the transposed virtual graph (parts of <= K in-edges).
//  * A warp owns chunks of 32 consecutive parts and keeps two chunks in flight: their part rows
//    (256-bit loads) and then all 2*K gathers of contrib[u] = x_u / outdeg(u) are issued before any
//    of them is consumed; the old value and out-degree of each chunk's segment ends are prefetched
//    alongside the gathers.
//  * Each lane sums its part's K values by a pairwise tree; parts of one vertex are combined by a
//    segmented warp scan of compensated (hi, lo) pairs.
//  * A vertex whose parts all sit in one chunk is finalised in place. A vertex whose parts span chunks
//    gets one FP64 atomic partial per chunk plus an arrival count; the warp that brings the count to
//    the number of chunks spanned finalises it. So a sweep needs ONE grid barrier.
//  * Stop test in FP64: ||x_{k+1}-x_k||_1 * d/(1-d) <= tol * ||x_{k+1}||_1 bounds the distance to the
//    fixed point (the Jacobi map contracts by d in the L1 norm).
//   SYNC variants: contrib double-buffered (deterministic Jacobi up to the FP64 partial order).
//   ASYNC variants: contrib updated in place (values of this sweep are used as soon as written; same
//   fixed point, fewer sweeps, order-dependent rounding).
#include <algorithm>
#include <cmath>

#include "internal.hpp"

namespace eeg {
namespace {

constexpr int PR_TPB = 1024;  // one CTA per SM: its shared memory holds the hot contributions
constexpr uint32_t PR_HOT_DEFAULT = 32768;
// chunks in flight per warp (K = 16 keeps one: its 16 ids + 16 gathered values already fill the registers)
template <int K>
struct InFlight {
    static constexpr int U = K >= 16 ? 1 : 2;
};

struct PRArgs {
    uint32_t n;
    uint32_t RP;
    const uint32_t* __restrict__ rvstart;
    const uint32_t* __restrict__ rvowner;
    const uint32_t* __restrict__ rvcol;   // transposed graph's neighbours, as ranks (see rank below)
    const uint2* __restrict__ info;       // per vertex: (rank in descending out-degree-class order, out-degree)
    uint32_t hot;                         // contributions of ranks < hot are staged in shared memory
    float* x;
    float* c0;
    float* c1;
    double* acc;       // FP64 partial sums of vertices whose parts span chunks
    uint32_t* arrive;  // chunks that have delivered their partial, per vertex
    uint32_t max_iters;
    PRCtrl* ctrl;
    float damping;
    float base;
    double tol;
    uint64_t timeout_ns;
    uint32_t inplace;
};

__device__ __forceinline__ void finalize(const PRArgs& a, uint32_t v, uint32_t rk, double sum, float xo, uint32_t od,
                                         float* cnext, double& r, double& nrm) {
    const float xn = a.base + a.damping * (float)sum;
    r += fabs((double)xn - (double)xo);
    nrm += (double)xn;
    a.x[v] = xn;
    cnext[rk] = od ? xn / (float)od : 0.f;
}

constexpr int XCAP = 64;  // per-warp list of (vertex, chunks spanned) awaiting their arrival count

// Count this warp's deliveries for the vertices in `xb` (their FP64 partials are already added): one
// fence makes all of the warp's partials visible first; a lane whose increment completes a vertex's
// count reads and clears the partial and finalises the vertex. Called by all 32 lanes, `nx` uniform.
template <class Fin>
__device__ __forceinline__ void settle_spanning(const PRArgs& a, const uint2* xb, uint32_t nx, uint32_t lane,
                                                Fin&& fin) {
    __syncwarp();
    __threadfence();
    for (uint32_t e = lane; e < nx; e += 32u) {
        const uint2 q = xb[e];
        if (atomicAdd(&a.arrive[q.x], 1u) + 1u == q.y) {
            __threadfence();
            const unsigned long long bits = atomicExch((unsigned long long*)&a.acc[q.x], 0ull);
            a.arrive[q.x] = 0u;
            fin(q.x, __longlong_as_double((long long)bits));
        }
    }
    __syncwarp();
}

template <int K>
__global__ void __launch_bounds__(PR_TPB, 1) k_pagerank(PRArgs a) {
    constexpr int PR_U = InFlight<K>::U;
    extern __shared__ float4 s_hot4[];  // contributions of the `hot` highest out-degree vertices
    const float* s_hot = reinterpret_cast<const float*>(s_hot4);
    __shared__ double s_red[2][PR_TPB / 32];
    __shared__ unsigned long long s_zero;
    __shared__ uint2 s_span[PR_TPB / 32][XCAP];
    __shared__ uint32_t s_next;  // next of this CTA's chunks to hand out in the current sweep
    __shared__ double s_rn[2];   // the last sweep's residual and norm
    uint2* xbuf = s_span[threadIdx.x >> 5];
    PRCtrl* ctrl = a.ctrl;
    const uint32_t gtid = blockIdx.x * PR_TPB + threadIdx.x;
    const uint32_t gthreads = gridDim.x * PR_TPB;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nchunks = (a.RP + 31u) / 32u;
    const uint64_t pol = l2_evict_first_policy();
    uint32_t epoch = 0;

    // ---- set-up: x0 = 1-d, contrib0, partial slots; count vertices without in-edges
    if (threadIdx.x == 0) s_zero = 0;
    __syncthreads();
    unsigned long long zero_in = 0;
    for (uint32_t v = gtid; v < a.n; v += gthreads) {
        a.x[v] = a.base;
        const uint2 inf = a.info[v];
        const uint32_t od = inf.y;
        const float c = od ? a.base / (float)od : 0.f;
        const uint32_t rk = inf.x;
        a.c0[rk] = c;
        a.c1[rk] = c;
        a.acc[v] = 0.0;
        a.arrive[v] = 0u;
        zero_in += (a.rvstart[v + 1] == a.rvstart[v]) ? 1ull : 0ull;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) zero_in += __shfl_down_sync(0xffffffffu, zero_in, off);
    if (lane == 0 && zero_in) atomicAdd(&s_zero, zero_in);
    __syncthreads();
    if (threadIdx.x == 0 && s_zero) atomicAdd(&ctrl->zero_in, s_zero);
    uint32_t s = 0;
    unsigned long long my_edges = 0;
    if (!grid_barrier_sync(&ctrl->bw, epoch, a.timeout_ns)) goto finish;
    {
        const double zero_norm = (double)*(volatile unsigned long long*)&ctrl->zero_in * (double)a.base;
        for (;; ++s) {
            if (s >= a.max_iters) {
                if (blockIdx.x == 0 && threadIdx.x == 0)
                    atomicCAS(&ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_ITER_CAP);
                break;
            }
            const uint32_t slot = s % 3u;
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                ctrl->resid[(s + 1u) % 3u] = 0.0;
                ctrl->norm[(s + 1u) % 3u] = 0.0;
            }
            // ccur is read through L1 (plain loads): the grid barrier's acquire makes the previous sweep's
            // values visible, and within a sweep they do not change (SYNC) or may be stale (ASYNC, allowed)
            const float* ccur = (s & 1u) && !a.inplace ? a.c1 : a.c0;
            float* cnext = a.inplace ? a.c0 : ((s & 1u) ? a.c0 : a.c1);
            double r = 0.0, nrm = 0.0;
            uint32_t nx = 0;  // warp-uniform fill of xbuf
            auto fin = [&](uint32_t vv, double sum) {
                const uint2 inf = __ldg(&a.info[vv]);
                finalize(a, vv, inf.x, sum, __ldcg(&a.x[vv]), inf.y, cnext, r, nrm);
            };
            // stage this sweep's hot contributions (the barrier before the sweep ordered every CTA's
            // writes of the previous sweep; ASYNC may see some of this sweep's, which it allows)
            {
                const float4* src4 = reinterpret_cast<const float4*>(ccur);
                for (uint32_t i = threadIdx.x; i < a.hot / 4u; i += PR_TPB) s_hot4[i] = src4[i];
                if (threadIdx.x == 0) s_next = 0u;
                __syncthreads();
            }

            // This CTA's share of the sweep is the strided chunk set blockIdx.x + i * gridDim.x (a mix of
            // hub and leaf regions, so CTAs get similar work); its warps draw from it through a shared
            // counter, so a warp never idles while another warp of the CTA still has chunks queued.
            const uint32_t my_chunks =
                nchunks > blockIdx.x ? (nchunks - blockIdx.x + gridDim.x - 1u) / gridDim.x : 0u;
            for (;;) {
                uint32_t i0 = 0;
                if (lane == 0) i0 = atomicAdd(&s_next, (uint32_t)PR_U);
                i0 = __shfl_sync(0xffffffffu, i0, 0);
                if (i0 >= my_chunks) break;
                uint32_t v[PR_U], col[PR_U][K], vb[PR_U];
                bool valid[PR_U];
#pragma unroll
                for (int u = 0; u < PR_U; ++u) {
                    const uint32_t ci = i0 + (uint32_t)u;
                    const uint32_t ch = blockIdx.x + ci * gridDim.x;
                    const uint32_t p = ch * 32u + lane;
                    valid[u] = ci < my_chunks && p < a.RP;
                    v[u] = vb[u] = 0xFFFFFFFFu;
                    if (valid[u]) {
                        v[u] = __ldg(&a.rvowner[p]);
                        ld_part<K>(a.rvcol + (size_t)p * K, col[u], pol);
                        // owners just outside the chunk: lane 0 the part before it, lane 31 the part after
                        if (lane == 0u && p > 0u) vb[u] = __ldg(&a.rvowner[p - 1u]);
                        if (lane == 31u && p + 1u < a.RP) vb[u] = __ldg(&a.rvowner[p + 1u]);
                    }
                }
                // padding slots gather 0 (adding an exact zero leaves the compensated sum unchanged),
                // so the id registers die here
                float y[PR_U][K];
                uint32_t nvalid = 0;
#pragma unroll
                for (int u = 0; u < PR_U; ++u)
#pragma unroll
                    for (int i = 0; i < K; ++i) {
                        const bool ok = valid[u] && col[u][i] != NO_EDGE;
                        nvalid += ok ? 1u : 0u;
                        y[u][i] = ok ? (col[u][i] < a.hot ? s_hot[col[u][i]] : ccur[col[u][i]]) : 0.f;
                    }
                my_edges += nvalid;
                // segment ends: prefetch what finalisation needs while the gathers are in flight
                bool last[PR_U];
                float xo[PR_U];
                uint32_t od[PR_U], rk[PR_U];
#pragma unroll
                for (int u = 0; u < PR_U; ++u) {
                    const uint32_t vn = __shfl_down_sync(0xffffffffu, v[u], 1);
                    last[u] = valid[u] && (lane == 31u || vn != v[u]);
                    xo[u] = 0.f;
                    od[u] = 0u;
                    rk[u] = 0u;
                    if (last[u]) {
                        const uint2 inf = __ldg(&a.info[v[u]]);
                        rk[u] = inf.x;
                        od[u] = inf.y;
                        xo[u] = __ldcg(&a.x[v[u]]);
                    }
                }
#pragma unroll
                for (int u = 0; u < PR_U; ++u) {
                    // the part's K values by a pairwise tree (rounding error <= log2(K) ulps of the
                    // part sum); parts and chunks are then combined with compensation
#pragma unroll
                    for (int w = K / 2; w >= 1; w >>= 1)
#pragma unroll
                        for (int i = 0; i < w; ++i) y[u][i] = __fadd_rn(y[u][i], y[u][i + w]);
                    float hi = y[u][0], lo = 0.f;
                    // segmented inclusive scan over lanes of the same vertex (a vertex's parts are contiguous):
                    // segment heads from one shuffle + ballot, and only as many steps as the longest segment
                    const uint32_t vprev = __shfl_up_sync(0xffffffffu, v[u], 1);
                    const uint32_t heads = __ballot_sync(0xffffffffu, lane == 0u || vprev != v[u]);
                    const uint32_t seg0 = 31u - __clz(heads & (0xffffffffu >> (31u - lane)));
                    const uint32_t span = __reduce_max_sync(0xffffffffu, lane - seg0 + 1u);
                    for (uint32_t off = 1; off < span; off <<= 1) {
                        const float ho = __shfl_up_sync(0xffffffffu, hi, off);
                        const float lo2 = __shfl_up_sync(0xffffffffu, lo, off);
                        if (lane >= seg0 + off) pair_add(hi, lo, ho, lo2);
                    }
                    bool spans = false;
                    uint32_t need = 0;
                    const uint32_t before0 = __shfl_sync(0xffffffffu, vb[u], 0);
                    if (last[u]) {
                        // the vertex began before this chunk, or continues after it
                        if (!((seg0 == 0u && before0 == v[u]) || (lane == 31u && vb[u] == v[u]))) {
                            finalize(a, v[u], rk[u], (double)hi + (double)lo, xo[u], od[u], cnext, r, nrm);
                        } else {  // partial now, arrival counted in the warp's next settle
                            atomicAdd(&a.acc[v[u]], (double)hi + (double)lo);
                            spans = true;
                            need = (__ldg(&a.rvstart[v[u] + 1]) - 1u) / 32u - __ldg(&a.rvstart[v[u]]) / 32u + 1u;
                        }
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, spans);
                    if (m) {
                        const uint32_t c = __popc(m);
                        if (nx + c > (uint32_t)XCAP) {
                            settle_spanning(a, xbuf, nx, lane, fin);
                            nx = 0;
                        }
                        if (spans) xbuf[nx + __popc(m & ((1u << lane) - 1u))] = make_uint2(v[u], need);
                        nx += c;
                    }
                }
            }
            if (nx) settle_spanning(a, xbuf, nx, lane, fin);
            // CTA reduction of the FP64 residual / norm, one atomic per CTA
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                r += __shfl_down_sync(0xffffffffu, r, off);
                nrm += __shfl_down_sync(0xffffffffu, nrm, off);
            }
            if (lane == 0) {
                s_red[0][threadIdx.x >> 5] = r;
                s_red[1][threadIdx.x >> 5] = nrm;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                double rr = 0.0, nn = 0.0;
                for (int w = 0; w < PR_TPB / 32; ++w) {
                    rr += s_red[0][w];
                    nn += s_red[1][w];
                }
                atomicAdd(&ctrl->resid[slot], rr);
                atomicAdd(&ctrl->norm[slot], nn);
            }
            if (!grid_barrier_sync(&ctrl->bw, epoch, a.timeout_ns)) break;
            // one thread per CTA reads the sweep's totals (every warp reading the same two words would
            // queue at one L2 slice); the CTA takes them from shared memory
            if (threadIdx.x == 0) {
                s_rn[0] = *(volatile double*)&ctrl->resid[slot];
                s_rn[1] = *(volatile double*)&ctrl->norm[slot];
            }
            __syncthreads();
            const double resid = s_rn[0];
            const double norm = s_rn[1] + zero_norm;
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                ctrl->last_resid = resid;
                ctrl->last_norm = norm;
            }
            if ((double)a.damping / (1.0 - (double)a.damping) * resid <= a.tol * norm) {
                ++s;
                break;
            }
        }
    }
finish:
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) my_edges += __shfl_down_sync(0xffffffffu, my_edges, off);
    if (lane == 0 && my_edges) atomicAdd(&ctrl->edges_scanned, my_edges);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->iterations = s;
}

template <int K>
eeg_status launch_pr(const PRArgs& args, int device, uint32_t bps, uint32_t hot_limit, cudaStream_t st) {
    auto kern = k_pagerank<K>;
    // shared memory left after the static arrays holds the hot contributions (multiple of 4 floats)
    cudaFuncAttributes fa{};
    EEG_CUDA(cudaFuncGetAttributes(&fa, kern));
    int optin = 0;
    EEG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    const size_t room = optin > (int)fa.sharedSizeBytes + 1024 ? (size_t)optin - fa.sharedSizeBytes - 1024 : 0;
    PRArgs a = args;
    // default 32K vertices (128 KB): a larger carve-out shrinks L1 below what the cold gathers and the
    // per-vertex loads need (measured on R-MAT s22: 128 KB best, 210 KB 35 % slower than none)
    size_t hot = std::min<size_t>(args.n, room / sizeof(float));
    hot = std::min<size_t>(hot, hot_limit ? hot_limit : PR_HOT_DEFAULT);
    a.hot = (uint32_t)(hot & ~(size_t)3);
    const size_t dyn = (size_t)a.hot * sizeof(float);
    EEG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    int per_sm = 0;
    EEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PR_TPB, dyn));
    if (per_sm <= 0) {
        set_last_error("pagerank kernel does not fit on an SM");
        return EEG_ERR_CUDA;
    }
    if (bps > 0 && (int)bps < per_sm) per_sm = (int)bps;
    uint64_t blocks = (uint64_t)per_sm * sm_count(device);
    const uint64_t work = std::max<uint64_t>(args.RP, args.n);
    const uint64_t need = (work + PR_TPB - 1) / PR_TPB;
    if (need < blocks) blocks = std::max<uint64_t>(need, 1);
    void* params[] = {(void*)&a};
    EEG_CUDA(cudaLaunchCooperativeKernel((const void*)kern, dim3((unsigned)blocks), dim3(PR_TPB), params, dyn, st));
    return EEG_OK;
}

// ---- degree-class relabelling of the transposed graph's neighbour ids (once per graph)
constexpr uint32_t RCLS = 129;  // quarter-octave out-degree classes, descending; class 128 = no out-edges
constexpr uint32_t RTILE = 4096;

__device__ __forceinline__ uint32_t deg_class(uint32_t d) {
    if (d == 0) return RCLS - 1;
    const uint32_t lg = 31u - __clz(d);
    const uint32_t frac = lg >= 2 ? (d >> (lg - 2)) & 3u : (d << (2 - lg)) & 3u;
    return 127u - (lg * 4u + frac);
}

__global__ void k_rank_hist(uint32_t n, const uint32_t* __restrict__ deg, uint32_t* hist) {
    __shared__ uint32_t sh[RCLS];
    for (uint32_t i = threadIdx.x; i < RCLS; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        atomicAdd(&sh[deg_class(deg[v])], 1u);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < RCLS; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[i], sh[i]);
}
// hist -> exclusive class offsets (in place), cursors zeroed
__global__ void k_rank_base(uint32_t* hist, uint32_t* cursor) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t i = 0; i < RCLS; ++i) {
            const uint32_t c = hist[i];
            hist[i] = run;
            run += c;
            cursor[i] = 0;
        }
    }
}
// rank[v] = class offset + a slot reserved per CTA and class (order within a class is not fixed;
// results do not depend on it)
__global__ void k_rank_scatter(uint32_t n, const uint32_t* __restrict__ deg, const uint32_t* __restrict__ base,
                               uint32_t* cursor, uint32_t* rank) {
    __shared__ uint32_t s_cnt[RCLS], s_off[RCLS];
    for (uint64_t t0 = (uint64_t)blockIdx.x * RTILE; t0 < n; t0 += (uint64_t)gridDim.x * RTILE) {
        for (uint32_t i = threadIdx.x; i < RCLS; i += blockDim.x) s_cnt[i] = 0;
        __syncthreads();
        constexpr int PER = RTILE / 256;
        uint32_t cls[PER], loc[PER];
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const uint64_t v = t0 + (uint64_t)j * blockDim.x + threadIdx.x;
            cls[j] = v < n ? deg_class(deg[v]) : RCLS;
            loc[j] = v < n ? atomicAdd(&s_cnt[cls[j]], 1u) : 0u;
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < RCLS; i += blockDim.x)
            s_off[i] = s_cnt[i] ? base[i] + atomicAdd(&cursor[i], s_cnt[i]) : 0u;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const uint64_t v = t0 + (uint64_t)j * blockDim.x + threadIdx.x;
            if (v < n) rank[v] = s_off[cls[j]] + loc[j];
        }
        __syncthreads();
    }
}
__global__ void k_rank_info(uint32_t n, const uint32_t* __restrict__ rank, const uint32_t* __restrict__ deg,
                            uint2* __restrict__ info) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        info[v] = make_uint2(rank[v], deg[v]);
}
__global__ void k_rank_cols(uint64_t slots, const uint32_t* __restrict__ col, const uint32_t* __restrict__ rank,
                            uint32_t* __restrict__ out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = col[i];
        out[i] = c == NO_EDGE ? NO_EDGE : rank[c];
    }
}

}  // namespace

static eeg_status ensure_pr_ws(eeg_vgraph* vg) {
    Workspace& ws = vg->ws;
    const size_t n = std::max<uint32_t>(vg->n, 1);
    if (!ws.x) EEG_TRY(vg_alloc(vg, (void**)&ws.x, sizeof(float) * n));
    if (!ws.contrib[0]) EEG_TRY(vg_alloc(vg, (void**)&ws.contrib[0], sizeof(float) * n));
    if (!ws.contrib[1]) EEG_TRY(vg_alloc(vg, (void**)&ws.contrib[1], sizeof(float) * n));
    if (!ws.acc) EEG_TRY(vg_alloc(vg, (void**)&ws.acc, sizeof(double) * n));
    if (!ws.arrive) EEG_TRY(vg_alloc(vg, (void**)&ws.arrive, sizeof(uint32_t) * n));
    if (!ws.pctrl) EEG_CUDA(cudaMalloc((void**)&ws.pctrl, sizeof(PRCtrl)));
    if (!ws.ev[0]) {
        EEG_CUDA(cudaEventCreate(&ws.ev[0]));
        EEG_CUDA(cudaEventCreate(&ws.ev[1]));
    }
    return EEG_OK;
}

// Ranks by descending out-degree class and the transposed graph's neighbour ids rewritten as ranks.
static eeg_status ensure_pr_rank(eeg_vgraph* vg, cudaStream_t st) {
    Workspace& ws = vg->ws;
    if (ws.pr_rcol) return EEG_OK;
    const uint32_t n = vg->n;
    const uint64_t slots = (uint64_t)vg->rev.P * vg->K;
    EEG_TRY(vg_alloc(vg, (void**)&ws.pr_rank, sizeof(uint32_t) * std::max<uint32_t>(n, 1) + 2 * RCLS * sizeof(uint32_t)));
    uint32_t* hist = ws.pr_rank + n;
    uint32_t* cursor = hist + RCLS;
    uint32_t* rcol = nullptr;
    EEG_TRY(vg_alloc(vg, (void**)&rcol, sizeof(uint32_t) * std::max<uint64_t>(slots, 4)));
    EEG_CUDA(cudaMemsetAsync(hist, 0, RCLS * sizeof(uint32_t), st));
    const unsigned g = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)sm_count(vg->device) * 8));
    k_rank_hist<<<g, 256, 0, st>>>(n, vg->fwd.deg, hist);
    k_rank_base<<<1, 32, 0, st>>>(hist, cursor);
    const unsigned gt = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + RTILE - 1) / RTILE, (uint64_t)sm_count(vg->device) * 8));
    k_rank_scatter<<<gt, 256, 0, st>>>(n, vg->fwd.deg, hist, cursor, ws.pr_rank);
    EEG_TRY(vg_alloc(vg, (void**)&ws.pr_info, sizeof(uint2) * std::max<uint32_t>(n, 1)));
    k_rank_info<<<g, 256, 0, st>>>(n, ws.pr_rank, vg->fwd.deg, ws.pr_info);
    if (slots) {
        const unsigned gs = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((slots + 255) / 256, (uint64_t)sm_count(vg->device) * 16));
        k_rank_cols<<<gs, 256, 0, st>>>(slots, vg->rev.vcol, ws.pr_rank, rcol);
    }
    EEG_CUDA(cudaGetLastError());
    ws.pr_rcol = rcol;
    return EEG_OK;
}

eeg_status run_pagerank(eeg_vgraph* vg, eeg_variant variant, const eeg_options& o, cudaStream_t st,
                        eeg_result* res) {
    if (!vg->has_rev) {
        set_last_error("PageRank needs the transposed graph (build with EEG_VG_REVERSE)");
        return EEG_ERR_INVALID;
    }
    if (vg->n == 0) {
        set_last_error("empty graph");
        return EEG_ERR_INVALID;
    }
    EEG_TRY(ensure_pr_ws(vg));
    EEG_TRY(ensure_pr_rank(vg, st));
    Workspace& ws = vg->ws;
    const float damping = o.pr_damping > 0.f ? o.pr_damping : 0.85f;
    EEG_CUDA(cudaMemsetAsync(ws.pctrl, 0, sizeof(PRCtrl), st));
    PRArgs a{};
    a.n = vg->n;
    a.RP = (uint32_t)vg->rev.P;
    a.rvstart = vg->rev.vstart;
    a.rvowner = vg->rev.vowner;
    a.rvcol = ws.pr_rcol;
    a.info = ws.pr_info;
    a.x = ws.x;
    a.c0 = ws.contrib[0];
    a.c1 = ws.contrib[1];
    a.acc = ws.acc;
    a.arrive = ws.arrive;
    a.max_iters = o.max_iterations ? o.max_iterations : 10000u;
    a.ctrl = ws.pctrl;
    a.damping = damping;
    a.base = 1.0f - damping;
    a.tol = o.pr_tolerance > 0.f ? (double)o.pr_tolerance : 1e-7;
    a.timeout_ns = wait_limit_ns(o);
    a.inplace = (variant == EEG_ASYNC_PUSH_TD || variant == EEG_ASYNC_PUSH_DD) ? 1u : 0u;

    EEG_CUDA(cudaEventRecord(ws.ev[0], st));
    eeg_status s;
    switch (vg->K) {
        case 4: s = launch_pr<4>(a, vg->device, o.blocks_per_sm, o.pr_hot_limit, st); break;
        case 8: s = launch_pr<8>(a, vg->device, o.blocks_per_sm, o.pr_hot_limit, st); break;
        case 16: s = launch_pr<16>(a, vg->device, o.blocks_per_sm, o.pr_hot_limit, st); break;
        default: set_last_error("K must be 4, 8 or 16"); return EEG_ERR_UNSUPPORTED;
    }
    if (s != EEG_OK) return s;
    EEG_CUDA(cudaEventRecord(ws.ev[1], st));
    PRCtrl hc;
    EEG_CUDA(cudaMemcpyAsync(&hc, ws.pctrl, sizeof(PRCtrl), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    EEG_CUDA(cudaEventElapsedTime(&ms, ws.ev[0], ws.ev[1]));
    if (res) {
        res->kernel_ms = ms;
        res->iterations = hc.iterations;
        res->edges_scanned = hc.edges_scanned;
        res->parts_processed = (uint64_t)hc.iterations * vg->rev.P;
        res->pr_residual = hc.last_resid;
        res->pr_l1_norm = hc.last_norm;
        res->launches = 1;
    }
    if (hc.bw.status == DEV_TIMEOUT) {
        set_last_error("grid barrier wait exceeded the timeout");
        return EEG_ERR_TIMEOUT;
    }
    if (hc.bw.status == DEV_ITER_CAP) {
        set_last_error("PageRank did not reach the tolerance within the sweep cap");
        return EEG_ERR_ITER_CAP;
    }
    return EEG_OK;
}

}  // namespace eeg
