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
//  * Each lane sums its part with a compensated (two-sum) FP32 accumulation; parts of one vertex are
//    combined by a segmented warp scan of (hi, lo) pairs.
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

constexpr int PR_TPB = 512;
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
    const uint32_t* __restrict__ rvcol;
    const uint32_t* __restrict__ outdeg;
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

__device__ __forceinline__ void finalize(const PRArgs& a, uint32_t v, double sum, float xo, uint32_t od, float* cnext,
                                         double& r, double& nrm) {
    const float xn = a.base + a.damping * (float)sum;
    r += fabs((double)xn - (double)xo);
    nrm += (double)xn;
    a.x[v] = xn;
    cnext[v] = od ? xn / (float)od : 0.f;
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
__global__ void __launch_bounds__(PR_TPB, 2) k_pagerank(PRArgs a) {
    constexpr int PR_U = InFlight<K>::U;
    __shared__ double s_red[2][PR_TPB / 32];
    __shared__ unsigned long long s_zero;
    __shared__ uint2 s_span[PR_TPB / 32][XCAP];
    uint2* xbuf = s_span[threadIdx.x >> 5];
    PRCtrl* ctrl = a.ctrl;
    const uint32_t gtid = blockIdx.x * PR_TPB + threadIdx.x;
    const uint32_t gthreads = gridDim.x * PR_TPB;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gwarp = gtid >> 5, nwarps = gthreads >> 5;
    const uint32_t nchunks = (a.RP + 31u) / 32u;
    const uint64_t pol = l2_evict_first_policy();
    uint32_t epoch = 0;

    // ---- set-up: x0 = 1-d, contrib0, partial slots; count vertices without in-edges
    if (threadIdx.x == 0) s_zero = 0;
    __syncthreads();
    unsigned long long zero_in = 0;
    for (uint32_t v = gtid; v < a.n; v += gthreads) {
        a.x[v] = a.base;
        const uint32_t od = a.outdeg[v];
        const float c = od ? a.base / (float)od : 0.f;
        a.c0[v] = c;
        a.c1[v] = c;
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
    if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) goto finish;
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
                finalize(a, vv, sum, __ldcg(&a.x[vv]), __ldg(&a.outdeg[vv]), cnext, r, nrm);
            };

            for (uint32_t base = gwarp; base < nchunks; base += nwarps * PR_U) {
                uint32_t v[PR_U], col[PR_U][K];
                bool valid[PR_U];
#pragma unroll
                for (int u = 0; u < PR_U; ++u) {
                    const uint32_t ch = base + (uint32_t)u * nwarps;
                    const uint32_t p = ch * 32u + lane;
                    valid[u] = ch < nchunks && p < a.RP;
                    v[u] = 0xFFFFFFFFu;
                    if (valid[u]) {
                        v[u] = __ldg(&a.rvowner[p]);
                        ld_part<K>(a.rvcol + (size_t)p * K, col[u], pol);
                    }
                }
                float y[PR_U][K];
#pragma unroll
                for (int u = 0; u < PR_U; ++u)
#pragma unroll
                    for (int i = 0; i < K; ++i)
                        y[u][i] = (valid[u] && col[u][i] != NO_EDGE) ? ccur[col[u][i]] : 0.f;
                // segment ends: prefetch what finalisation needs while the gathers are in flight
                bool last[PR_U];
                float xo[PR_U];
                uint32_t od[PR_U], vs0[PR_U], vs1[PR_U];
#pragma unroll
                for (int u = 0; u < PR_U; ++u) {
                    const uint32_t vn = __shfl_down_sync(0xffffffffu, v[u], 1);
                    last[u] = valid[u] && (lane == 31u || vn != v[u]);
                    xo[u] = 0.f;
                    od[u] = 0u;
                    vs0[u] = vs1[u] = 0u;
                    if (last[u]) {
                        xo[u] = __ldcg(&a.x[v[u]]);
                        od[u] = __ldg(&a.outdeg[v[u]]);
                        vs0[u] = __ldg(&a.rvstart[v[u]]);
                        vs1[u] = __ldg(&a.rvstart[v[u] + 1]);
                    }
                }
#pragma unroll
                for (int u = 0; u < PR_U; ++u) {
                    float hi = 0.f, lo = 0.f;
#pragma unroll
                    for (int i = 0; i < K; ++i) {
                        if (!valid[u] || col[u][i] == NO_EDGE) break;
                        ++my_edges;
                        float t, e;
                        two_sum(hi, y[u][i], t, e);
                        hi = t;
                        lo = __fadd_rn(lo, e);
                    }
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
                    if (last[u]) {
                        const uint32_t ch = base + (uint32_t)u * nwarps;
                        const uint32_t first_chunk = vs0[u] / 32u, last_chunk = (vs1[u] - 1u) / 32u;
                        if (first_chunk == ch && last_chunk == ch) {
                            finalize(a, v[u], (double)hi + (double)lo, xo[u], od[u], cnext, r, nrm);
                        } else {  // partial now, arrival counted in the warp's next settle
                            atomicAdd(&a.acc[v[u]], (double)hi + (double)lo);
                            spans = true;
                            need = last_chunk - first_chunk + 1u;
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
            if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) break;
            const double resid = *(volatile double*)&ctrl->resid[slot];
            const double norm = *(volatile double*)&ctrl->norm[slot] + zero_norm;
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
eeg_status launch_pr(const PRArgs& args, int device, uint32_t bps, cudaStream_t st) {
    auto kern = k_pagerank<K>;
    int per_sm = 0;
    EEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PR_TPB, 0));
    if (per_sm <= 0) {
        set_last_error("pagerank kernel does not fit on an SM");
        return EEG_ERR_CUDA;
    }
    if (bps > 0 && (int)bps < per_sm) per_sm = (int)bps;
    uint64_t blocks = (uint64_t)per_sm * sm_count(device);
    const uint64_t work = std::max<uint64_t>(args.RP, args.n);
    const uint64_t need = (work + PR_TPB - 1) / PR_TPB;
    if (need < blocks) blocks = std::max<uint64_t>(need, 1);
    PRArgs a = args;
    void* params[] = {(void*)&a};
    EEG_CUDA(cudaLaunchCooperativeKernel((const void*)kern, dim3((unsigned)blocks), dim3(PR_TPB), params, 0, st));
    return EEG_OK;
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
    Workspace& ws = vg->ws;
    const float damping = o.pr_damping > 0.f ? o.pr_damping : 0.85f;
    EEG_CUDA(cudaMemsetAsync(ws.pctrl, 0, sizeof(PRCtrl), st));
    PRArgs a{};
    a.n = vg->n;
    a.RP = (uint32_t)vg->rev.P;
    a.rvstart = vg->rev.vstart;
    a.rvowner = vg->rev.vowner;
    a.rvcol = vg->rev.vcol;
    a.outdeg = vg->fwd.deg;
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
    a.timeout_ns = (uint64_t)(o.timeout_ms ? o.timeout_ms : 10000u) * 1000000ull;
    a.inplace = (variant == EEG_ASYNC_PUSH_TD || variant == EEG_ASYNC_PUSH_DD) ? 1u : 0u;

    EEG_CUDA(cudaEventRecord(ws.ev[0], st));
    eeg_status s;
    switch (vg->K) {
        case 4: s = launch_pr<4>(a, vg->device, o.blocks_per_sm, st); break;
        case 8: s = launch_pr<8>(a, vg->device, o.blocks_per_sm, st); break;
        case 16: s = launch_pr<16>(a, vg->device, o.blocks_per_sm, st); break;
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
