// pagerank.cu -- PageRank over the K-bounded virtual graph, one persistent cooperative launch.
//
// Reference: pr::{sync,async}_push_{td,dd} (src/pr.cu:3-288) with init delta=0.15, value=0
// (src/eegraph.cu:1046-1062) and damping 0.85 (src/pr.cu:43). Its fixed point is
//     x_v = (1-d) + d * sum_{u->v} x_u / outdeg(u)        (mass of dangling vertices dropped)
// The reference applies the per-vertex update once per virtual part (src/pr.cu:28-56), which
// over-counts vertices with more than K out-edges; here each vertex is updated exactly once per sweep.
//
// GB300 form: Jacobi sweeps that PULL over the transposed virtual graph (parts of <= K in-edges).
// A warp owns 32 consecutive parts: each lane sums its part with a compensated (two-sum) FP32
// accumulation of contrib[u] = x_u / outdeg(u); parts of one vertex are combined by a segmented
// warp scan; a vertex whose parts all sit in the warp's chunk is finalised in place, a vertex whose
// parts span chunks adds its pair sum to an FP64 slot that a second phase finalises. The stop test
// uses FP64 reductions: ||x_{k+1}-x_k||_1 * d/(1-d) <= tol * ||x_{k+1}||_1 bounds the distance to the
// fixed point (the Jacobi map contracts by d in the L1 norm).
//   SYNC variants: contrib double-buffered (deterministic Jacobi).
//   ASYNC variants: contrib updated in place (Gauss-Seidel-like: values of this sweep are used as
//   soon as they are written; same fixed point, fewer sweeps, order-dependent rounding).
#include <algorithm>
#include <cmath>

#include "internal.hpp"

namespace eeg {
namespace {

constexpr int PR_TPB = 512;

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
    double* acc;
    const uint32_t* __restrict__ cross;
    uint32_t ncross;
    uint32_t max_iters;
    PRCtrl* ctrl;
    float damping;
    float base;
    double tol;
    double zero_in_norm;
    uint64_t timeout_ns;
    uint32_t inplace;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}
// (h1,l1) + (h2,l2) -> normalised pair
__device__ __forceinline__ void pair_add(float& h1, float& l1, float h2, float l2) {
    float s, e;
    two_sum(h1, h2, s, e);
    const float t = __fadd_rn(__fadd_rn(l1, l2), e);
    h1 = __fadd_rn(s, t);
    l1 = __fsub_rn(t, __fsub_rn(h1, s));
}

__device__ __forceinline__ void finalize(const PRArgs& a, uint32_t v, double sum, float* cnext, double& r,
                                         double& nrm) {
    const float xn = a.base + a.damping * (float)sum;
    const float xo = __ldcg(&a.x[v]);
    r += fabs((double)xn - (double)xo);
    nrm += (double)xn;
    a.x[v] = xn;
    const uint32_t od = __ldg(&a.outdeg[v]);
    cnext[v] = od ? xn / (float)od : 0.f;
}

template <int K>
__global__ void __launch_bounds__(PR_TPB) k_pagerank(PRArgs a) {
    __shared__ double s_red[2][PR_TPB / 32];
    PRCtrl* ctrl = a.ctrl;
    const uint32_t gtid = blockIdx.x * PR_TPB + threadIdx.x;
    const uint32_t gthreads = gridDim.x * PR_TPB;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gwarp = gtid >> 5, nwarps = gthreads >> 5;
    const uint32_t nchunks = (a.RP + 31u) / 32u;
    const uint64_t pol = l2_evict_first_policy();
    uint32_t epoch = 0;

    for (uint32_t v = gtid; v < a.n; v += gthreads) {
        a.x[v] = a.base;
        const uint32_t od = a.outdeg[v];
        const float c = od ? a.base / (float)od : 0.f;
        a.c0[v] = c;
        a.c1[v] = c;
        a.acc[v] = 0.0;
    }
    uint32_t s = 0;
    unsigned long long my_edges = 0;
    if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) goto finish;

    for (;; ++s) {
        if (s >= a.max_iters) {
            if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_ITER_CAP);
            break;
        }
        const uint32_t slot = s % 3u;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctrl->resid[(s + 1u) % 3u] = 0.0;
            ctrl->norm[(s + 1u) % 3u] = 0.0;
        }
        const float* __restrict__ ccur = (s & 1u) && !a.inplace ? a.c1 : a.c0;
        float* cnext = a.inplace ? a.c0 : ((s & 1u) ? a.c0 : a.c1);
        double r = 0.0, nrm = 0.0;

        // ---- phase P: pull over parts
        for (uint32_t ch = gwarp; ch < nchunks; ch += nwarps) {
            const uint32_t p = ch * 32u + lane;
            const bool valid = p < a.RP;
            uint32_t v = 0xFFFFFFFFu;
            float hi = 0.f, lo = 0.f;
            if (valid) {
                v = __ldg(&a.rvowner[p]);
                uint32_t col[K];
                ld_part<K>(a.rvcol + (size_t)p * K, col, pol);
                float y[K];
#pragma unroll
                for (int i = 0; i < K; ++i) y[i] = col[i] != NO_EDGE ? __ldcg(&ccur[col[i]]) : 0.f;
#pragma unroll
                for (int i = 0; i < K; ++i) {
                    if (col[i] == NO_EDGE) break;
                    ++my_edges;
                    float t, e;
                    two_sum(hi, y[i], t, e);
                    hi = t;
                    lo = __fadd_rn(lo, e);
                }
            }
            // segmented inclusive scan over lanes holding the same vertex (parts of a vertex are contiguous)
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t vo = __shfl_up_sync(0xffffffffu, v, off);
                const float ho = __shfl_up_sync(0xffffffffu, hi, off);
                const float lo2 = __shfl_up_sync(0xffffffffu, lo, off);
                if (lane >= (uint32_t)off && vo == v) pair_add(hi, lo, ho, lo2);
            }
            const uint32_t vnext = __shfl_down_sync(0xffffffffu, v, 1);
            const uint32_t vprev = __shfl_up_sync(0xffffffffu, v, 1);
            const bool head = (lane == 0) || (vprev != v);
            const uint32_t head_mask = __ballot_sync(0xffffffffu, head);
            const bool last = (lane == 31) || (vnext != v);
            if (valid && last) {
                const uint32_t below = head_mask & (0xffffffffu >> (31u - lane));
                const uint32_t head_lane = 31u - __clz(below);
                bool complete = true;
                if (head_lane == 0 && __ldg(&a.rvstart[v]) < ch * 32u) complete = false;
                if (lane == 31 && __ldg(&a.rvstart[v + 1]) > ch * 32u + 32u) complete = false;
                if (complete) finalize(a, v, (double)hi + (double)lo, cnext, r, nrm);
                else atomicAdd(&a.acc[v], (double)hi + (double)lo);
            }
        }
        if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) break;

        // ---- phase F: vertices whose parts span warp chunks
        for (uint32_t i = gtid; i < a.ncross; i += gthreads) {
            const uint32_t v = a.cross[i];
            const double sum = __ldcg(&a.acc[v]);
            a.acc[v] = 0.0;
            finalize(a, v, sum, cnext, r, nrm);
        }
        // block reduction of the FP64 residual / norm, one atomic per CTA
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
        const double norm = *(volatile double*)&ctrl->norm[slot] + a.zero_in_norm;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctrl->last_resid = resid;
            ctrl->last_norm = norm;
        }
        if ((double)a.damping / (1.0 - (double)a.damping) * resid <= a.tol * norm) {
            ++s;
            break;
        }
    }
finish:
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) my_edges += __shfl_down_sync(0xffffffffu, my_edges, off);
    if (lane == 0 && my_edges) atomicAdd(&ctrl->edges_scanned, my_edges);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->iterations = s;
}

// Vertices whose in-parts are not inside one 32-part chunk, and the number of vertices without
// in-edges (their value stays 1-d, a constant part of ||x||_1).
__global__ void k_cross(const uint32_t* __restrict__ rvstart, uint32_t n, uint32_t* cross, uint32_t* ncross,
                        unsigned long long* zero_in) {
    unsigned long long z = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const uint32_t a = rvstart[v], b = rvstart[v + 1];
        if (b == a) {
            ++z;
            continue;
        }
        if (a / 32u != (b - 1u) / 32u) cross[atomicAdd(ncross, 1u)] = v;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) z += __shfl_down_sync(0xffffffffu, z, off);
    if ((threadIdx.x & 31u) == 0 && z) atomicAdd(zero_in, z);
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

static eeg_status ensure_pr_ws(eeg_vgraph* vg, cudaStream_t st, uint32_t* launched) {
    Workspace& ws = vg->ws;
    const size_t n = std::max<uint32_t>(vg->n, 1);
    if (!ws.x) EEG_TRY(vg_alloc(vg, (void**)&ws.x, sizeof(float) * n));
    if (!ws.contrib[0]) EEG_TRY(vg_alloc(vg, (void**)&ws.contrib[0], sizeof(float) * n));
    if (!ws.contrib[1]) EEG_TRY(vg_alloc(vg, (void**)&ws.contrib[1], sizeof(float) * n));
    if (!ws.acc) EEG_TRY(vg_alloc(vg, (void**)&ws.acc, sizeof(double) * n));
    if (!ws.pctrl) EEG_CUDA(cudaMalloc((void**)&ws.pctrl, sizeof(PRCtrl)));
    if (!ws.ev[0]) {
        EEG_CUDA(cudaEventCreate(&ws.ev[0]));
        EEG_CUDA(cudaEventCreate(&ws.ev[1]));
    }
    if (!ws.cross) {
        EEG_TRY(vg_alloc(vg, (void**)&ws.cross, sizeof(uint32_t) * n));
        unsigned long long* cnt = nullptr;
        EEG_CUDA(cudaMalloc((void**)&cnt, 16));
        EEG_CUDA(cudaMemsetAsync(cnt, 0, 16, st));
        const unsigned blocks = (unsigned)std::min<uint64_t>((vg->n + 255) / 256 + 1, (uint64_t)sm_count(vg->device) * 8);
        k_cross<<<blocks, 256, 0, st>>>(vg->rev.vstart, vg->n, ws.cross, (uint32_t*)cnt, cnt + 1);
        EEG_CUDA(cudaGetLastError());
        unsigned long long h[2];
        EEG_CUDA(cudaMemcpyAsync(h, cnt, 16, cudaMemcpyDeviceToHost, st));
        EEG_CUDA(cudaStreamSynchronize(st));
        ws.ncross = (uint32_t)(h[0] & 0xFFFFFFFFull);
        ws.zero_in = h[1];
        cudaFree(cnt);
        *launched += 1;
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
    uint32_t launches = 1;  // the persistent kernel (+1 the first time: the chunk-crossing list)
    EEG_TRY(ensure_pr_ws(vg, st, &launches));
    Workspace& ws = vg->ws;
    const float damping = o.pr_damping > 0.f ? o.pr_damping : 0.85f;
    const float base = 1.0f - damping;
    ws.zero_in_norm = (double)ws.zero_in * (double)base;
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
    a.cross = ws.cross;
    a.ncross = ws.ncross;
    a.max_iters = o.max_iterations ? o.max_iterations : 10000u;
    a.ctrl = ws.pctrl;
    a.damping = damping;
    a.base = base;
    a.tol = o.pr_tolerance > 0.f ? (double)o.pr_tolerance : 1e-7;
    a.zero_in_norm = ws.zero_in_norm;
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
        res->launches = launches;
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
