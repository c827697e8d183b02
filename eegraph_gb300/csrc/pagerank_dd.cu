// pagerank_dd.cu -- data-driven PageRank: a residual frontier over the forward virtual graph.
//
// Reference: pr::sync_push_dd and pr::async_push_dd (src/pr.cu:110-169, 227-288) with their driver
// (src/eegraph.cu:1046-1232). Every vertex holds a residual `delta` (initially 1-d = 0.15) and a value
// (initially 0); a vertex whose residual exceeds the activation threshold `acc` (--accuracy,
// src/argument_parsing.cpp:119-121) adds it to its value and pushes d * delta / outdeg to each
// out-neighbour, and only vertices that received a push in the previous round are looked at again.
// Its fixed point is the one of the topology-driven kernels, x = (1-d) + d A^T D^-1 x (the mass of
// vertices without out-edges dropped): at every moment x* = x + (I - d P^T)^-1 r, so stopping when no
// residual exceeds acc leaves ||x* - x||_1 <= ||r||_1 / (1-d).
//
// GB300 form: one cooperative persistent launch; each round has two phases separated by the bounded
// grid barrier.
//   A (vertices): a dense scan of the residuals -- every vertex whose residual t exceeds acc (no push
//     lands in this phase, so a plain read and reset is exact) adds t to its FP64 value, records its push
//     amount d * t / outdeg, and its parts join the round's part queue (one reservation per warp; the
//     whole warp writes a hub's part ids). The scan reads 8 bytes per vertex per round; the vertices it
//     activates are the ones the reference's labels would hold.
//   B (parts): each queued part pushes its owner's amount to its <= K targets with FP64 reductions
//     (atomic adds whose old value nobody waits for). A round that queues no part ends the run: every
//     residual is then <= acc.
// Residuals and values are FP64 (a hub's residual collects ~10^5 pushes per round; FP32 accumulation
// would not hold the 1e-6 L1 bound); the output is FP32. Tracking which pushes lift a residual past acc
// instead of scanning needs the atomics' old values: 25 % slower on R-MAT s22 (154.6 against 123.4 ms),
// every returning FP64 atomic a long-scoreboard wait.
// The reference's two DD kernels differ only in when a vertex's label is cleared (in the kernel that
// processes it, or by clearLabel after it); with the residual taken once per round in a phase of its
// own that makes no difference, so SYNC_PUSH_DD and ASYNC_PUSH_DD run these same rounds.
#include <algorithm>

#include "internal.hpp"

namespace eeg {
namespace {

constexpr int DD_TPB = 512;

struct DDArgs {
    uint32_t n;
    uint32_t P;
    const uint32_t* __restrict__ vstart;
    const uint32_t* __restrict__ vowner;
    const uint32_t* __restrict__ vcol;
    const uint32_t* __restrict__ deg;
    double* r;
    double* xv;
    double* amt;
    float* x;
    uint32_t* pq;
    PRDDCtrl* ctrl;
    double acc;
    double damping;
    double base;
    uint32_t max_iters;
    uint64_t timeout_ns;
};

// Warp-collective: append the parts [s0, s0 + np) of each lane's vertex to the part queue.
__device__ __forceinline__ void append_parts(uint32_t s0, uint32_t np, uint32_t* ctr, uint32_t* pq, uint32_t cap,
                                             uint32_t lane) {
    uint32_t inc = np;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= (uint32_t)off) inc += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    if (total == 0u) return;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(ctr, total);
    base = __shfl_sync(0xffffffffu, base, 0);
    const uint32_t pos = base + inc - np;
    if (np <= 32u)
        for (uint32_t j = 0; j < np; ++j)
            if (pos + j < cap) pq[pos + j] = s0 + j;
    uint32_t big = __ballot_sync(0xffffffffu, np > 32u);
    while (big) {  // hub vertices: the whole warp writes their part ids
        const int l = __ffs(big) - 1;
        big &= big - 1u;
        const uint32_t bs0 = __shfl_sync(0xffffffffu, s0, l);
        const uint32_t bnp = __shfl_sync(0xffffffffu, np, l);
        const uint32_t bpos = __shfl_sync(0xffffffffu, pos, l);
        for (uint32_t j = lane; j < bnp; j += 32u)
            if (bpos + j < cap) pq[bpos + j] = bs0 + j;
    }
}

template <int K>
__global__ void __launch_bounds__(DD_TPB, 2) k_pagerank_dd(DDArgs a) {
    __shared__ uint32_t s_len;
    __shared__ double s_red[2][DD_TPB / 32];
    PRDDCtrl* ctrl = a.ctrl;
    const uint32_t gtid = blockIdx.x * DD_TPB + threadIdx.x;
    const uint32_t gthreads = gridDim.x * DD_TPB;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gwarp = gtid >> 5, nwarps = gthreads >> 5;
    const uint64_t pol = l2_evict_first_policy();
    uint32_t epoch = 0;
    uint32_t it = 0;
    unsigned long long my_pushes = 0, my_parts = 0, my_taken = 0;

    for (uint32_t v = gtid; v < a.n; v += gthreads) {
        a.r[v] = a.base;
        a.xv[v] = 0.0;
    }
    if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) goto finish;

    for (;; ++it) {
        const uint32_t cur = it % 3u, nxt = (it + 1u) % 3u;
        if (it >= a.max_iters) {
            if (blockIdx.x == 0 && threadIdx.x == 0)
                atomicCAS(&ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_ITER_CAP);
            break;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->plen[nxt] = 0u;  // last read in round it-2
        // ---- phase A: every vertex whose residual exceeds acc takes it (a dense scan of the residuals)
        for (uint32_t b0 = gwarp * 32u; b0 < a.n; b0 += nwarps * 32u) {
            const uint32_t v = b0 + lane;
            uint32_t s0 = 0, np = 0;
            if (v < a.n) {
                const double t = __ldcg(&a.r[v]);
                if (t > a.acc) {
                    a.r[v] = 0.0;
                    a.xv[v] = __ldcg(&a.xv[v]) + t;
                    ++my_taken;
                    const uint32_t d = __ldg(&a.deg[v]);
                    if (d) {
                        a.amt[v] = a.damping * t / (double)d;
                        s0 = __ldg(&a.vstart[v]);
                        np = __ldg(&a.vstart[v + 1]) - s0;
                    }
                }
            }
            append_parts(s0, np, &ctrl->plen[cur], a.pq, a.P, lane);
        }
        if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) break;
        if (threadIdx.x == 0) s_len = ld_relaxed(&ctrl->plen[cur]);
        __syncthreads();
        uint32_t npq = s_len;
        __syncthreads();
        if (npq == 0u) break;  // nothing pushes: every residual stays <= acc
        if (npq > a.P) {
            if (blockIdx.x == 0 && threadIdx.x == 0)
                atomicCAS(&ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_OVERFLOW);
            npq = a.P;
        }
        // ---- phase B: push the amounts along the queued parts (reductions: no value comes back)
        for (uint32_t b0 = gwarp * 32u; b0 < npq; b0 += nwarps * 32u) {
            const uint32_t i = b0 + lane;
            if (i < npq) {
                uint32_t col[K];
                const uint32_t p = __ldcg(&a.pq[i]);
                const double am = __ldcg(&a.amt[__ldg(&a.vowner[p])]);
                ld_part<K>(a.vcol + (size_t)p * K, col, pol);
                ++my_parts;
#pragma unroll
                for (int k = 0; k < K; ++k)
                    if (col[k] != NO_EDGE) {
                        atomicAdd(&a.r[col[k]], am);
                        ++my_pushes;
                    }
            }
        }
        if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) break;
    }
finish:
    {
        // the output, and what is left: residual mass (error bound resid / (1-d)) and the value norm
        double rs = 0.0, xs = 0.0;
        for (uint32_t v = gtid; v < a.n; v += gthreads) {
            const double xv = __ldcg(&a.xv[v]);
            a.x[v] = (float)xv;
            rs += __ldcg(&a.r[v]);
            xs += xv;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            rs += __shfl_down_sync(0xffffffffu, rs, off);
            xs += __shfl_down_sync(0xffffffffu, xs, off);
            my_pushes += __shfl_down_sync(0xffffffffu, my_pushes, off);
            my_parts += __shfl_down_sync(0xffffffffu, my_parts, off);
            my_taken += __shfl_down_sync(0xffffffffu, my_taken, off);
        }
        if (lane == 0) {
            s_red[0][threadIdx.x >> 5] = rs;
            s_red[1][threadIdx.x >> 5] = xs;
            if (my_pushes) atomicAdd(&ctrl->pushes, my_pushes);
            if (my_parts) atomicAdd(&ctrl->parts, my_parts);
            if (my_taken) atomicAdd(&ctrl->consumed, my_taken);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double r2 = 0.0, x2 = 0.0;
            for (int w = 0; w < DD_TPB / 32; ++w) {
                r2 += s_red[0][w];
                x2 += s_red[1][w];
            }
            atomicAdd(&ctrl->resid, r2);
            atomicAdd(&ctrl->norm, x2);
            if (blockIdx.x == 0) ctrl->iterations = it;
        }
    }
}

template <int K>
eeg_status launch_dd(const DDArgs& a, int device, uint32_t bps, cudaStream_t st) {
    auto kern = k_pagerank_dd<K>;
    int per_sm = 0;
    EEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, DD_TPB, 0));
    if (per_sm <= 0) {
        set_last_error("data-driven PageRank kernel does not fit on an SM");
        return EEG_ERR_CUDA;
    }
    if (bps > 0 && (int)bps < per_sm) per_sm = (int)bps;
    uint64_t blocks = (uint64_t)per_sm * sm_count(device);
    const uint64_t work = std::max<uint64_t>(a.P, a.n);
    const uint64_t need = (work + DD_TPB - 1) / DD_TPB;
    if (need < blocks) blocks = std::max<uint64_t>(need, 1);
    DDArgs args = a;
    void* params[] = {(void*)&args};
    EEG_CUDA(cudaLaunchCooperativeKernel((const void*)kern, dim3((unsigned)blocks), dim3(DD_TPB), params, 0, st));
    return EEG_OK;
}

}  // namespace

eeg_status run_pagerank_dd(eeg_vgraph* vg, eeg_variant variant, const eeg_options& o, cudaStream_t st,
                           eeg_result* res) {
    (void)variant;
    if (vg->n == 0) {
        set_last_error("empty graph");
        return EEG_ERR_INVALID;
    }
    if (!vg->fwd_parts) {
        set_last_error("data-driven PageRank pushes along out-edges: this graph was built without its forward "
                       "parts (EEG_VG_REVERSE_ONLY); use a topology-driven variant or build the forward graph");
        return EEG_ERR_INVALID;
    }
    Workspace& ws = vg->ws;
    const size_t n = std::max<uint32_t>(vg->n, 1);
    const size_t P = std::max<uint64_t>(vg->fwd.P, 1);
    if (!ws.x) EEG_TRY(vg_alloc(vg, (void**)&ws.x, sizeof(float) * n));
    if (!ws.dd_r) EEG_TRY(vg_alloc(vg, (void**)&ws.dd_r, sizeof(double) * n));
    if (!ws.dd_x) EEG_TRY(vg_alloc(vg, (void**)&ws.dd_x, sizeof(double) * n));
    if (!ws.dd_amt) EEG_TRY(vg_alloc(vg, (void**)&ws.dd_amt, sizeof(double) * n));
    if (!ws.dd_pq) EEG_TRY(vg_alloc(vg, (void**)&ws.dd_pq, sizeof(uint32_t) * P));
    if (!ws.ddctrl) EEG_CUDA(cudaMalloc((void**)&ws.ddctrl, sizeof(PRDDCtrl)));
    if (!ws.ev[0]) {
        EEG_CUDA(cudaEventCreate(&ws.ev[0]));
        EEG_CUDA(cudaEventCreate(&ws.ev[1]));
    }
    EEG_CUDA(cudaMemsetAsync(ws.ddctrl, 0, sizeof(PRDDCtrl), st));
    const double damping = o.pr_damping > 0.f ? (double)o.pr_damping : 0.85;
    const double tol = o.pr_tolerance > 0.f ? (double)o.pr_tolerance : 1e-7;
    DDArgs a{};
    a.n = vg->n;
    a.P = (uint32_t)vg->fwd.P;
    a.vstart = vg->fwd.vstart;
    a.vowner = vg->fwd.vowner;
    a.vcol = vg->fwd.vcol;
    a.deg = vg->fwd.deg;
    a.r = ws.dd_r;
    a.xv = ws.dd_x;
    a.amt = ws.dd_amt;
    a.x = ws.x;
    a.pq = ws.dd_pq;
    a.ctrl = ws.ddctrl;
    a.damping = damping;
    a.base = 1.0 - damping;
    // The reference's activation threshold when given; otherwise one that meets the tolerance: every
    // value ends >= 1-d, so residuals <= tol*(1-d)^2 bound ||x*-x||_1 <= n*acc/(1-d) <= tol*||x||_1.
    a.acc = o.pr_accuracy > 0.f ? (double)o.pr_accuracy : tol * (1.0 - damping) * (1.0 - damping);
    a.max_iters = o.max_iterations ? o.max_iterations : 10000u;
    a.timeout_ns = wait_limit_ns(o);

    EEG_CUDA(cudaEventRecord(ws.ev[0], st));
    eeg_status s;
    switch (vg->K) {
        case 4: s = launch_dd<4>(a, vg->device, o.blocks_per_sm, st); break;
        case 8: s = launch_dd<8>(a, vg->device, o.blocks_per_sm, st); break;
        case 16: s = launch_dd<16>(a, vg->device, o.blocks_per_sm, st); break;
        default: set_last_error("K must be 4, 8 or 16"); return EEG_ERR_UNSUPPORTED;
    }
    if (s != EEG_OK) return s;
    EEG_CUDA(cudaEventRecord(ws.ev[1], st));
    PRDDCtrl hc;
    EEG_CUDA(cudaMemcpyAsync(&hc, ws.ddctrl, sizeof(PRDDCtrl), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    EEG_CUDA(cudaEventElapsedTime(&ms, ws.ev[0], ws.ev[1]));
    if (res) {
        res->kernel_ms = ms;
        res->iterations = hc.iterations;
        res->edges_scanned = hc.pushes;
        res->parts_processed = hc.parts;
        res->updates = hc.consumed;
        res->pr_residual = hc.resid;
        res->pr_l1_norm = hc.norm;
        res->launches = 1;
    }
    if (hc.bw.status == DEV_TIMEOUT) {
        set_last_error("grid barrier wait exceeded the timeout");
        return EEG_ERR_TIMEOUT;
    }
    if (hc.bw.status == DEV_ITER_CAP) {
        set_last_error("data-driven PageRank did not empty its frontier within the round cap");
        return EEG_ERR_ITER_CAP;
    }
    if (hc.bw.status == DEV_OVERFLOW) {
        set_last_error("internal error: a PageRank frontier exceeded its capacity");
        return EEG_ERR_CUDA;
    }
    return EEG_OK;
}

}  // namespace eeg
