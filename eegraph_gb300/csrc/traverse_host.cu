// traverse_host.cu -- host side of the persistent traversal: workspace, launch, statistics.
#include "traverse.cuh"

namespace eeg {
using namespace trav;

eeg_status reached_stats(eeg_vgraph* vg, int op, const uint32_t* d_dist, cudaStream_t st, uint64_t* n_r,
                         uint64_t* m_r) {
    Workspace& ws = vg->ws;
    if (!ws.stats) EEG_CUDA(cudaMalloc((void**)&ws.stats, 4 * sizeof(unsigned long long)));
    EEG_CUDA(cudaMemsetAsync(ws.stats, 0, 2 * sizeof(unsigned long long), st));
    const unsigned blocks = (unsigned)std::min<uint64_t>((vg->n + 255) / 256 + 1, (uint64_t)sm_count(vg->device) * 8);
    switch (op) {
        case OP_BFS: k_reached<OP_BFS><<<blocks, 256, 0, st>>>(d_dist, vg->fwd.deg, vg->n, ws.stats); break;
        case OP_SSSP: k_reached<OP_SSSP><<<blocks, 256, 0, st>>>(d_dist, vg->fwd.deg, vg->n, ws.stats); break;
        case OP_SSWP: k_reached<OP_SSWP><<<blocks, 256, 0, st>>>(d_dist, vg->fwd.deg, vg->n, ws.stats); break;
        default: k_reached<OP_CC><<<blocks, 256, 0, st>>>(d_dist, vg->fwd.deg, vg->n, ws.stats); break;
    }
    EEG_CUDA(cudaGetLastError());
    unsigned long long h[2];
    EEG_CUDA(cudaMemcpyAsync(h, ws.stats, sizeof(h), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    *n_r = h[0];
    *m_r = h[1];
    return EEG_OK;
}

static eeg_status ensure_traversal_ws(eeg_vgraph* vg, uint32_t activity_cap) {
    Workspace& ws = vg->ws;
    const size_t n = vg->n, P = std::max<uint64_t>(vg->fwd.P, 1);
    if (!ws.dist) EEG_TRY(vg_alloc(vg, (void**)&ws.dist, sizeof(uint32_t) * std::max<size_t>(n, 1)));
    if (!ws.stamp) EEG_TRY(vg_alloc(vg, (void**)&ws.stamp, sizeof(uint32_t) * std::max<size_t>(n, 1)));
    if (!ws.pushed) EEG_TRY(vg_alloc(vg, (void**)&ws.pushed, sizeof(uint32_t) * P));
    if (!ws.q[0]) EEG_TRY(vg_alloc(vg, (void**)&ws.q[0], sizeof(uint32_t) * P));
    if (!ws.q[1]) EEG_TRY(vg_alloc(vg, (void**)&ws.q[1], sizeof(uint32_t) * P));
    if (!ws.tctrl) EEG_CUDA(cudaMalloc((void**)&ws.tctrl, sizeof(TravCtrl)));
    if (activity_cap > ws.activity_cap) {
        if (ws.activity) cudaFree(ws.activity);
        ws.activity = nullptr;
        EEG_CUDA(cudaMalloc((void**)&ws.activity, sizeof(uint32_t) * activity_cap));
        ws.activity_cap = activity_cap;
    }
    if (!ws.ev[0]) {
        EEG_CUDA(cudaEventCreate(&ws.ev[0]));
        EEG_CUDA(cudaEventCreate(&ws.ev[1]));
    }
    return EEG_OK;
}

eeg_status run_traversal(eeg_vgraph* vg, int op, eeg_variant variant, uint32_t source, const eeg_options& o,
                         cudaStream_t st, eeg_result* res, uint32_t* activity_host, uint32_t activity_cap) {
    const bool td = (variant == EEG_ASYNC_PUSH_TD || variant == EEG_SYNC_PUSH_TD);
    // ASYNC_PUSH_DD starts with every vertex active, SYNC_PUSH_DD with the source only
    // (src/eegraph.cu:41-49); for CC that gives SYNC_PUSH_DD its own fixed point (src/eegraph.cu:544-553).
    const bool seed_all = (variant == EEG_ASYNC_PUSH_DD);
    if (vg->n == 0) {
        set_last_error("empty graph");
        return EEG_ERR_INVALID;
    }
    if (!vg->fwd_parts) {
        set_last_error("graph built with EEG_VG_REVERSE_ONLY has no forward parts (PageRank only)");
        return EEG_ERR_INVALID;
    }
    if (source >= vg->n) {
        set_last_error("source vertex out of range");
        return EEG_ERR_INVALID;
    }
    const bool cc_zero = op == OP_CC && o.cc_components;
    if (op != OP_BFS && !cc_zero && !vg->fwd.vw && vg->fwd.P > 0) {
        set_last_error("graph was built without weights");
        return EEG_ERR_INVALID;
    }
    EEG_TRY(ensure_traversal_ws(vg, activity_host ? activity_cap : 0));
    Workspace& ws = vg->ws;
    const bool bucketed = o.delta && !td && !seed_all && (op == OP_SSSP || op == OP_SSWP);
    if (bucketed && !ws.far) EEG_TRY(vg_alloc(vg, (void**)&ws.far, sizeof(uint32_t) * 4 * (size_t)vg->n));
    EEG_CUDA(cudaMemsetAsync(ws.tctrl, 0, sizeof(TravCtrl), st));

    TravArgs a{};
    a.n = vg->n;
    a.P = (uint32_t)vg->fwd.P;
    a.vstart = vg->fwd.vstart;
    a.vowner = vg->fwd.vowner;
    a.vcol = vg->fwd.vcol;
    a.vw = vg->fwd.vw;
    a.dist = ws.dist;
    a.q0 = ws.q[0];
    a.q1 = ws.q[1];
    a.stamp = ws.stamp;
    a.pushed = ws.pushed;
    // source-seeded BFS pulls in its large rounds when the transposed parts exist
    if (op == OP_BFS && variant == EEG_SYNC_PUSH_DD && vg->has_rev && vg->rev.P && !o.bfs_push_only && !bucketed) {
        if (!ws.plist) EEG_TRY(vg_alloc(vg, (void**)&ws.plist, sizeof(uint32_t) * 2 * (size_t)vg->n));
        a.rvstart = vg->rev.vstart;
        a.rvcol = vg->rev.vcol;
        a.plist = ws.plist;
    }
    a.ctrl = ws.tctrl;
    a.activity = activity_host ? ws.activity : nullptr;
    a.activity_cap = activity_host ? activity_cap : 0;
    a.source = source;
    a.seed_all = seed_all ? 1u : 0u;
    a.partner = (variant == EEG_SYNC_PUSH_TD) ? 1u : 0u;
    a.cc_zero = cc_zero ? 1u : 0u;
    a.max_iters = o.max_iterations ? o.max_iterations : (vg->n > 0xFFFFFFF0u ? 0xFFFFFFFFu : vg->n + 2u);
    if (bucketed) {
        // far rounds come on top of the frontier rounds (each moves at least one vertex back)
        if (!o.max_iterations) a.max_iters = (uint32_t)std::min<uint64_t>(64ull * vg->n + 1024u, 0xFFFFFFF0u);
        a.delta = o.delta;
        a.fpile = ws.far;
        a.fflag = ws.far + 3 * (size_t)vg->n;
    }
    a.timeout_ns = wait_limit_ns(o);
    a.it_start = 0;
    a.rounds_limit = o.host_loop ? 1u : 0u;

    EEG_CUDA(cudaEventRecord(ws.ev[0], st));
    TravCtrl hc;
    uint32_t launches = 0;
    for (;;) {
        eeg_status s;
        switch (op) {
            case OP_BFS: s = launch_bfs(a, td, vg->K, vg->device, o.blocks_per_sm, st); break;
            case OP_SSSP: s = launch_sssp(a, td, vg->K, vg->device, o.blocks_per_sm, st); break;
            case OP_SSWP: s = launch_sswp(a, td, vg->K, vg->device, o.blocks_per_sm, st); break;
            case OP_CC: s = launch_cc(a, td, vg->K, vg->device, o.blocks_per_sm, st); break;
            default: set_last_error("unknown algorithm"); return EEG_ERR_INVALID;
        }
        if (s != EEG_OK) return s;
        ++launches;
        if (!o.host_loop) break;
        // host-loop mode: read the round's outcome back before deciding on the next launch
        EEG_CUDA(cudaMemcpyAsync(&hc, ws.tctrl, sizeof(TravCtrl), cudaMemcpyDeviceToHost, st));
        EEG_CUDA(cudaStreamSynchronize(st));
        if (hc.done || hc.bw.status != DEV_OK) break;
        a.it_start = hc.iterations;
        // every launch counts its barrier arrivals from zero
        EEG_CUDA(cudaMemsetAsync(&ws.tctrl->bw.arrive, 0, sizeof(uint32_t), st));
    }
    EEG_CUDA(cudaEventRecord(ws.ev[1], st));

    EEG_CUDA(cudaMemcpyAsync(&hc, ws.tctrl, sizeof(TravCtrl), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    if (res) res->launches = launches + 1;  // + the reached-set statistics kernel
    float ms = 0.f;
    EEG_CUDA(cudaEventElapsedTime(&ms, ws.ev[0], ws.ev[1]));
    if (res) {
        res->kernel_ms = ms;
        res->iterations = hc.iterations;
        res->parts_processed = hc.parts_processed;
        res->edges_scanned = hc.edges_scanned;
        res->updates = hc.updates;
        res->pull_rounds = hc.pull_rounds;
    }
    if (activity_host && activity_cap) {
        const uint32_t cnt = std::min<uint32_t>(hc.iterations, activity_cap);
        if (cnt) EEG_CUDA(cudaMemcpy(activity_host, ws.activity, sizeof(uint32_t) * cnt, cudaMemcpyDeviceToHost));
        if (res) res->num_activity = cnt;
    }
    if (hc.bw.status == DEV_TIMEOUT) {
        set_last_error("grid barrier wait exceeded the timeout");
        return EEG_ERR_TIMEOUT;
    }
    if (hc.bw.status == DEV_ITER_CAP) {
        set_last_error("iteration cap reached before the fixed point");
        return EEG_ERR_ITER_CAP;
    }
    if (hc.bw.status == DEV_OVERFLOW) {
        set_last_error("internal error: a frontier queue exceeded its capacity");
        return EEG_ERR_CUDA;
    }
    return EEG_OK;
}

}  // namespace eeg
