// capi.cu -- implementation of the C ABI declared in include/eegraph_c.h.
//
// Replaces the library entry points eegraph_<algo>[_um] (reference include/eegraph.cuh:21-39,
// src/eegraph.cu) at the C level: handles own their device memory, results go to caller-owned
// buffers, every failure is a returned status (the reference calls exit(), include/gpu_error_check.cuh:8-16).
#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "internal.hpp"

namespace eeg {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

eeg_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_last_error = buf;
    if (e == cudaErrorMemoryAllocation) return EEG_ERR_NOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return EEG_ERR_NO_DEVICE;
    return EEG_ERR_CUDA;
}

// Graph and workspace arrays come from the device's stream-ordered pool, which keeps freed memory
// (release threshold raised once per device): a caller that builds and drops graphs repeatedly reuses
// memory instead of paying cudaMalloc/cudaFree each time. Reuse across streams is made safe by the
// pool's internal dependencies; handles are destroyed after a device synchronisation (cudaFree's
// semantics), so no freed array is still in use.
static void retain_pool_memory(int device) {
    static std::mutex mu;
    static bool done[64] = {false};
    if (device < 0 || device >= 64) return;
    std::lock_guard<std::mutex> lk(mu);
    if (done[device]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    (void)cudaGetLastError();
    done[device] = true;
}

eeg_status vg_alloc(eeg_vgraph* vg, void** p, size_t bytes) {
    if (bytes == 0) bytes = 4;
    cudaError_t e;
    if (vg->managed) {
        e = cudaMallocManaged(p, bytes);
        if (e == cudaSuccess) {
            cudaMemLocation loc{};
            loc.type = cudaMemLocationTypeDevice;
            loc.id = vg->device;
            cudaMemAdvise(*p, bytes, cudaMemAdviseSetPreferredLocation, loc);
            (void)cudaGetLastError();
        }
    } else {
        retain_pool_memory(vg->device);
        e = cudaMallocAsync(p, bytes, 0);
        if (e == cudaSuccess) e = cudaStreamSynchronize(0);  // usable from any stream on return
    }
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, vg->managed ? "cudaMallocManaged" : "cudaMallocAsync", __FILE__, __LINE__);
    }
    return EEG_OK;
}

// Callers synchronise the device first (handle destruction).
void vg_free(eeg_vgraph* vg, void* p) {
    if (!p) return;
    if (vg->managed) cudaFree(p);
    else cudaFreeAsync(p, 0);
}

static void free_dir(eeg_vgraph* vg, VDir& d) {
    vg_free(vg, d.vstart);
    vg_free(vg, d.vowner);
    vg_free(vg, d.vcol);
    vg_free(vg, d.vw);
    vg_free(vg, d.veid);
    vg_free(vg, d.deg);
    d = VDir{};
}

static void free_ws(eeg_vgraph* vg) {
    Workspace& w = vg->ws;
    vg_free(vg, w.dist);
    vg_free(vg, w.far);
    vg_free(vg, w.q[0]);
    vg_free(vg, w.q[1]);
    vg_free(vg, w.stamp);
    vg_free(vg, w.pushed);
    vg_free(vg, w.plist);
    if (w.activity) cudaFree(w.activity);
    if (w.tctrl) cudaFree(w.tctrl);
    vg_free(vg, w.x);
    vg_free(vg, w.contrib[0]);
    vg_free(vg, w.contrib[1]);
    vg_free(vg, w.acc);
    vg_free(vg, w.arrive);
    vg_free(vg, w.pr_rank);
    vg_free(vg, w.pr_rcol);
    vg_free(vg, w.pr_info);
    if (w.pctrl) cudaFree(w.pctrl);
    vg_free(vg, w.dd_r);
    vg_free(vg, w.dd_x);
    vg_free(vg, w.dd_amt);
    vg_free(vg, w.dd_pq);
    if (w.ddctrl) cudaFree(w.ddctrl);
    if (w.stats) cudaFree(w.stats);
    if (w.ev[0]) cudaEventDestroy(w.ev[0]);
    if (w.ev[1]) cudaEventDestroy(w.ev[1]);
    w = Workspace{};
}

}  // namespace eeg

using namespace eeg;

extern "C" {

EEG_API const char* eeg_status_string(eeg_status s) {
    switch (s) {
        case EEG_OK: return "ok";
        case EEG_ERR_INVALID: return "invalid argument";
        case EEG_ERR_IO: return "i/o error";
        case EEG_ERR_CUDA: return "CUDA error";
        case EEG_ERR_NOMEM: return "out of memory";
        case EEG_ERR_TIMEOUT: return "device wait timed out";
        case EEG_ERR_ITER_CAP: return "iteration cap reached";
        case EEG_ERR_UNSUPPORTED: return "unsupported";
        case EEG_ERR_NO_DEVICE: return "no CUDA device";
        case EEG_ERR_ENERGY: return "energy unavailable";
    }
    return "unknown status";
}

EEG_API const char* eeg_last_error(void) { return g_last_error.c_str(); }

EEG_API const char* eeg_version(void) { return "eegraph-gb300 0.1 (sm_103a)"; }

EEG_API int eeg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    return n;
}

EEG_API eeg_status eeg_set_device(int device) {
    EEG_CUDA(cudaSetDevice(device));
    return EEG_OK;
}

EEG_API eeg_status eeg_managed_alloc(size_t bytes, void** out) {
    if (!out) {
        set_last_error("null output pointer");
        return EEG_ERR_INVALID;
    }
    *out = nullptr;
    EEG_CUDA(cudaMallocManaged(out, bytes ? bytes : 4));
    return EEG_OK;
}

EEG_API void eeg_managed_free(void* p) {
    if (p) cudaFree(p);
}

EEG_API void eeg_options_init(eeg_options* o) {
    if (o) memset(o, 0, sizeof(*o));
}

static eeg_status build_impl(uint32_t n, uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w,
                             uint32_t K, uint32_t flags, void* stream, eeg_vgraph** out) {
    if (!out) {
        set_last_error("null output handle");
        return EEG_ERR_INVALID;
    }
    *out = nullptr;
    if (K != 4 && K != 8 && K != 16) {
        set_last_error("K must be 4, 8 or 16");
        return EEG_ERR_UNSUPPORTED;
    }
    if (m && (!src || !dst)) {
        set_last_error("null edge arrays");
        return EEG_ERR_INVALID;
    }
    if (flags & EEG_VG_REVERSE_ONLY) flags |= EEG_VG_REVERSE;
    const bool symmetrize = (flags & EEG_VG_SYMMETRIZE) != 0;
    if (m >= (symmetrize ? 0x7FFFFFFFull : 0xFFFFFFFFull) || n == 0xFFFFFFFFu) {
        set_last_error("graph too large for 32-bit ids/offsets");
        return EEG_ERR_UNSUPPORTED;
    }
    if (eeg_device_count() == 0) {
        set_last_error("no CUDA device visible");
        return EEG_ERR_NO_DEVICE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    eeg_vgraph* vg = new eeg_vgraph();
    cudaGetDevice(&vg->device);
    vg->n = n;
    vg->m = symmetrize ? 2 * m : m;  // arcs
    vg->K = K;
    vg->flags = flags;
    vg->managed = (flags & EEG_VG_MANAGED) != 0;
    vg->weighted = true;

    auto fail = [&](eeg_status s) {
        eeg_vgraph_destroy(vg);
        return s;
    };
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        set_last_error("cudaEventCreate failed");
        delete vg;
        return EEG_ERR_CUDA;
    }
    const bool on_device = (flags & EEG_VG_INPUT_DEVICE) != 0;
    const uint32_t *ds = src, *dd = dst, *dw = w;
    uint32_t* tmp = nullptr;
    eeg_status s = EEG_OK;
    // page-locked host arrays are read by the first build kernel in place (over NVLink-C2C / PCIe),
    // which saves a copy into device temporaries
    auto mapped = [](const uint32_t* p, const uint32_t** out) -> bool {
        if (!p) {
            *out = nullptr;
            return true;
        }
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
            (void)cudaGetLastError();
            return false;
        }
        if (at.type == cudaMemoryTypeHost && at.devicePointer) {
            *out = (const uint32_t*)at.devicePointer;
            return true;
        }
        return false;
    };
    const uint32_t *ms = nullptr, *md = nullptr, *mw = nullptr;
    // a two-direction build copies the input once (the copy engine moves it as fast as the in-place
    // reads) instead of reading it over the host link twice
    const bool zero_copy = !on_device && m > 0 && !(flags & EEG_VG_REVERSE) && mapped(src, &ms) && mapped(dst, &md) &&
                           mapped(w, &mw);
    cudaEventRecord(e0, st);
    if (zero_copy) {
        ds = ms;
        dd = md;
        dw = mw;
    } else if (!on_device && m > 0) {
        const size_t words = (size_t)m * (w ? 3 : 2);
        cudaError_t ce = cudaMallocAsync((void**)&tmp, words * sizeof(uint32_t), st);
        if (ce != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return fail(cuda_fail(ce, "cudaMallocAsync(edges)", __FILE__, __LINE__));
        }
        cudaMemcpyAsync(tmp, src, m * 4, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(tmp + m, dst, m * 4, cudaMemcpyHostToDevice, st);
        if (w) cudaMemcpyAsync(tmp + 2 * m, w, m * 4, cudaMemcpyHostToDevice, st);
        ds = tmp;
        dd = tmp + m;
        dw = w ? tmp + 2 * m : nullptr;
    }
    if (flags & EEG_VG_REVERSE_ONLY) {
        s = build_out_degrees(vg, &vg->fwd, ds, dd, st);
        vg->fwd_parts = false;
    } else {
        s = build_direction(vg, &vg->fwd, ds, dd, dw, false, st);
    }
    if (s == EEG_OK && !(flags & EEG_VG_REVERSE) && (flags & (EEG_VG_SYMMETRIC | EEG_VG_SYMMETRIZE))) {
        vg->rev = vg->fwd;  // undirected: in-edges are the out-edges
        vg->has_rev = true;
        vg->rev_alias = true;
    }
    if (s == EEG_OK && (flags & EEG_VG_REVERSE)) {
        s = build_direction(vg, &vg->rev, ds, dd, nullptr, true, st);
        vg->has_rev = (s == EEG_OK);
    }
    if (tmp) cudaFreeAsync(tmp, st);
    cudaEventRecord(e1, st);
    cudaError_t ce = cudaStreamSynchronize(st);
    if (s == EEG_OK && ce != cudaSuccess) s = cuda_fail(ce, "virtual graph build", __FILE__, __LINE__);
    if (s == EEG_OK) cudaEventElapsedTime(&vg->build_ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != EEG_OK) return fail(s);
    *out = vg;
    return EEG_OK;
}

EEG_API eeg_status eeg_vgraph_build(const eeg_graph* g, uint32_t K, uint32_t flags, void* stream, eeg_vgraph** out) {
    if (!g) {
        set_last_error("null graph");
        return EEG_ERR_INVALID;
    }
    // 1-based files are shifted down by one, as VirtualGraph::VirtualGraph does (src/virtual_graph.cpp:5-12)
    uint32_t f = flags & ~(uint32_t)EEG_VG_INPUT_DEVICE;
    if (!g->has_zero_id) f |= EEG_VG_SHIFT_ONE;
    else f &= ~(uint32_t)EEG_VG_SHIFT_ONE;
    return build_impl(g->num_nodes, g->num_edges, g->src.data(), g->dst.data(),
                      g->weight.empty() ? nullptr : g->weight.data(), K, f, stream, out);
}

EEG_API eeg_status eeg_vgraph_build_arrays(uint32_t num_nodes, uint64_t num_edges, const uint32_t* src,
                                           const uint32_t* dst, const uint32_t* weight, uint32_t K, uint32_t flags,
                                           void* stream, eeg_vgraph** out) {
    return build_impl(num_nodes, num_edges, src, dst, weight, K, flags, stream, out);
}

EEG_API eeg_status eeg_vgraph_get_info(const eeg_vgraph* vg, eeg_vgraph_info* o) {
    if (!vg || !o) {
        set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    o->num_nodes = vg->n;
    o->num_edges = vg->m;
    o->K = vg->K;
    o->num_parts = vg->fwd.P;
    o->num_rparts = vg->has_rev ? vg->rev.P : 0;
    o->max_out_degree = vg->max_deg;
    o->max_degree_vertex = vg->max_deg_vertex;
    o->device_bytes = vg->bytes;
    o->build_ms = vg->build_ms;
    return EEG_OK;
}

EEG_API eeg_status eeg_vgraph_download(const eeg_vgraph* vg, uint32_t* vstart, uint32_t* vowner, uint32_t* vcol,
                                       uint32_t* vw, uint32_t* outdeg) {
    if (!vg) {
        set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    if (!vg->fwd_parts) {
        set_last_error("graph built with EEG_VG_REVERSE_ONLY has no forward parts");
        return EEG_ERR_INVALID;
    }
    EEG_CUDA(cudaSetDevice(vg->device));
    const size_t n = vg->n, P = vg->fwd.P, S = P * vg->K;
    if (vstart) EEG_CUDA(cudaMemcpy(vstart, vg->fwd.vstart, 4 * (n + 1), cudaMemcpyDeviceToHost));
    if (vowner && P) EEG_CUDA(cudaMemcpy(vowner, vg->fwd.vowner, 4 * P, cudaMemcpyDeviceToHost));
    if (vcol && S) EEG_CUDA(cudaMemcpy(vcol, vg->fwd.vcol, 4 * S, cudaMemcpyDeviceToHost));
    if (vw && S && vg->fwd.vw) EEG_CUDA(cudaMemcpy(vw, vg->fwd.vw, 4 * S, cudaMemcpyDeviceToHost));
    if (outdeg) EEG_CUDA(cudaMemcpy(outdeg, vg->fwd.deg, 4 * n, cudaMemcpyDeviceToHost));
    return EEG_OK;
}

EEG_API eeg_status eeg_vgraph_export_reference_layout(const eeg_vgraph* vg, uint32_t* nodePointer,
                                                      uint32_t* edgeList, uint32_t* partNodePointer) {
    if (!vg) {
        set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    const size_t n = vg->n, P = vg->fwd.P, K = vg->K;
    std::vector<uint32_t> vstart(n + 1), deg(n), vcol(P * K), vw(P * K, 1u);
    EEG_TRY(eeg_vgraph_download(vg, vstart.data(), nullptr, vcol.data(), vg->fwd.vw ? vw.data() : nullptr, deg.data()));
    uint64_t counter = 0, part = 0;
    for (size_t v = 0; v < n; ++v) {
        if (nodePointer) nodePointer[v] = (uint32_t)counter;
        if (edgeList) {
            edgeList[counter] = deg[v];
            const size_t base = (size_t)vstart[v] * K;
            for (uint32_t r = 0; r < deg[v]; ++r) {
                edgeList[counter + 1 + 2 * (uint64_t)r] = vcol[base + r];
                edgeList[counter + 2 + 2 * (uint64_t)r] = vw[base + r];
            }
        }
        counter += 2 * (uint64_t)deg[v] + 1;
        const uint32_t np = vstart[v + 1] - vstart[v];
        for (uint32_t j = 0; j < np; ++j, ++part) {
            if (partNodePointer) {
                partNodePointer[2 * part] = (uint32_t)v;
                partNodePointer[2 * part + 1] = j;
            }
        }
    }
    return EEG_OK;
}

EEG_API eeg_status eeg_autotune_k(uint32_t num_nodes, uint64_t num_edges, const uint32_t* src, const uint32_t* dst,
                                  const uint32_t* weight, uint32_t reps, uint32_t* best_k, float* ms_per_k) {
    if (!best_k) {
        set_last_error("eeg_autotune_k: null output");
        return EEG_ERR_INVALID;
    }
    static std::mutex mu;
    static std::map<std::tuple<uint32_t, uint64_t, uint32_t>, std::pair<uint32_t, std::array<float, 3>>> cache;
    reps = reps ? reps : 3;
    const uint32_t ks[3] = {4, 8, 16};
    std::array<float, 3> times{};
    std::tuple<uint32_t, uint64_t, uint32_t> key;
    for (int i = 0; i < 3; ++i) {
        eeg_vgraph* vg = nullptr;
        EEG_TRY(eeg_vgraph_build_arrays(num_nodes, num_edges, src, dst, weight, ks[i], 0, nullptr, &vg));
        if (i == 0) {
            key = std::make_tuple(num_nodes, num_edges, vg->max_deg);
            std::lock_guard<std::mutex> lk(mu);
            auto it = cache.find(key);
            if (it != cache.end()) {
                eeg_vgraph_destroy(vg);
                *best_k = it->second.first;
                if (ms_per_k) std::copy(it->second.second.begin(), it->second.second.end(), ms_per_k);
                return EEG_OK;
            }
        }
        std::vector<float> t;
        eeg_status s = EEG_OK;
        for (uint32_t r = 0; r < reps + 1 && s == EEG_OK; ++r) {  // first run warms up
            eeg_result a{}, b{};
            s = eeg_run(vg, EEG_BFS, EEG_SYNC_PUSH_DD, vg->max_deg_vertex, nullptr, nullptr, 0, nullptr, 0, nullptr, &a);
            if (s == EEG_OK)
                s = eeg_run(vg, EEG_SSSP, EEG_SYNC_PUSH_DD, vg->max_deg_vertex, nullptr, nullptr, 0, nullptr, 0, nullptr, &b);
            if (r > 0) t.push_back(a.kernel_ms + b.kernel_ms);
        }
        eeg_vgraph_destroy(vg);
        if (s != EEG_OK) return s;
        std::sort(t.begin(), t.end());
        times[i] = t[t.size() / 2];
    }
    const int best = (int)(std::min_element(times.begin(), times.end()) - times.begin());
    *best_k = ks[best];
    if (ms_per_k) std::copy(times.begin(), times.end(), ms_per_k);
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = std::make_pair(ks[best], times);
    return EEG_OK;
}

EEG_API eeg_status eeg_autotune(uint32_t num_nodes, uint64_t num_edges, const uint32_t* src, const uint32_t* dst,
                                const uint32_t* weight, eeg_algo algo, uint32_t reps, eeg_tuning* out) {
    if (!out || (unsigned)algo > (unsigned)EEG_PR) {
        set_last_error("eeg_autotune: null output or unknown algorithm");
        return EEG_ERR_INVALID;
    }
    reps = reps ? reps : 3;
    const uint32_t ks[3] = {4, 8, 16};
    eeg_tuning t{};
    t.ms = -1.f;
    for (float& x : t.ms_table) x = -1.f;
    // PageRank: the transposed graph for the pull variants, the forward parts for the data-driven ones
    const uint32_t flags = algo == EEG_PR ? (uint32_t)EEG_VG_REVERSE : 0u;
    const uint32_t* w = (algo == EEG_BFS || algo == EEG_PR) ? nullptr : weight;
    for (int i = 0; i < 3; ++i) {
        eeg_vgraph* vg = nullptr;
        EEG_TRY(eeg_vgraph_build_arrays(num_nodes, num_edges, src, dst, w, ks[i], flags, nullptr, &vg));
        eeg_status s = EEG_OK;
        for (int v = 0; v < 4 && s == EEG_OK; ++v) {
            if (algo == EEG_CC && v == EEG_SYNC_PUSH_DD) continue;  // another fixed point
            std::vector<float> times;
            for (uint32_t r = 0; r < reps + 1 && s == EEG_OK; ++r) {  // the first run warms up
                eeg_result res{};
                s = eeg_run(vg, algo, (eeg_variant)v, vg->max_deg_vertex, nullptr, nullptr, 0, nullptr, 0, nullptr,
                            &res);
                if (s == EEG_OK && r > 0) times.push_back(res.kernel_ms);
            }
            if (s != EEG_OK) break;
            std::sort(times.begin(), times.end());
            const float med = times[times.size() / 2];
            t.ms_table[i * 4 + v] = med;
            if (t.ms < 0.f || med < t.ms) {
                t.ms = med;
                t.K = ks[i];
                t.variant = (eeg_variant)v;
            }
        }
        eeg_vgraph_destroy(vg);
        if (s != EEG_OK) return s;
    }
    // resident CTAs per SM for the chosen (K, variant)
    t.blocks_per_sm = 0;
    t.ms_per_blocks[0] = t.ms_per_blocks[1] = -1.f;
    {
        eeg_vgraph* vg = nullptr;
        EEG_TRY(eeg_vgraph_build_arrays(num_nodes, num_edges, src, dst, w, t.K, flags, nullptr, &vg));
        const bool pull = algo == EEG_PR && (t.variant == EEG_SYNC_PUSH_TD || t.variant == EEG_ASYNC_PUSH_TD);
        eeg_status s = EEG_OK;
        for (uint32_t b = 1; b <= (pull ? 1u : 2u) && s == EEG_OK; ++b) {
            eeg_options o;
            eeg_options_init(&o);
            o.blocks_per_sm = b;
            std::vector<float> times;
            for (uint32_t r = 0; r < reps + 1 && s == EEG_OK; ++r) {
                eeg_result res{};
                s = eeg_run(vg, algo, t.variant, vg->max_deg_vertex, &o, nullptr, 0, nullptr, 0, nullptr, &res);
                if (s == EEG_OK && r > 0) times.push_back(res.kernel_ms);
            }
            if (s != EEG_OK) break;
            std::sort(times.begin(), times.end());
            t.ms_per_blocks[b - 1] = times[times.size() / 2];
            if (t.blocks_per_sm == 0 || t.ms_per_blocks[b - 1] < t.ms_per_blocks[t.blocks_per_sm - 1]) t.blocks_per_sm = b;
        }
        eeg_vgraph_destroy(vg);
        if (s != EEG_OK) return s;
    }
    *out = t;
    return EEG_OK;
}

EEG_API void eeg_vgraph_destroy(eeg_vgraph* vg) {
    if (!vg) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(vg->device);
    cudaDeviceSynchronize();  // no kernel may still use the arrays (cudaFree would have waited too)
    if (!vg->rev_alias) free_dir(vg, vg->rev);
    free_dir(vg, vg->fwd);
    free_ws(vg);
    cudaStreamSynchronize(0);
    cudaSetDevice(prev);
    delete vg;
}

EEG_API eeg_status eeg_run(eeg_vgraph* vg, eeg_algo algo, eeg_variant variant, uint32_t source,
                           const eeg_options* opts, void* out, int out_on_device, uint32_t* activity,
                           uint32_t activity_cap, void* stream, eeg_result* res) {
    if (!vg) {
        set_last_error("null graph handle");
        return EEG_ERR_INVALID;
    }
    if ((unsigned)variant > 3u) {
        set_last_error("unknown variant");
        return EEG_ERR_INVALID;
    }
    eeg_options o;
    eeg_options_init(&o);
    if (opts) o = *opts;
    eeg_result r;
    memset(&r, 0, sizeof(r));
    cudaStream_t st = (cudaStream_t)stream;
    EEG_CUDA(cudaSetDevice(vg->device));
    eeg_status s;
    if (algo == EEG_PR) {
        const bool dd = variant == EEG_SYNC_PUSH_DD || variant == EEG_ASYNC_PUSH_DD;
        s = dd ? run_pagerank_dd(vg, variant, o, st, &r) : run_pagerank(vg, variant, o, st, &r);
        if (s == EEG_OK || s == EEG_ERR_ITER_CAP) {
            if (out) {
                EEG_CUDA(cudaMemcpyAsync(out, vg->ws.x, sizeof(float) * vg->n,
                                         out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
                EEG_CUDA(cudaStreamSynchronize(st));
            }
            r.reached_vertices = vg->n;
            r.reached_edges = vg->m;
            if (dd) {  // work-minimal bytes of the pushes made: per push its 4-byte target and 8-byte
                       // residual update; per activation the vertex's residual, value, amount and row bounds
                r.algorithmic_bytes = 12.0 * (double)r.edges_scanned + 32.0 * (double)r.updates;
                r.gteps = r.kernel_ms > 0 ? (double)r.edges_scanned / (r.kernel_ms * 1e-3) / 1e9 : 0.0;
            } else {
                r.algorithmic_bytes = (double)r.iterations * (12.0 * vg->n + 8.0 * (double)vg->m);
                r.gteps = r.kernel_ms > 0 ? (double)r.iterations * (double)vg->m / (r.kernel_ms * 1e-3) / 1e9 : 0.0;
            }
        }
        if (activity && activity_cap && res) r.num_activity = 0;
    } else {
        int op;
        switch (algo) {
            case EEG_BFS: op = OP_BFS; break;
            case EEG_SSSP: op = OP_SSSP; break;
            case EEG_SSWP: op = OP_SSWP; break;
            case EEG_CC: op = OP_CC; break;
            default: set_last_error("unknown algorithm"); return EEG_ERR_INVALID;
        }
        s = run_traversal(vg, op, variant, source, o, st, &r, activity, activity_cap);
        if (s == EEG_OK || s == EEG_ERR_ITER_CAP) {
            if (out) {
                EEG_CUDA(cudaMemcpyAsync(out, vg->ws.dist, sizeof(uint32_t) * vg->n,
                                         out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
            }
            uint64_t nr = 0, mr = 0;
            eeg_status s2 = reached_stats(vg, op, vg->ws.dist, st, &nr, &mr);
            if (s2 != EEG_OK) return s2;
            r.reached_vertices = nr;
            r.reached_edges = mr;
            r.algorithmic_bytes = 12.0 * (double)nr + (op == OP_BFS ? 8.0 : 12.0) * (double)mr;
            r.gteps = r.kernel_ms > 0 ? (double)mr / (r.kernel_ms * 1e-3) / 1e9 : 0.0;
        }
    }
    if (res) *res = r;
    return s;
}

}  // extern "C"
