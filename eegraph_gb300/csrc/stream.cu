// stream.cu -- graphs larger than device memory: active-subgraph streaming (Subway's model).
//
// Reference (the Subway code vendored in the reference repository): the active vertices of a round
// found by a labelling and prefix sums on the GPU and their out-edges gathered into one active edge
// list on 64 host threads (Subway/shared/subgraph_generator.cu:10-97, 126-195); that list cut into
// partitions of at most a quarter of device memory (Subway/shared/partitioner.cu:12-91,
// Subway/shared/subgraph.cu:8-48); each partition copied to the GPU and relaxed, one thread per active
// vertex (Subway/shared/gpu_kernels.cu), once per round in the sync programs and until the partition
// settles in the async ones (Subway/subway/{bfs,sssp,sswp,cc}-{sync,async}.cu).
//
// GB300 form. The graph's CSR (offsets and (target, weight) records) stays in page-locked host memory
// mapped into the GPU's address space; the device holds O(n) state (values, two active labellings,
// degrees, offsets, compaction arrays) and two partition buffers of a caller-set byte budget. A round:
//   1. k_s_flags + two device scans: the active vertices with out-edges, each split into ceil(deg/K)
//      parts (the K-bounded virtual nodes of the in-memory path), are compacted with their part offsets;
//   2. the round's parts are cut into partitions of at most the buffer's part capacity;
//   3. for each partition, k_s_gather reads its parts' edges straight from host memory over the
//      CPU-GPU link (consecutive threads read consecutive edges of a row) into K-aligned rows of an HBM
//      buffer, on a copy stream, while the previous partition is relaxed from the other buffer;
//   4. k_s_relax expands one part per thread with the relax operators of the persistent kernels; an
//      improved target is labelled active for the next round (sync). Async also repeats passes over the
//      partition's rows, expanding only the parts of vertices improved in the previous pass, until no
//      vertex of the partition's id range improved (the subgraph is already in HBM).
// Results are the fixed points of the in-memory path (BFS levels, Dijkstra distances, widest paths,
// min-plus labels), whatever the budget or variant.
#include <algorithm>
#include <cstring>
#include <vector>

#include "traverse.cuh"

struct eeg_stream {
    int device = 0;
    uint32_t n = 0;
    uint64_t m = 0;
    uint32_t K = 8;
    uint64_t budget = 0;       // device bytes for the two partition buffers
    uint32_t cap_parts = 0;    // parts per partition buffer
    // host CSR (page-locked, mapped)
    uint64_t* h_off = nullptr;  // n+1
    uint2* h_rec = nullptr;     // m (target, weight)
    const uint2* d_rec = nullptr;  // device-side address of h_rec
    // device state
    uint64_t* d_off = nullptr;
    uint32_t* d_deg = nullptr;
    uint32_t* d_dist = nullptr;
    uint8_t* d_lab[2] = {nullptr, nullptr};
    uint32_t* d_dirty = nullptr;
    uint32_t* d_flag = nullptr;    // n+1, then its exclusive scan in place
    uint32_t* d_cnt = nullptr;     // n+1, then its exclusive scan in place (part offsets)
    uint32_t* d_active = nullptr;  // compacted active vertices
    uint32_t* d_cstart = nullptr;  // their part offsets (+ the total)
    uint32_t* d_tmp = nullptr;     // scan partials
    uint32_t* d_col[2] = {nullptr, nullptr};
    uint32_t* d_w[2] = {nullptr, nullptr};
    uint32_t* d_owner[2] = {nullptr, nullptr};
    uint32_t* d_again = nullptr;
    unsigned long long* d_stats = nullptr;  // pushes, updates, reached n_r, m_r
    cudaStream_t copy = nullptr;
    cudaEvent_t ev_start = nullptr, ev_end = nullptr;
    cudaEvent_t ev_gathered[2] = {nullptr, nullptr}, ev_relaxed[2] = {nullptr, nullptr};
    cudaEvent_t ev_ready = nullptr;  // the round's compaction is done (gathers may start)
};

namespace eeg {
namespace stream {

constexpr int S_TPB = 256;

template <int OP>
__global__ void k_s_init(uint32_t n, uint32_t source, uint32_t seed_all, uint32_t* dist, uint8_t* lab0,
                         uint8_t* lab1, uint32_t* dirty) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        dist[v] = trav::init_value<OP>(v, source);
        lab0[v] = (seed_all || v == source) ? 1 : 0;
        lab1[v] = 0;
        dirty[v] = 0;
    }
}

// flag[v] = v is active and has out-edges; cnt[v] = its parts; index n holds zeros (scans give totals)
__global__ void k_s_flags(uint32_t n, uint32_t K, const uint8_t* __restrict__ lab, const uint32_t* __restrict__ deg,
                          uint32_t* __restrict__ flag, uint32_t* __restrict__ cnt) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x) {
        const uint32_t d = v < n && lab[v] ? deg[v] : 0u;
        flag[v] = d ? 1u : 0u;
        cnt[v] = (d + K - 1) / K;
    }
}

// compaction: active[i] = the i-th flagged vertex, cstart[i] = its first part; cstart[nact] = total
__global__ void k_s_compact(uint32_t n, const uint32_t* __restrict__ deg, const uint8_t* __restrict__ lab,
                            const uint32_t* __restrict__ fidx, const uint32_t* __restrict__ pstart,
                            uint32_t* __restrict__ active, uint32_t* __restrict__ cstart) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x) {
        if (v == n) {
            cstart[fidx[n]] = pstart[n];
        } else if (lab[v] && deg[v]) {
            active[fidx[v]] = v;
            cstart[fidx[v]] = pstart[v];
        }
    }
}

// Gather of the parts [p0, p0 + np) of the round into K-aligned rows: a block covers S_TPB / K parts.
// Thread 0 finds the compacted index of the block's first part by binary search; the block's owners
// (at most one per part) and their part offsets are staged in shared memory, where each thread finds
// its part's owner. Slot j of part P of vertex v holds edge off[v] + (P - first part of v) * K + j.
template <int K>
__global__ void __launch_bounds__(S_TPB) k_s_gather(uint32_t nact, const uint32_t* __restrict__ active,
                                                    const uint32_t* __restrict__ cstart,
                                                    const uint64_t* __restrict__ off, const uint2* rec,
                                                    uint32_t p0, uint32_t np, uint32_t* __restrict__ col,
                                                    uint32_t* __restrict__ w, uint32_t* __restrict__ owner) {
    constexpr uint32_t BPP = S_TPB / K;  // parts per block
    __shared__ uint32_t s_first;
    __shared__ uint32_t s_cs[BPP + 1], s_v[BPP + 1];
    const uint32_t lp0 = blockIdx.x * BPP;  // first local part of the block
    if (lp0 >= np) return;
    if (threadIdx.x == 0) {
        const uint32_t P = p0 + lp0;
        uint32_t lo = 0, hi = nact - 1;  // largest i with cstart[i] <= P
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (cstart[mid] <= P) lo = mid;
            else hi = mid - 1;
        }
        s_first = lo;
    }
    __syncthreads();
    const uint32_t i0 = s_first;
    if (threadIdx.x <= BPP) {
        const uint32_t i = i0 + threadIdx.x;
        s_cs[threadIdx.x] = i <= nact ? cstart[i] : 0xFFFFFFFFu;
        s_v[threadIdx.x] = i < nact ? active[i] : 0u;
    }
    __syncthreads();
    const uint32_t lp = lp0 + threadIdx.x / K, j = threadIdx.x % K;
    if (lp >= np) return;
    const uint32_t P = p0 + lp;
    uint32_t k = 0;  // largest k with s_cs[k] <= P (parts of the block span at most BPP owners)
#pragma unroll
    for (uint32_t step = 32; step >= 1; step >>= 1)
        if (k + step <= BPP && s_cs[k + step] <= P) k += step;
    const uint32_t v = s_v[k];
    const uint64_t e = off[v] + (uint64_t)(P - s_cs[k]) * K + j;
    uint2 r = make_uint2(NO_EDGE, 0u);
    if (e < off[v + 1]) r = rec[e];  // a read of host memory over the CPU-GPU link
    col[(size_t)lp * K + j] = r.x;
    w[(size_t)lp * K + j] = r.y;
    if (j == 0) owner[lp] = v;
}

// One part per thread. pass == 0: every part (sync, and the first pass of async); pass > 0: only parts
// whose owner improved in pass `pass - 1` of this partition (async). An improvement labels the target
// active for the next round; async also marks it dirty for this pass and raises `again` when the target
// lies in the partition's owner-id range.
template <int OP, int K>
__global__ void __launch_bounds__(S_TPB) k_s_relax(uint32_t np, const uint32_t* __restrict__ owner,
                                                   const uint32_t* __restrict__ col, const uint32_t* __restrict__ w,
                                                   uint32_t* dist, uint8_t* lab_next, uint32_t* dirty, uint32_t pass_id,
                                                   uint32_t only_dirty, uint32_t mark, uint32_t* again,
                                                   uint32_t cc_zero, unsigned long long* stats) {
    __shared__ unsigned long long s_st[2];
    if (threadIdx.x == 0) s_st[0] = s_st[1] = 0ull;
    __syncthreads();
    const uint32_t p = blockIdx.x * S_TPB + threadIdx.x;
    unsigned long long pushes = 0, upd = 0;
    if (p < np) {
        const uint32_t v = owner[p];
        const bool go = !only_dirty || dirty[v] == pass_id - 1u;
        const uint32_t d = dist[v];
        if (go && !trav::unreached<OP>(d)) {
            const uint32_t vlo = owner[0], vhi = owner[np - 1];
            uint32_t c[K], wt[K];
#pragma unroll
            for (int i = 0; i < K; ++i) {
                c[i] = col[(size_t)p * K + i];
                wt[i] = w[(size_t)p * K + i];
            }
#pragma unroll
            for (int i = 0; i < K; ++i) {
                if (c[i] == NO_EDGE) continue;
                ++pushes;
                const uint32_t nd = trav::relax_value<OP>(d, OP == OP_BFS ? 1u : (cc_zero ? 0u : wt[i]));
                if (trav::better<OP>(nd, dist[c[i]])) {
                    const uint32_t prev = trav::atomic_improve<OP>(&dist[c[i]], nd);
                    if (trav::better<OP>(nd, prev)) {
                        ++upd;
                        lab_next[c[i]] = 1;
                        if (mark) {
                            dirty[c[i]] = pass_id;
                            if (c[i] >= vlo && c[i] <= vhi) *again = 1u;
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        pushes += __shfl_down_sync(0xffffffffu, pushes, o);
        upd += __shfl_down_sync(0xffffffffu, upd, o);
    }
    if ((threadIdx.x & 31u) == 0 && (pushes | upd)) {
        atomicAdd(&s_st[0], pushes);
        atomicAdd(&s_st[1], upd);
    }
    __syncthreads();
    if (threadIdx.x == 0 && (s_st[0] | s_st[1])) {
        atomicAdd(&stats[0], s_st[0]);
        atomicAdd(&stats[1], s_st[1]);
    }
}

template <int OP>
eeg_status launch_init(eeg_stream* s, uint32_t source, bool seed_all, unsigned grid, cudaStream_t st) {
    k_s_init<OP><<<grid, S_TPB, 0, st>>>(s->n, source, seed_all ? 1u : 0u, s->d_dist, s->d_lab[0], s->d_lab[1],
                                          s->d_dirty);
    EEG_CUDA(cudaGetLastError());
    return EEG_OK;
}

template <int OP, int K>
void launch_relax(eeg_stream* s, int b, uint32_t np, uint8_t* lab_next, uint32_t pass_id, bool only_dirty, bool mark,
                  bool cc_zero, cudaStream_t st) {
    k_s_relax<OP, K><<<(np + S_TPB - 1) / S_TPB, S_TPB, 0, st>>>(np, s->d_owner[b], s->d_col[b], s->d_w[b], s->d_dist,
                                                                  lab_next, s->d_dirty, pass_id, only_dirty ? 1u : 0u,
                                                                  mark ? 1u : 0u, s->d_again, cc_zero ? 1u : 0u,
                                                                  s->d_stats);
}

template <int OP>
void relax_dispatch(eeg_stream* s, int b, uint32_t np, uint8_t* lab_next, uint32_t pass_id, bool only_dirty, bool mark,
                    bool cc_zero, cudaStream_t st) {
    switch (s->K) {
        case 4: launch_relax<OP, 4>(s, b, np, lab_next, pass_id, only_dirty, mark, cc_zero, st); break;
        case 8: launch_relax<OP, 8>(s, b, np, lab_next, pass_id, only_dirty, mark, cc_zero, st); break;
        default: launch_relax<OP, 16>(s, b, np, lab_next, pass_id, only_dirty, mark, cc_zero, st); break;
    }
}

void gather_dispatch(eeg_stream* s, int b, uint32_t nact, uint32_t p0, uint32_t np, cudaStream_t st) {
    const uint32_t bpp = S_TPB / s->K;
    const unsigned blocks = (np + bpp - 1) / bpp;
    switch (s->K) {
        case 4:
            k_s_gather<4><<<blocks, S_TPB, 0, st>>>(nact, s->d_active, s->d_cstart, s->d_off, s->d_rec, p0, np,
                                                    s->d_col[b], s->d_w[b], s->d_owner[b]);
            break;
        case 8:
            k_s_gather<8><<<blocks, S_TPB, 0, st>>>(nact, s->d_active, s->d_cstart, s->d_off, s->d_rec, p0, np,
                                                    s->d_col[b], s->d_w[b], s->d_owner[b]);
            break;
        default:
            k_s_gather<16><<<blocks, S_TPB, 0, st>>>(nact, s->d_active, s->d_cstart, s->d_off, s->d_rec, p0, np,
                                                     s->d_col[b], s->d_w[b], s->d_owner[b]);
            break;
    }
}

}  // namespace stream
}  // namespace eeg

using namespace eeg;

namespace {

void stream_free(eeg_stream* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    cudaDeviceSynchronize();
    if (s->h_off) cudaFreeHost(s->h_off);
    if (s->h_rec) cudaFreeHost(s->h_rec);
    void* dev[] = {s->d_off, s->d_deg, s->d_dist, s->d_lab[0], s->d_lab[1], s->d_dirty, s->d_flag, s->d_cnt,
                   s->d_active, s->d_cstart, s->d_tmp, s->d_col[0], s->d_col[1], s->d_w[0], s->d_w[1],
                   s->d_owner[0], s->d_owner[1], s->d_again, s->d_stats};
    for (void* p : dev)
        if (p) cudaFree(p);
    if (s->copy) cudaStreamDestroy(s->copy);
    cudaEvent_t evs[] = {s->ev_start, s->ev_end, s->ev_gathered[0], s->ev_gathered[1], s->ev_relaxed[0],
                         s->ev_relaxed[1], s->ev_ready};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    delete s;
}

}  // namespace

extern "C" {

EEG_API eeg_status eeg_stream_create(const eeg_graph* g, uint32_t K, uint64_t device_budget_bytes, eeg_stream** out) {
    if (!g || !out) {
        set_last_error("eeg_stream_create: null argument");
        return EEG_ERR_INVALID;
    }
    *out = nullptr;
    if (K != 4 && K != 8 && K != 16) {
        set_last_error("eeg_stream_create: K must be 4, 8 or 16");
        return EEG_ERR_UNSUPPORTED;
    }
    const uint32_t n = g->num_nodes;
    const uint64_t m = g->num_edges;
    if (n == 0) {
        set_last_error("eeg_stream_create: graph has no vertices");
        return EEG_ERR_INVALID;
    }
    // every round's part offsets are 32-bit: sum over v of ceil(deg/K) < 2^32
    if (m / K + n >= 0xFFFFFFF0ull) {
        set_last_error("eeg_stream_create: more than 2^32 virtual parts (use a larger K)");
        return EEG_ERR_UNSUPPORTED;
    }
    eeg_stream* s = new eeg_stream();
    s->n = n;
    s->m = m;
    s->K = K;
    auto fail = [&](eeg_status st) {
        stream_free(s);
        return st;
    };
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) return fail(cuda_fail(e, "cudaGetDevice", __FILE__, __LINE__));
    // host CSR: offsets, then (target, weight) records grouped by source in input order (1-based ids
    // are shifted down by one, as the in-memory builds do)
    const uint32_t shift = g->has_zero_id ? 0u : 1u;
    if ((e = cudaHostAlloc((void**)&s->h_off, sizeof(uint64_t) * ((size_t)n + 1), cudaHostAllocMapped)) != cudaSuccess ||
        (e = cudaHostAlloc((void**)&s->h_rec, sizeof(uint2) * std::max<uint64_t>(m, 1), cudaHostAllocMapped)) != cudaSuccess)
        return fail(cuda_fail(e, "cudaHostAlloc", __FILE__, __LINE__));
    std::vector<uint32_t> deg(n, 0);
    for (uint64_t i = 0; i < m; ++i) {
        const uint32_t a = g->src[i] - shift, b = g->dst[i] - shift;
        if (a >= n || b >= n) {
            set_last_error("eeg_stream_create: edge endpoint outside num_nodes");
            return fail(EEG_ERR_INVALID);
        }
        deg[a]++;
    }
    s->h_off[0] = 0;
    for (uint32_t v = 0; v < n; ++v) s->h_off[v + 1] = s->h_off[v] + deg[v];
    {
        std::vector<uint64_t> pos(s->h_off, s->h_off + n);
        const bool wt = !g->weight.empty();
        for (uint64_t i = 0; i < m; ++i) {
            const uint32_t a = g->src[i] - shift;
            s->h_rec[pos[a]++] = make_uint2(g->dst[i] - shift, wt ? g->weight[i] : 1u);
        }
    }
    void* dp = nullptr;
    if ((e = cudaHostGetDevicePointer(&dp, s->h_rec, 0)) != cudaSuccess)
        return fail(cuda_fail(e, "cudaHostGetDevicePointer", __FILE__, __LINE__));
    s->d_rec = (const uint2*)dp;
    // device state, O(n)
    const size_t n1 = (size_t)n + 1;
    const uint64_t tmpw = device_scan_tmp_words(n1);
    if ((e = cudaMalloc((void**)&s->d_off, sizeof(uint64_t) * n1)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_deg, sizeof(uint32_t) * n)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_dist, sizeof(uint32_t) * n)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_lab[0], n)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_lab[1], n)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_dirty, sizeof(uint32_t) * n)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_flag, sizeof(uint32_t) * n1)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_cnt, sizeof(uint32_t) * n1)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_active, sizeof(uint32_t) * n)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_cstart, sizeof(uint32_t) * n1)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_tmp, sizeof(uint32_t) * tmpw)) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_again, sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMalloc((void**)&s->d_stats, 4 * sizeof(unsigned long long))) != cudaSuccess)
        return fail(cuda_fail(e, "cudaMalloc", __FILE__, __LINE__));
    if ((e = cudaMemcpy(s->d_off, s->h_off, sizeof(uint64_t) * n1, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(s->d_deg, deg.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(cuda_fail(e, "cudaMemcpy", __FILE__, __LINE__));
    // the partition buffers: two of (K targets + K weights + an owner) per part
    const uint64_t per_part = 2ull * (8ull * K + 4ull);
    uint64_t budget = device_budget_bytes;
    if (budget == 0) {  // a quarter of the free device memory, as Subway sizes its partition buffer
        size_t fr = 0, tot = 0;
        if ((e = cudaMemGetInfo(&fr, &tot)) != cudaSuccess) return fail(cuda_fail(e, "cudaMemGetInfo", __FILE__, __LINE__));
        budget = fr / 4;
    }
    const uint64_t all_parts = m / K + n + 1;
    uint64_t cap = budget / per_part;
    if (cap == 0) {
        set_last_error("eeg_stream_create: the device budget holds no part (at least " + std::to_string(per_part) +
                       " bytes are needed)");
        return fail(EEG_ERR_INVALID);
    }
    cap = std::min<uint64_t>(cap, all_parts);
    cap = std::min<uint64_t>(cap, 0x7FFFFFFFull);
    s->cap_parts = (uint32_t)cap;
    s->budget = cap * per_part;
    for (int b = 0; b < 2; ++b) {
        if ((e = cudaMalloc((void**)&s->d_col[b], sizeof(uint32_t) * K * cap)) != cudaSuccess ||
            (e = cudaMalloc((void**)&s->d_w[b], sizeof(uint32_t) * K * cap)) != cudaSuccess ||
            (e = cudaMalloc((void**)&s->d_owner[b], sizeof(uint32_t) * cap)) != cudaSuccess)
            return fail(cuda_fail(e, "cudaMalloc (partition buffers)", __FILE__, __LINE__));
    }
    if ((e = cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking)) != cudaSuccess)
        return fail(cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__));
    cudaEvent_t* evs[] = {&s->ev_start, &s->ev_end};
    for (cudaEvent_t* ev : evs)
        if ((e = cudaEventCreate(ev)) != cudaSuccess) return fail(cuda_fail(e, "cudaEventCreate", __FILE__, __LINE__));
    cudaEvent_t* sync_evs[] = {&s->ev_gathered[0], &s->ev_gathered[1], &s->ev_relaxed[0], &s->ev_relaxed[1],
                               &s->ev_ready};
    for (cudaEvent_t* ev : sync_evs)
        if ((e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming)) != cudaSuccess)
            return fail(cuda_fail(e, "cudaEventCreate", __FILE__, __LINE__));
    *out = s;
    return EEG_OK;
}

EEG_API eeg_status eeg_stream_get_info(const eeg_stream* s, eeg_stream_info* o) {
    if (!s || !o) {
        set_last_error("eeg_stream_get_info: null argument");
        return EEG_ERR_INVALID;
    }
    o->num_nodes = s->n;
    o->num_edges = s->m;
    o->K = s->K;
    o->partition_parts = s->cap_parts;
    o->device_budget_bytes = s->budget;
    o->host_bytes = sizeof(uint64_t) * ((uint64_t)s->n + 1) + sizeof(uint2) * s->m;
    return EEG_OK;
}

EEG_API void eeg_stream_destroy(eeg_stream* s) { stream_free(s); }

}  // extern "C"

namespace {

template <int OP>
eeg_status stream_run_op(eeg_stream* s, bool async, uint32_t source, const eeg_options& o, cudaStream_t st,
                         eeg_result* r) {
    using namespace eeg::stream;
    const uint32_t n = s->n;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(((uint64_t)n + S_TPB) / S_TPB,
                                                                             (uint64_t)sm_count(s->device) * 16));
    const bool cc_zero = OP == OP_CC && o.cc_components;
    const uint32_t max_rounds = o.max_iterations ? o.max_iterations : (n > 0xFFFFFFF0u ? 0xFFFFFFFFu : n + 2u);
    const uint32_t max_passes = 1000;  // async passes per partition (more only delay work to the next round)
    EEG_CUDA(cudaMemsetAsync(s->d_stats, 0, 4 * sizeof(unsigned long long), st));
    EEG_CUDA(cudaEventRecord(s->ev_start, st));
    EEG_TRY(launch_init<OP>(s, source, OP == OP_CC, grid, st));
    for (int b = 0; b < 2; ++b) EEG_CUDA(cudaEventRecord(s->ev_relaxed[b], st));
    uint32_t rounds = 0, launches = 1, pass_id = 0;
    uint64_t parts_total = 0, partitions = 0;
    eeg_status status = EEG_OK;
    for (;; ++rounds) {
        uint8_t* lab_cur = s->d_lab[rounds & 1u];
        uint8_t* lab_nxt = s->d_lab[(rounds & 1u) ^ 1u];
        k_s_flags<<<grid, S_TPB, 0, st>>>(n, s->K, lab_cur, s->d_deg, s->d_flag, s->d_cnt);
        EEG_TRY(device_scan_u32(s->d_flag, s->d_flag, (uint64_t)n + 1, false, SCAN_ADD, s->d_tmp, st));
        EEG_TRY(device_scan_u32(s->d_cnt, s->d_cnt, (uint64_t)n + 1, false, SCAN_ADD, s->d_tmp, st));
        launches += 7;
        uint32_t tot[2] = {0, 0};  // active vertices with out-edges, their parts
        EEG_CUDA(cudaMemcpyAsync(&tot[0], s->d_flag + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        EEG_CUDA(cudaMemcpyAsync(&tot[1], s->d_cnt + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        EEG_CUDA(cudaStreamSynchronize(st));
        if (tot[1] == 0) break;
        if (rounds >= max_rounds) {
            set_last_error("iteration cap reached before the fixed point");
            status = EEG_ERR_ITER_CAP;
            break;
        }
        k_s_compact<<<grid, S_TPB, 0, st>>>(n, s->d_deg, lab_cur, s->d_flag, s->d_cnt, s->d_active, s->d_cstart);
        EEG_CUDA(cudaMemsetAsync(lab_nxt, 0, n, st));  // this round's improvements label the next round
        EEG_CUDA(cudaEventRecord(s->ev_ready, st));
        EEG_CUDA(cudaStreamWaitEvent(s->copy, s->ev_ready, 0));
        ++launches;
        const uint32_t nq = (tot[1] + s->cap_parts - 1) / s->cap_parts;
        for (uint32_t q = 0; q < nq; ++q) {
            const int b = (int)(q & 1u);
            const uint32_t p0 = q * s->cap_parts;
            const uint32_t np = std::min<uint32_t>(s->cap_parts, tot[1] - p0);
            // buffer b is free once the partition that used it two steps ago is relaxed
            EEG_CUDA(cudaStreamWaitEvent(s->copy, s->ev_relaxed[b], 0));
            gather_dispatch(s, b, tot[0], p0, np, s->copy);
            EEG_CUDA(cudaGetLastError());
            EEG_CUDA(cudaEventRecord(s->ev_gathered[b], s->copy));
            EEG_CUDA(cudaStreamWaitEvent(st, s->ev_gathered[b], 0));
            ++pass_id;
            if (async) EEG_CUDA(cudaMemsetAsync(s->d_again, 0, sizeof(uint32_t), st));
            relax_dispatch<OP>(s, b, np, lab_nxt, pass_id, false, async, cc_zero, st);
            EEG_CUDA(cudaGetLastError());
            launches += 2;
            // async: relax the partition again from HBM while its own vertices keep improving
            for (uint32_t pass = 1; async && pass < max_passes; ++pass) {
                uint32_t again = 0;
                EEG_CUDA(cudaMemcpyAsync(&again, s->d_again, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
                EEG_CUDA(cudaStreamSynchronize(st));
                if (!again) break;
                ++pass_id;
                EEG_CUDA(cudaMemsetAsync(s->d_again, 0, sizeof(uint32_t), st));
                relax_dispatch<OP>(s, b, np, lab_nxt, pass_id, true, true, cc_zero, st);
                EEG_CUDA(cudaGetLastError());
                ++launches;
            }
            EEG_CUDA(cudaEventRecord(s->ev_relaxed[b], st));
        }
        parts_total += tot[1];
        partitions += nq;
    }
    EEG_CUDA(cudaEventRecord(s->ev_end, st));
    trav::k_reached<OP><<<grid, 256, 0, st>>>(s->d_dist, s->d_deg, n, s->d_stats + 2);
    EEG_CUDA(cudaGetLastError());
    ++launches;
    unsigned long long h[4];
    EEG_CUDA(cudaMemcpyAsync(h, s->d_stats, sizeof(h), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    EEG_CUDA(cudaEventElapsedTime(&ms, s->ev_start, s->ev_end));
    r->kernel_ms = ms;
    r->iterations = rounds;
    r->parts_processed = parts_total;
    r->edges_scanned = h[0];
    r->updates = h[1];
    r->reached_vertices = h[2];
    r->reached_edges = h[3];
    r->algorithmic_bytes = 12.0 * (double)h[2] + (OP == OP_BFS ? 8.0 : 12.0) * (double)h[3];
    r->gteps = ms > 0 ? (double)h[3] / (ms * 1e-3) / 1e9 : 0.0;
    r->launches = launches;
    r->partitions = (uint32_t)std::min<uint64_t>(partitions, 0xFFFFFFFFull);
    return status;
}

}  // namespace

extern "C" {

EEG_API eeg_status eeg_stream_run(eeg_stream* s, eeg_algo algo, eeg_variant variant, uint32_t source,
                                  const eeg_options* opts, uint32_t* out, int out_on_device, void* stream,
                                  eeg_result* res) {
    if (!s) {
        set_last_error("eeg_stream_run: null handle");
        return EEG_ERR_INVALID;
    }
    if ((unsigned)variant > 3u) {
        set_last_error("eeg_stream_run: unknown variant");
        return EEG_ERR_INVALID;
    }
    if (algo == EEG_PR) {
        set_last_error("eeg_stream_run: PageRank is not streamed (BFS, SSSP, SSWP and CC are)");
        return EEG_ERR_UNSUPPORTED;
    }
    if (algo != EEG_CC && source >= s->n) {
        set_last_error("eeg_stream_run: source out of range");
        return EEG_ERR_INVALID;
    }
    eeg_options o;
    eeg_options_init(&o);
    if (opts) o = *opts;
    eeg_result r;
    memset(&r, 0, sizeof(r));
    EEG_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    const bool async = variant == EEG_ASYNC_PUSH_TD || variant == EEG_ASYNC_PUSH_DD;
    eeg_status status;
    switch (algo) {
        case EEG_BFS: status = stream_run_op<OP_BFS>(s, async, source, o, st, &r); break;
        case EEG_SSSP: status = stream_run_op<OP_SSSP>(s, async, source, o, st, &r); break;
        case EEG_SSWP: status = stream_run_op<OP_SSWP>(s, async, source, o, st, &r); break;
        case EEG_CC: status = stream_run_op<OP_CC>(s, async, source, o, st, &r); break;
        default: set_last_error("eeg_stream_run: unknown algorithm"); return EEG_ERR_INVALID;
    }
    if ((status == EEG_OK || status == EEG_ERR_ITER_CAP) && out) {
        EEG_CUDA(cudaMemcpyAsync(out, s->d_dist, sizeof(uint32_t) * s->n,
                                 out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
        EEG_CUDA(cudaStreamSynchronize(st));
    }
    if (res) *res = r;
    return status;
}

}  // extern "C"
