// noalloc.cu -- allocation-free variant of the persistent traversal run.
//
// Some callers cannot allocate device memory at the moment they want a traversal: a query-engine or
// database plugin whose host application owns every byte of GPU memory, a framework that routes all
// allocations through its own caching pool, or a latency-critical service loop in which cudaMalloc
// (which may synchronise the device) is not allowed. They can hand in the graph and the output, both
// in memory they already own, but not the traversal's working memory. This entry point keeps that
// working memory -- the control block, the two part queues and the per-vertex round stamps -- in one
// fixed file-scope device array, so the call itself never allocates.
//
// Limits and sharing: the array holds EEG_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that loads the
// library, for the life of the process. A run needs 256 + 4*(2*num_parts + num_nodes) bytes of it
// (rounded up to 256-byte blocks); larger graphs are rejected with EEG_ERR_INVALID. Every call on a
// device shares the same array and leaves its contents behind: each call clears what must start at
// zero (control block; stamps and values are reset by the kernel), and calls that overlap on the GPU
// (different streams or threads without ordering) race on it.
#include <mutex>

#include "traverse.cuh"

namespace {

constexpr size_t kScratchBytes = (size_t)EEG_NOALLOC_SCRATCH_BYTES;

// The working memory: never allocated, never freed.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};  // device address of g_noalloc_scratch, per device

size_t round256(size_t b) { return (b + 255u) & ~(size_t)255u; }

// Once per device, with that device current: look up the array's device address. The host-side
// symbol g_noalloc_scratch is only a stand-in for the device object and must never be passed to a kernel.
eeg_status scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) return eeg::cuda_fail(e, "cudaGetSymbolAddress(scratch)", __FILE__, __LINE__);
        g_addr[device] = p;
    }
    *out = (unsigned char*)g_addr[device];
    return EEG_OK;
}

}  // namespace

using namespace eeg;
using namespace eeg::trav;

extern "C" EEG_API eeg_status eeg_run_noalloc(eeg_algo algo, eeg_variant variant, uint32_t num_nodes,
                                              uint64_t num_parts, uint32_t K, const uint32_t* vstart,
                                              const uint32_t* vowner, const uint32_t* vcol, const uint32_t* vw,
                                              uint32_t source, uint32_t* dist, void* stream,
                                              uint32_t* iterations) {
    if (algo != EEG_BFS && algo != EEG_SSSP && algo != EEG_SSWP && algo != EEG_CC) {
        set_last_error("eeg_run_noalloc: algo must be BFS, SSSP, SSWP or CC");
        return EEG_ERR_INVALID;
    }
    if ((unsigned)variant > 3u || num_nodes == 0 || source >= num_nodes || !vstart || !dist ||
        (num_parts && (!vowner || !vcol || (algo != EEG_BFS && !vw)))) {
        set_last_error("eeg_run_noalloc: invalid argument (null pointer, empty graph or source out of range)");
        return EEG_ERR_INVALID;
    }
    if (K != 4 && K != 8 && K != 16) {
        set_last_error("eeg_run_noalloc: K must be 4, 8 or 16");
        return EEG_ERR_UNSUPPORTED;
    }
    const size_t q_bytes = round256(4 * (size_t)(num_parts ? num_parts : 1));
    const size_t need = round256(sizeof(TravCtrl)) + 2 * q_bytes + round256(4 * (size_t)num_nodes);
    if (num_parts > 0xFFFFFFFFull || need > kScratchBytes) {
        set_last_error("eeg_run_noalloc: graph needs " + std::to_string(need) + " bytes of working memory, more than the " +
                       std::to_string(kScratchBytes) + "-byte fixed array (use eeg_run)");
        return EEG_ERR_INVALID;
    }
    int device = 0;
    EEG_CUDA(cudaGetDevice(&device));
    if (device < 0 || device >= kMaxDevices) {
        set_last_error("eeg_run_noalloc: device index out of range");
        return EEG_ERR_INVALID;
    }
    unsigned char* base = nullptr;
    EEG_TRY(scratch_address(device, &base));
    cudaStream_t st = (cudaStream_t)stream;
    TravCtrl* ctrl = (TravCtrl*)base;
    uint32_t* q0 = (uint32_t*)(base + round256(sizeof(TravCtrl)));
    uint32_t* q1 = (uint32_t*)((unsigned char*)q0 + q_bytes);
    uint32_t* stamp = (uint32_t*)((unsigned char*)q1 + q_bytes);
    EEG_CUDA(cudaMemsetAsync(ctrl, 0, sizeof(TravCtrl), st));  // the previous call's counters must not leak in

    TravArgs a{};
    a.n = num_nodes;
    a.P = (uint32_t)num_parts;
    a.vstart = vstart;
    a.vowner = vowner;
    a.vcol = vcol;
    a.vw = vw;
    a.dist = dist;  // the caller's output doubles as the value array
    a.q0 = q0;
    a.q1 = q1;
    a.stamp = stamp;
    a.ctrl = ctrl;
    a.activity = nullptr;
    a.activity_cap = 0;
    a.source = source;
    a.seed_all = variant == EEG_ASYNC_PUSH_DD ? 1u : 0u;
    a.partner = variant == EEG_SYNC_PUSH_TD ? 1u : 0u;
    a.max_iters = num_nodes > 0xFFFFFFF0u ? 0xFFFFFFFFu : num_nodes + 2u;
    a.timeout_ns = 10000ull * 1000000ull;
    const bool td = variant == EEG_ASYNC_PUSH_TD || variant == EEG_SYNC_PUSH_TD;
    eeg_status s;
    switch (algo) {
        case EEG_BFS: s = launch_bfs(a, td, K, device, 0, st); break;
        case EEG_SSSP: s = launch_sssp(a, td, K, device, 0, st); break;
        case EEG_SSWP: s = launch_sswp(a, td, K, device, 0, st); break;
        default: s = launch_cc(a, td, K, device, 0, st); break;
    }
    if (s != EEG_OK) return s;
    uint32_t words[4] = {0, 0, 0, 0};  // barrier words: arrive, abort, status, pad
    EEG_CUDA(cudaMemcpyAsync(words, &ctrl->bw, sizeof(words), cudaMemcpyDeviceToHost, st));
    uint32_t its = 0;
    EEG_CUDA(cudaMemcpyAsync(&its, &ctrl->iterations, sizeof(its), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    if (iterations) *iterations = its;
    if (words[2] == DEV_TIMEOUT) {
        set_last_error("grid barrier wait exceeded the timeout");
        return EEG_ERR_TIMEOUT;
    }
    if (words[2] == DEV_ITER_CAP) {
        set_last_error("iteration cap reached before the fixed point");
        return EEG_ERR_ITER_CAP;
    }
    if (words[2] == DEV_OVERFLOW) {
        set_last_error("internal error: a frontier queue exceeded its capacity");
        return EEG_ERR_CUDA;
    }
    return EEG_OK;
}
