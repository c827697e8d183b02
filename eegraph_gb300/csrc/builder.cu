// builder.cu -- GPU construction of the K-bounded virtual graph.
//
// Replaces VirtualGraph::VirtualGraph + VirtualGraph::MakeGraph (reference src/virtual_graph.cpp:3-112,
// UM twin src/um_virtual_graph.cu:36-111), which build an interleaved host array on one core and
// drop every edge whose slot index reaches num_edges (src/virtual_graph.cpp:86-88). Here:
//
//   1. degree histogram            deg[s]++ for every edge (atomics in L2)
//   2. part counts                 np[v] = ceil(deg[v] / K)
//   3. exclusive scan              vstart[v] = sum_{u<v} np[u]; vstart[n] = P (numParts)
//   4. owner table (segmented)     vowner[vstart[v]] = v for v with parts, then inclusive max-scan
//   5. scatter                     edge r of vertex s -> slot vstart[s]*K + r (part r/K, lane r%K)
//
// The result is lossless. Part p of vertex v holds out-edges [ (p - vstart[v]) * K, +K ) of v in one
// K-slot row, so a thread reads a whole part with K/4 aligned 128-bit loads. Edges keep the order of
// the atomic rank within a vertex; fixed points do not depend on it.
#include <algorithm>
#include <cstdio>

#include "internal.hpp"

namespace eeg {

// ------------------------------------------------------------------ device-wide scan
namespace {

constexpr int SCAN_TPB = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr uint64_t SCAN_TILE = (uint64_t)SCAN_TPB * SCAN_ITEMS;

__device__ __forceinline__ uint32_t scan_op(uint32_t a, uint32_t b, int op) {
    return op == SCAN_ADD ? a + b : (a > b ? a : b);
}

__device__ __forceinline__ uint32_t warp_inclusive(uint32_t x, int op) {
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= (uint32_t)off) x = scan_op(x, y, op);
    }
    return x;
}

// CTA scan of one value per thread (blockDim == SCAN_TPB). Returns the EXCLUSIVE prefix
// (identity 0 for thread 0) and sets *total to the CTA aggregate.
__device__ __forceinline__ uint32_t cta_exclusive(uint32_t x, int op, uint32_t* s_warp, uint32_t* s_inc,
                                                  uint32_t* total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t inc = warp_inclusive(x, op);
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) s_warp[lane] = warp_inclusive(s_warp[lane], op);  // 32 warps
    __syncthreads();
    inc = warp > 0 ? scan_op(s_warp[warp - 1], inc, op) : inc;
    s_inc[threadIdx.x] = inc;
    __syncthreads();
    uint32_t ex = threadIdx.x > 0 ? s_inc[threadIdx.x - 1] : 0u;
    *total = s_warp[31];
    __syncthreads();
    return ex;
}

__global__ void __launch_bounds__(SCAN_TPB) k_scan_reduce(const uint32_t* __restrict__ in, uint64_t n,
                                                          uint32_t* __restrict__ partials, int op) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_inc[SCAN_TPB];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint32_t acc = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint64_t idx = base + (uint64_t)i * SCAN_TPB + threadIdx.x;
        if (idx < n) acc = scan_op(acc, in[idx], op);
    }
    uint32_t total;
    cta_exclusive(acc, op, s_warp, s_inc, &total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

// Single CTA: exclusive scan of the tile partials, in place.
__global__ void __launch_bounds__(SCAN_TPB) k_scan_partials(uint32_t* partials, uint64_t nt, int op) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_inc[SCAN_TPB];
    uint32_t carry = 0;
    for (uint64_t base = 0; base < nt; base += SCAN_TPB) {
        uint64_t idx = base + threadIdx.x;
        uint32_t x = idx < nt ? partials[idx] : 0u;
        uint32_t total;
        uint32_t ex = cta_exclusive(x, op, s_warp, s_inc, &total);
        if (idx < nt) partials[idx] = threadIdx.x == 0 ? carry : scan_op(carry, ex, op);
        carry = scan_op(carry, total, op);
    }
}

__global__ void __launch_bounds__(SCAN_TPB) k_scan_apply(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                         uint64_t n, const uint32_t* __restrict__ partials,
                                                         int inclusive, int op) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_inc[SCAN_TPB];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    // each thread owns SCAN_ITEMS consecutive items (blocked arrangement keeps scan order)
    uint32_t v[SCAN_ITEMS];
    const uint64_t t0 = base + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t acc = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint64_t idx = t0 + i;
        v[i] = idx < n ? in[idx] : 0u;
        acc = scan_op(acc, v[i], op);
    }
    uint32_t total;
    uint32_t ex = cta_exclusive(acc, op, s_warp, s_inc, &total);
    const uint32_t tile_prefix = partials[blockIdx.x];
    uint32_t run = threadIdx.x == 0 ? tile_prefix : scan_op(tile_prefix, ex, op);
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint64_t idx = t0 + i;
        uint32_t before = run;
        run = scan_op(run, v[i], op);
        if (idx < n) out[idx] = inclusive ? run : before;
    }
}

}  // namespace

uint64_t device_scan_tmp_words(uint64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

eeg_status device_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, bool inclusive, ScanOp op,
                           uint32_t* tmp, cudaStream_t st) {
    if (n == 0) return EEG_OK;
    const uint64_t nt = (n + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_reduce<<<(unsigned)nt, SCAN_TPB, 0, st>>>(in, n, tmp, (int)op);
    k_scan_partials<<<1, SCAN_TPB, 0, st>>>(tmp, nt, (int)op);
    k_scan_apply<<<(unsigned)nt, SCAN_TPB, 0, st>>>(in, out, n, tmp, inclusive ? 1 : 0, (int)op);
    EEG_CUDA(cudaGetLastError());
    return EEG_OK;
}

// ------------------------------------------------------------------ builder kernels
namespace {

constexpr int B_TPB = 256;

__global__ void k_degree(const uint32_t* __restrict__ src, const uint32_t* __restrict__ dst, uint64_t m, uint32_t n,
                         uint32_t shift, uint32_t* __restrict__ deg, uint32_t* __restrict__ err) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = src[e] - shift, t = dst[e] - shift;
        if (s >= n || t >= n) {
            atomicOr(err, 1u);
            continue;
        }
        atomicAdd(&deg[s], 1u);
    }
}

// np[v] = ceil(deg/K) for v < n, np[n] = 0; also the max-degree vertex (lowest id among ties).
__global__ void k_nparts(const uint32_t* __restrict__ deg, uint32_t n, uint32_t K, uint32_t* __restrict__ np,
                         unsigned long long* __restrict__ best) {
    unsigned long long mine = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x) {
        if (v == n) {
            np[v] = 0;
            continue;
        }
        uint32_t d = deg[v];
        np[v] = (d + K - 1) / K;
        unsigned long long key = ((unsigned long long)d << 32) | (unsigned long long)(0xFFFFFFFFu - v);
        mine = key > mine ? key : mine;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_down_sync(0xffffffffu, mine, off);
        mine = o > mine ? o : mine;
    }
    if ((threadIdx.x & 31u) == 0 && mine) atomicMax(best, mine);
}

__global__ void k_heads(const uint32_t* __restrict__ vstart, uint32_t n, uint32_t* __restrict__ vowner) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        uint32_t a = vstart[v], b = vstart[v + 1];
        if (b > a) vowner[a] = v;
    }
}

__global__ void k_scatter(const uint32_t* __restrict__ src, const uint32_t* __restrict__ dst,
                          const uint32_t* __restrict__ w, uint64_t m, uint32_t shift, uint32_t K,
                          const uint32_t* __restrict__ vstart, uint32_t* __restrict__ cursor,
                          uint32_t* __restrict__ vcol, uint32_t* __restrict__ vw) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = src[e] - shift, t = dst[e] - shift;
        uint32_t r = atomicAdd(&cursor[s], 1u);
        size_t slot = (size_t)vstart[s] * K + r;
        vcol[slot] = t;
        if (vw) vw[slot] = w ? w[e] : 1u;
    }
}

}  // namespace

int sm_count(int device) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || v <= 0) v = 132;
    return v;
}

static unsigned grid_for(uint64_t work, int device) {
    uint64_t blocks = (work + B_TPB - 1) / B_TPB;
    uint64_t cap = (uint64_t)sm_count(device) * 16;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    return (unsigned)blocks;
}

// Build one direction. reverse: edges (s,t) are inserted as (t,s) -- the transposed graph.
eeg_status build_direction(eeg_vgraph* vg, VDir* d, const uint32_t* d_src, const uint32_t* d_dst,
                           const uint32_t* d_w, bool reverse, cudaStream_t st) {
    const uint32_t n = vg->n, K = vg->K;
    const uint64_t m = vg->m;
    const uint32_t shift = (vg->flags & EEG_VG_SHIFT_ONE) ? 1u : 0u;
    const uint32_t* a = reverse ? d_dst : d_src;
    const uint32_t* b = reverse ? d_src : d_dst;

    EEG_TRY(vg_alloc(vg, (void**)&d->deg, sizeof(uint32_t) * (size_t)(n + 1)));
    EEG_TRY(vg_alloc(vg, (void**)&d->vstart, sizeof(uint32_t) * (size_t)(n + 1)));
    uint32_t* np = nullptr;
    uint32_t* tmp = nullptr;
    uint32_t* err = nullptr;
    unsigned long long* best = nullptr;
    const uint64_t tmpw = device_scan_tmp_words(std::max<uint64_t>(n + 1, 1));
    EEG_CUDA(cudaMallocAsync((void**)&np, sizeof(uint32_t) * (size_t)(n + 1), st));
    EEG_CUDA(cudaMallocAsync((void**)&tmp, sizeof(uint32_t) * (size_t)tmpw, st));
    EEG_CUDA(cudaMallocAsync((void**)&err, 16, st));
    best = (unsigned long long*)(err + 2);
    EEG_CUDA(cudaMemsetAsync(err, 0, 16, st));
    EEG_CUDA(cudaMemsetAsync(d->deg, 0, sizeof(uint32_t) * (size_t)(n + 1), st));

    k_degree<<<grid_for(m, vg->device), B_TPB, 0, st>>>(a, b, m, n, shift, d->deg, err);
    k_nparts<<<grid_for((uint64_t)n + 1, vg->device), B_TPB, 0, st>>>(d->deg, n, K, np, best);
    EEG_TRY(device_scan_u32(np, d->vstart, (uint64_t)n + 1, false, SCAN_ADD, tmp, st));

    uint32_t hbuf[4] = {0, 0, 0, 0};
    uint32_t P32 = 0;
    EEG_CUDA(cudaMemcpyAsync(hbuf, err, 16, cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaMemcpyAsync(&P32, d->vstart + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    if (hbuf[0]) {
        cudaFreeAsync(np, st);
        cudaFreeAsync(tmp, st);
        cudaFreeAsync(err, st);
        set_last_error("edge endpoint outside [0, num_nodes)");
        return EEG_ERR_INVALID;
    }
    if (!reverse) {
        unsigned long long key = ((unsigned long long)hbuf[3] << 32) | hbuf[2];
        vg->max_deg = (uint32_t)(key >> 32);
        vg->max_deg_vertex = key ? 0xFFFFFFFFu - (uint32_t)(key & 0xFFFFFFFFu) : 0u;
    }
    const uint64_t P = P32;
    d->P = P;
    const size_t slots = (size_t)P * K;
    EEG_TRY(vg_alloc(vg, (void**)&d->vowner, sizeof(uint32_t) * (size_t)std::max<uint64_t>(P, 1)));
    EEG_TRY(vg_alloc(vg, (void**)&d->vcol, sizeof(uint32_t) * std::max<size_t>(slots, 4)));
    const bool with_w = (d_w != nullptr) || (!reverse && vg->weighted);
    if (with_w) EEG_TRY(vg_alloc(vg, (void**)&d->vw, sizeof(uint32_t) * std::max<size_t>(slots, 4)));

    if (P > 0) {
        EEG_CUDA(cudaMemsetAsync(d->vowner, 0, sizeof(uint32_t) * (size_t)P, st));
        EEG_CUDA(cudaMemsetAsync(d->vcol, 0xFF, sizeof(uint32_t) * slots, st));
        if (d->vw) EEG_CUDA(cudaMemsetAsync(d->vw, 0, sizeof(uint32_t) * slots, st));
        k_heads<<<grid_for(n, vg->device), B_TPB, 0, st>>>(d->vstart, n, d->vowner);
        uint32_t* tmp2 = nullptr;
        EEG_CUDA(cudaMallocAsync((void**)&tmp2, sizeof(uint32_t) * (size_t)device_scan_tmp_words(P), st));
        EEG_TRY(device_scan_u32(d->vowner, d->vowner, P, true, SCAN_MAX, tmp2, st));
        EEG_CUDA(cudaFreeAsync(tmp2, st));
        // cursor reuses np (n+1 words)
        EEG_CUDA(cudaMemsetAsync(np, 0, sizeof(uint32_t) * (size_t)(n + 1), st));
        k_scatter<<<grid_for(m, vg->device), B_TPB, 0, st>>>(a, b, d_w, m, shift, K, d->vstart, np, d->vcol, d->vw);
    }
    EEG_CUDA(cudaGetLastError());
    EEG_CUDA(cudaFreeAsync(np, st));
    EEG_CUDA(cudaFreeAsync(tmp, st));
    EEG_CUDA(cudaFreeAsync(err, st));
    vg->bytes += sizeof(uint32_t) * ((size_t)(n + 1) * 2 + (size_t)P + slots * (with_w ? 2 : 1));
    return EEG_OK;
}

}  // namespace eeg
