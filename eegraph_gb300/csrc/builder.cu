// builder.cu -- GPU construction of the K-bounded virtual graph.
//
// Replaces VirtualGraph::VirtualGraph + VirtualGraph::MakeGraph (reference src/virtual_graph.cpp:3-112,
// UM twin src/um_virtual_graph.cu:36-111), which build an interleaved host array on one core and
// drop every edge whose slot index reaches num_edges (src/virtual_graph.cpp:86-88). Here:
//
//   1. stable radix sort           (owner, neighbour[, weight]) by owner, 8-bit digits (no hot atomics:
//                                  a hub's edges are ranked inside each 2048-key tile)
//   2. runs                        first/last index of each owner -> degree
//   3. part counts + scan          np[v] = ceil(deg[v] / K); vstart = exclusive scan; vstart[n] = P
//   4. owner table (segmented)     vowner[vstart[v]] = v for v with parts, then inclusive max-scan
//   5. placement                   sorted edge of rank r of vertex s -> slot vstart[s]*K + r (part r/K)
//
// The result is lossless and deterministic. Part p of vertex v holds out-edges [ (p - vstart[v]) * K,
// +K ) of v in one K-slot row, in input order (the order MakeGraph gives them), so a thread reads a
// whole part with one or two aligned 256-bit loads.
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
// stable LSD radix sort of (owner, neighbour[, weight]) by owner: 8-bit digits, tiles of 2048 keys;
// warp w of a tile owns keys [w*256, w*256+256) of it and takes them 32 at a time, in order.
constexpr int R_TPB = 256;
constexpr int R_WARPS = R_TPB / 32;
constexpr int R_ITEMS = 8;  // rounds of 32 keys per warp
constexpr int R_TILE = R_TPB * R_ITEMS;
constexpr int R_BINS = 256;
static_assert(R_TPB == R_BINS, "one thread per digit in the cross-warp prefix");

// 0-based owner/neighbour (+ weight, or the arc index when eid != 0) of the m input edges into the sort
// buffers; with sym, arc m + e is the reverse of edge e. Endpoints outside [0, n) raise err.
__global__ void k_prepare(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, const uint32_t* __restrict__ w,
                          uint64_t m, uint32_t n, uint32_t shift, uint32_t* __restrict__ key, uint32_t* __restrict__ nb,
                          uint32_t* __restrict__ wt, uint32_t* __restrict__ err, int eid, int sym) {
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = a[e] - shift, t = b[e] - shift;
        if (s >= n || t >= n) {
            atomicOr(err, 1u);
            s = 0;
            t = 0;
        }
        const uint32_t wv = w ? w[e] : 1u;
        key[e] = s;
        nb[e] = t;
        if (wt) wt[e] = eid ? (uint32_t)e : wv;
        if (sym) {
            key[m + e] = t;
            nb[m + e] = s;
            if (wt) wt[m + e] = eid ? (uint32_t)(m + e) : wv;
        }
    }
}

// Same, four edges per thread with 128-bit loads and stores (all arrays 16-byte aligned, and m a
// multiple of 4 with sym): when the inputs are page-locked host memory read in place, four times the
// bytes are in flight per load.
__device__ __forceinline__ void prep_one(uint32_t s, uint32_t t, uint32_t n, uint32_t shift, uint32_t& ks, uint32_t& kt,
                                         uint32_t* err) {
    s -= shift;
    t -= shift;
    if (s >= n || t >= n) {
        atomicOr(err, 1u);
        s = 0;
        t = 0;
    }
    ks = s;
    kt = t;
}
__global__ void k_prepare4(const uint4* __restrict__ a, const uint4* __restrict__ b, const uint4* __restrict__ w,
                           uint64_t m, uint32_t n, uint32_t shift, uint4* __restrict__ key, uint4* __restrict__ nb,
                           uint4* __restrict__ wt, uint32_t* __restrict__ err, int eid, int sym) {
    const uint64_t m4 = m / 4, stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m4; i += stride) {
        const uint4 s4 = a[i], t4 = b[i];
        uint4 w4 = make_uint4(1u, 1u, 1u, 1u);
        if (w && !eid) w4 = w[i];
        uint4 k, c;
        prep_one(s4.x, t4.x, n, shift, k.x, c.x, err);
        prep_one(s4.y, t4.y, n, shift, k.y, c.y, err);
        prep_one(s4.z, t4.z, n, shift, k.z, c.z, err);
        prep_one(s4.w, t4.w, n, shift, k.w, c.w, err);
        key[i] = k;
        nb[i] = c;
        if (wt) {
            const uint32_t e = (uint32_t)(4 * i);
            wt[i] = eid ? make_uint4(e, e + 1u, e + 2u, e + 3u) : w4;
        }
        if (sym) {
            key[m4 + i] = c;
            nb[m4 + i] = k;
            if (wt) {
                const uint32_t e = (uint32_t)(m + 4 * i);
                wt[m4 + i] = eid ? make_uint4(e, e + 1u, e + 2u, e + 3u) : w4;
            }
        }
    }
    // tail (m % 4 edges)
    const uint32_t* a1 = reinterpret_cast<const uint32_t*>(a);
    const uint32_t* b1 = reinterpret_cast<const uint32_t*>(b);
    const uint32_t* w1 = reinterpret_cast<const uint32_t*>(w);
    for (uint64_t e = 4 * m4 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += stride) {
        uint32_t ks, kt;
        prep_one(a1[e], b1[e], n, shift, ks, kt, err);
        reinterpret_cast<uint32_t*>(key)[e] = ks;
        reinterpret_cast<uint32_t*>(nb)[e] = kt;
        if (wt) reinterpret_cast<uint32_t*>(wt)[e] = eid ? (uint32_t)e : (w1 ? w1[e] : 1u);
        if (sym) {  // not reached: sym takes this kernel only when m is a multiple of 4
            reinterpret_cast<uint32_t*>(key)[m + e] = kt;
            reinterpret_cast<uint32_t*>(nb)[m + e] = ks;
            if (wt) reinterpret_cast<uint32_t*>(wt)[m + e] = eid ? (uint32_t)(m + e) : (w1 ? w1[e] : 1u);
        }
    }
}

// digit counts of one tile, stored digit-major: hist[digit * ntiles + tile]
__global__ void __launch_bounds__(R_TPB) k_radix_hist(const uint32_t* __restrict__ key, uint64_t m, uint32_t shift,
                                                      uint32_t* __restrict__ hist, uint32_t ntiles) {
    __shared__ uint32_t h[R_BINS];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * R_TILE;
    uint32_t k[R_ITEMS];
#pragma unroll
    for (int j = 0; j < R_ITEMS; ++j) {
        const uint64_t idx = base + (uint64_t)j * R_TPB + threadIdx.x;
        k[j] = idx < m ? key[idx] : 0xFFFFFFFFu;
    }
#pragma unroll
    for (int j = 0; j < R_ITEMS; ++j) {
        const uint64_t idx = base + (uint64_t)j * R_TPB + threadIdx.x;
        if (idx < m) atomicAdd(&h[(k[j] >> shift) & (R_BINS - 1)], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile by digit: a key's place = the tile's global offset for its digit + the keys
// with that digit earlier in the tile (earlier warps, earlier rounds of its warp, lower lanes).
__global__ void __launch_bounds__(R_TPB) k_radix_scatter(const uint32_t* __restrict__ key_in,
                                                         const uint32_t* __restrict__ nb_in,
                                                         const uint32_t* __restrict__ w_in, uint32_t* __restrict__ key_out,
                                                         uint32_t* __restrict__ nb_out, uint32_t* __restrict__ w_out,
                                                         uint64_t m, uint32_t shift, const uint32_t* __restrict__ offs,
                                                         uint32_t ntiles) {
    __shared__ uint32_t s_cnt[R_WARPS][R_BINS];
    __shared__ uint32_t s_key[R_TILE], s_nb[R_TILE], s_w[R_TILE];
    __shared__ uint32_t s_dstart[R_BINS], s_goff[R_BINS], s_warp[33];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint64_t wbase = (uint64_t)blockIdx.x * R_TILE + (uint64_t)warp * (32 * R_ITEMS);
#pragma unroll
    for (int w = 0; w < R_WARPS; ++w) s_cnt[w][threadIdx.x] = 0;
    uint32_t k[R_ITEMS], v[R_ITEMS], wv[R_ITEMS], rank[R_ITEMS];
#pragma unroll
    for (int j = 0; j < R_ITEMS; ++j) {  // all loads first (coalesced: 32 consecutive keys per round)
        const uint64_t idx = wbase + (uint64_t)j * 32 + lane;
        const bool valid = idx < m;
        k[j] = valid ? key_in[idx] : 0u;
        v[j] = valid ? nb_in[idx] : 0u;
        wv[j] = (valid && w_out) ? w_in[idx] : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < R_ITEMS; ++j) {
        const uint64_t idx = wbase + (uint64_t)j * 32 + lane;
        const uint32_t digit = idx < m ? (k[j] >> shift) & (R_BINS - 1) : (uint32_t)R_BINS;
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t rk = __popc(peers & ((1u << lane) - 1u));
        const uint32_t before = digit < R_BINS ? s_cnt[warp][digit] : 0u;
        __syncwarp();
        if (digit < R_BINS && rk == 0) s_cnt[warp][digit] = before + __popc(peers);
        __syncwarp();
        rank[j] = before + rk;
    }
    __syncthreads();
    // per digit (thread = digit): offsets of each warp's keys inside the digit's run, and the run length
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < R_WARPS; ++w) {
        const uint32_t c = s_cnt[w][threadIdx.x];
        s_cnt[w][threadIdx.x] = cnt;
        cnt += c;
    }
    // the tile in digit order in shared memory: digit runs start at the exclusive scan of the counts
    uint32_t total;
    const uint32_t dstart = block_exclusive_sum(cnt, s_warp, &total);
    s_dstart[threadIdx.x] = dstart;
    s_goff[threadIdx.x] = offs[(size_t)threadIdx.x * ntiles + blockIdx.x];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < R_ITEMS; ++j) {
        const uint64_t idx = wbase + (uint64_t)j * 32 + lane;
        if (idx < m) {
            const uint32_t d = (k[j] >> shift) & (R_BINS - 1);
            const uint32_t lp = s_dstart[d] + s_cnt[warp][d] + rank[j];
            s_key[lp] = k[j];
            s_nb[lp] = v[j];
            if (w_out) s_w[lp] = wv[j];
        }
    }
    __syncthreads();
    // write the digit runs out: consecutive threads -> consecutive addresses inside each run
    for (uint32_t i = threadIdx.x; i < total; i += R_TPB) {
        const uint32_t kk = s_key[i];
        const uint32_t d = (kk >> shift) & (R_BINS - 1);
        const uint32_t gp = s_goff[d] + (i - s_dstart[d]);
        key_out[gp] = kk;
        nb_out[gp] = s_nb[i];
        if (w_out) w_out[gp] = s_w[i];
    }
}

// first and one-past-last index of every owner's run in the sorted keys
__global__ void k_runs(const uint32_t* __restrict__ key, uint64_t m, uint32_t* __restrict__ rs,
                       uint32_t* __restrict__ re) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t o = key[i];
        if (i == 0 || key[i - 1] != o) rs[o] = (uint32_t)i;
        if (i + 1 == m || key[i + 1] != o) re[o] = (uint32_t)(i + 1);
    }
}

// deg[v] = run length; np[v] = ceil(deg/K) for v < n, np[n] = 0; also the max-degree vertex
// (lowest id among ties).
__global__ void k_nparts(const uint32_t* __restrict__ rs, const uint32_t* __restrict__ re, uint32_t n, uint32_t K,
                         uint32_t* __restrict__ deg, uint32_t* __restrict__ np, unsigned long long* __restrict__ best) {
    unsigned long long mine = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += gridDim.x * blockDim.x) {
        if (v == n) {
            np[v] = 0;
            continue;
        }
        const uint32_t d = re[v] - rs[v];
        deg[v] = d;
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

// sorted edge i of owner o (rank r = i - rs[o]) goes to slot vstart[o]*K + r: part r/K, lane r%K
// With veid (edge-index mode) the sorted payload is the arc index: the weight is gathered from the
// input array by it (arc e >= m_in of a symmetrised build is the reverse of input edge e - m_in; m_in
// is 0 otherwise) and the index is kept per slot.
__global__ void k_place(const uint32_t* __restrict__ key, const uint32_t* __restrict__ nb, const uint32_t* __restrict__ wt,
                        uint64_t m, uint32_t K, const uint32_t* __restrict__ rs, const uint32_t* __restrict__ vstart,
                        uint32_t* __restrict__ vcol, uint32_t* __restrict__ vw, const uint32_t* __restrict__ w_in,
                        uint32_t* __restrict__ veid, uint64_t m_in) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t o = key[i];
        const size_t slot = (size_t)vstart[o] * K + (i - rs[o]);
        vcol[slot] = nb[i];
        if (veid) {
            const uint32_t e = wt[i];
            veid[slot] = e;
            if (vw) vw[slot] = w_in ? w_in[(m_in && e >= m_in) ? e - m_in : e] : 1u;
        } else if (vw) {
            vw[slot] = wt ? wt[i] : 1u;
        }
    }
}

// Out-degree histogram of the input edges (with sym, of both directions); endpoints outside [0, n)
// are counted nowhere (the transposed build reports them). The lowest OUTDEG_HOT ids count in shared
// memory first, each CTA adding its non-zero counters at the end: generators that do not permute ids
// (R-MAT) put their hubs there, and per-edge global atomics on a hub's counter queue at one L2 slice.
constexpr uint32_t OUTDEG_HOT = 8192;
__global__ void __launch_bounds__(256) k_outdeg(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                                                uint64_t m, uint32_t n, uint32_t shift, int sym,
                                                uint32_t* __restrict__ deg) {
    __shared__ uint32_t s_cnt[OUTDEG_HOT];
    for (uint32_t i = threadIdx.x; i < OUTDEG_HOT; i += blockDim.x) s_cnt[i] = 0u;
    __syncthreads();
    auto count = [&](uint32_t v) {
        if (v < OUTDEG_HOT) atomicAdd(&s_cnt[v], 1u);
        else atomicAdd(&deg[v], 1u);
    };
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = a[e] - shift, t = b[e] - shift;
        if (s < n && t < n) {
            count(s);
            if (sym) count(t);
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < OUTDEG_HOT && i < n; i += blockDim.x)
        if (s_cnt[i]) atomicAdd(&deg[i], s_cnt[i]);
}
// Largest degree and its smallest vertex, packed (degree << 32 | ~vertex) into one 64-bit max.
__global__ void k_deg_best(const uint32_t* __restrict__ deg, uint32_t n, unsigned long long* best) {
    unsigned long long b = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        if (deg[v]) b = max(b, ((unsigned long long)deg[v] << 32) | (0xFFFFFFFFu - v));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_down_sync(0xffffffffu, b, o));
    if ((threadIdx.x & 31u) == 0 && b) atomicMax(best, b);
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

namespace {
// stream-ordered temporaries released on every exit path
struct TempSet {
    cudaStream_t st;
    void* p[16] = {nullptr};
    int k = 0;
    explicit TempSet(cudaStream_t s) : st(s) {}
    eeg_status get(void** out, size_t bytes) {
        if (k == 16) {
            set_last_error("builder: too many temporaries");
            return EEG_ERR_INVALID;
        }
        cudaError_t e = cudaMallocAsync(out, bytes ? bytes : 4, st);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync(builder temporaries)", __FILE__, __LINE__);
        p[k++] = *out;
        return EEG_OK;
    }
    ~TempSet() {
        for (int i = 0; i < k; ++i) cudaFreeAsync(p[i], st);
    }
};
}  // namespace

eeg_status build_out_degrees(eeg_vgraph* vg, VDir* d, const uint32_t* d_src, const uint32_t* d_dst, cudaStream_t st) {
    const uint32_t n = vg->n;
    const bool sym = (vg->flags & EEG_VG_SYMMETRIZE) != 0;
    const uint64_t m_in = sym ? vg->m / 2 : vg->m;
    const uint32_t shift = (vg->flags & EEG_VG_SHIFT_ONE) ? 1u : 0u;
    EEG_TRY(vg_alloc(vg, (void**)&d->deg, sizeof(uint32_t) * (size_t)(n + 1)));
    TempSet T(st);
    unsigned long long* best = nullptr;
    EEG_TRY(T.get((void**)&best, sizeof(unsigned long long)));
    EEG_CUDA(cudaMemsetAsync(d->deg, 0, sizeof(uint32_t) * (size_t)(n + 1), st));
    EEG_CUDA(cudaMemsetAsync(best, 0, sizeof(unsigned long long), st));
    // two CTAs per SM: each flushes its shared counters once
    if (m_in)
        k_outdeg<<<(unsigned)std::max<uint64_t>(1, std::min<uint64_t>((m_in + 255) / 256, (uint64_t)sm_count(vg->device) * 2)),
                   256, 0, st>>>(d_src, d_dst, m_in, n, shift, sym ? 1 : 0, d->deg);
    k_deg_best<<<grid_for(n, vg->device), B_TPB, 0, st>>>(d->deg, n, best);
    EEG_CUDA(cudaGetLastError());
    unsigned long long hb = 0;
    EEG_CUDA(cudaMemcpyAsync(&hb, best, sizeof(hb), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    vg->max_deg = (uint32_t)(hb >> 32);
    vg->max_deg_vertex = hb ? 0xFFFFFFFFu - (uint32_t)(hb & 0xFFFFFFFFu) : 0u;
    d->P = 0;
    vg->bytes += sizeof(uint32_t) * (size_t)(n + 1);
    return EEG_OK;
}

// Build one direction. reverse: edges (s,t) are inserted as (t,s) -- the transposed graph.
// Edges are sorted by owner with a stable radix sort, so each vertex's edges keep the input order
// (the order the reference's MakeGraph gives them) and the layout is deterministic. With
// EEG_VG_SYMMETRIZE the vg->m arcs are the vg->m / 2 input edges followed by their reverses.
eeg_status build_direction(eeg_vgraph* vg, VDir* d, const uint32_t* d_src, const uint32_t* d_dst,
                           const uint32_t* d_w, bool reverse, cudaStream_t st) {
    const uint32_t n = vg->n, K = vg->K;
    const uint64_t m = vg->m;
    const bool sym = (vg->flags & EEG_VG_SYMMETRIZE) != 0;
    const uint64_t m_in = sym ? m / 2 : m;  // input edges
    const uint32_t shift = (vg->flags & EEG_VG_SHIFT_ONE) ? 1u : 0u;
    const uint32_t* a = reverse ? d_dst : d_src;
    const uint32_t* b = reverse ? d_src : d_dst;
    const bool with_w = (d_w != nullptr) || (!reverse && vg->weighted);
    const bool eid = (vg->flags & EEG_VG_EDGE_IDS) != 0;
    const bool payload = with_w || eid;  // the sort carries a third word: weight, or edge index

    EEG_TRY(vg_alloc(vg, (void**)&d->deg, sizeof(uint32_t) * (size_t)(n + 1)));
    EEG_TRY(vg_alloc(vg, (void**)&d->vstart, sizeof(uint32_t) * (size_t)(n + 1)));
    TempSet T(st);
    uint32_t *key[2] = {nullptr, nullptr}, *nb[2] = {nullptr, nullptr}, *wt[2] = {nullptr, nullptr};
    uint32_t *rs = nullptr, *re = nullptr, *np = nullptr, *tmp = nullptr, *err = nullptr, *hist = nullptr;
    for (int i = 0; i < 2; ++i) {
        EEG_TRY(T.get((void**)&key[i], sizeof(uint32_t) * m));
        EEG_TRY(T.get((void**)&nb[i], sizeof(uint32_t) * m));
        if (payload) EEG_TRY(T.get((void**)&wt[i], sizeof(uint32_t) * m));
    }
    EEG_TRY(T.get((void**)&rs, sizeof(uint32_t) * (size_t)(n + 1)));
    EEG_TRY(T.get((void**)&re, sizeof(uint32_t) * (size_t)(n + 1)));
    EEG_TRY(T.get((void**)&np, sizeof(uint32_t) * (size_t)(n + 1)));
    EEG_TRY(T.get((void**)&err, 16));
    unsigned long long* best = (unsigned long long*)(err + 2);
    const uint64_t ntiles = (m + R_TILE - 1) / R_TILE;
    const uint64_t hwords = std::max<uint64_t>(ntiles * R_BINS, 1);
    EEG_TRY(T.get((void**)&hist, sizeof(uint32_t) * hwords));
    EEG_TRY(T.get((void**)&tmp, sizeof(uint32_t) * device_scan_tmp_words(std::max<uint64_t>(hwords, (uint64_t)n + 1))));
    EEG_CUDA(cudaMemsetAsync(err, 0, 16, st));
    EEG_CUDA(cudaMemsetAsync(rs, 0, sizeof(uint32_t) * (size_t)(n + 1), st));
    EEG_CUDA(cudaMemsetAsync(re, 0, sizeof(uint32_t) * (size_t)(n + 1), st));

    int cur = 0;
    if (m > 0) {
        const uint32_t* wi = with_w ? d_w : nullptr;
        auto al16 = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
        if (al16(a) && al16(b) && al16(wi) && m_in >= 4 && (!sym || m_in % 4 == 0))
            k_prepare4<<<grid_for(m_in / 4, vg->device), B_TPB, 0, st>>>(
                reinterpret_cast<const uint4*>(a), reinterpret_cast<const uint4*>(b), reinterpret_cast<const uint4*>(wi),
                m_in, n, shift, reinterpret_cast<uint4*>(key[0]), reinterpret_cast<uint4*>(nb[0]),
                payload ? reinterpret_cast<uint4*>(wt[0]) : nullptr, err, eid ? 1 : 0, sym ? 1 : 0);
        else
            k_prepare<<<grid_for(m_in, vg->device), B_TPB, 0, st>>>(a, b, wi, m_in, n, shift, key[0], nb[0],
                                                                     payload ? wt[0] : nullptr, err, eid ? 1 : 0,
                                                                     sym ? 1 : 0);
        const uint32_t bits = n > 1 ? 32u - (uint32_t)__builtin_clz(n - 1) : 1u;
        for (uint32_t sh = 0; sh < bits; sh += 8) {
            k_radix_hist<<<(unsigned)ntiles, R_TPB, 0, st>>>(key[cur], m, sh, hist, (uint32_t)ntiles);
            EEG_TRY(device_scan_u32(hist, hist, ntiles * R_BINS, false, SCAN_ADD, tmp, st));
            k_radix_scatter<<<(unsigned)ntiles, R_TPB, 0, st>>>(key[cur], nb[cur], wt[cur], key[cur ^ 1], nb[cur ^ 1],
                                                                payload ? wt[cur ^ 1] : nullptr, m, sh, hist,
                                                                (uint32_t)ntiles);
            cur ^= 1;
        }
        k_runs<<<grid_for(m, vg->device), B_TPB, 0, st>>>(key[cur], m, rs, re);
    }
    k_nparts<<<grid_for((uint64_t)n + 1, vg->device), B_TPB, 0, st>>>(rs, re, n, K, d->deg, np, best);
    EEG_TRY(device_scan_u32(np, d->vstart, (uint64_t)n + 1, false, SCAN_ADD, tmp, st));

    uint32_t hbuf[4] = {0, 0, 0, 0};
    uint32_t P32 = 0;
    EEG_CUDA(cudaMemcpyAsync(hbuf, err, 16, cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaMemcpyAsync(&P32, d->vstart + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    if (hbuf[0]) {
        set_last_error("edge endpoint outside [0, num_nodes)");
        return EEG_ERR_INVALID;
    }
    if (!reverse) {
        unsigned long long kbest = ((unsigned long long)hbuf[3] << 32) | hbuf[2];
        vg->max_deg = (uint32_t)(kbest >> 32);
        vg->max_deg_vertex = kbest ? 0xFFFFFFFFu - (uint32_t)(kbest & 0xFFFFFFFFu) : 0u;
    }
    const uint64_t P = P32;
    d->P = P;
    const size_t slots = (size_t)P * K;
    EEG_TRY(vg_alloc(vg, (void**)&d->vowner, sizeof(uint32_t) * (size_t)std::max<uint64_t>(P, 1)));
    EEG_TRY(vg_alloc(vg, (void**)&d->vcol, sizeof(uint32_t) * std::max<size_t>(slots, 4)));
    if (with_w) EEG_TRY(vg_alloc(vg, (void**)&d->vw, sizeof(uint32_t) * std::max<size_t>(slots, 4)));
    if (eid) EEG_TRY(vg_alloc(vg, (void**)&d->veid, sizeof(uint32_t) * std::max<size_t>(slots, 4)));

    if (P > 0) {
        EEG_CUDA(cudaMemsetAsync(d->vowner, 0, sizeof(uint32_t) * (size_t)P, st));
        EEG_CUDA(cudaMemsetAsync(d->vcol, 0xFF, sizeof(uint32_t) * slots, st));
        if (d->vw) EEG_CUDA(cudaMemsetAsync(d->vw, 0, sizeof(uint32_t) * slots, st));
        if (d->veid) EEG_CUDA(cudaMemsetAsync(d->veid, 0xFF, sizeof(uint32_t) * slots, st));
        k_heads<<<grid_for(n, vg->device), B_TPB, 0, st>>>(d->vstart, n, d->vowner);
        uint32_t* tmp2 = nullptr;
        EEG_TRY(T.get((void**)&tmp2, sizeof(uint32_t) * (size_t)device_scan_tmp_words(P)));
        EEG_TRY(device_scan_u32(d->vowner, d->vowner, P, true, SCAN_MAX, tmp2, st));
        k_place<<<grid_for(m, vg->device), B_TPB, 0, st>>>(key[cur], nb[cur], payload ? wt[cur] : nullptr, m, K, rs,
                                                            d->vstart, d->vcol, d->vw, with_w ? d_w : nullptr,
                                                            d->veid, sym ? m_in : 0);
    }
    EEG_CUDA(cudaGetLastError());
    vg->bytes += sizeof(uint32_t) * ((size_t)(n + 1) * 2 + (size_t)P + slots * (1 + (with_w ? 1 : 0) + (eid ? 1 : 0)));
    return EEG_OK;
}

}  // namespace eeg
