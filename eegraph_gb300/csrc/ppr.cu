// ppr.cu -- differentiable personalised PageRank: forward solve, implicit adjoint solve and the
// edge / teleport gradients over the K-bounded virtual graph. A project-added form: the reference's
// PageRank (src/pr.cu:3-288) is unweighted, unpersonalised and has no adjoint.
//
// Model, per column, with row-normalised weights W_uv = w_uv / s_u (s_u = sum of u's out-weights):
//   forward  X = (1-d) T + d W^T X    -- pull over the transposed graph: x_v gathers rows X_u
//   adjoint  L = G + d W L            -- pull over the forward graph:   l_u gathers rows L_v
//   dLoss/dW_uv = d <X_u, L_v>,  dLoss/dw_uv = (dLoss/dW_uv - sum_v' dLoss/dW_uv' W_uv') / s_u,
//   dLoss/dT = (1-d) L.
// Neither solve needs atomics on values, a transpose at run time or stored iterates.
//
// Work decomposition (both directions, both forms): the part list is cut into chunks of <= 128 slots.
// A chunk holds whole vertices, except that a vertex with more than 128 slots (a hub) gets chunks of
// its own. Each hub chunk writes a partial; the last chunk of a group of 32 to arrive sums the group
// (compensated FP32, in chunk order) and the last group sums the groups. Deterministic, and a sweep
// needs one grid barrier (Jacobi, double-buffered iterates).
//   Batched rows (2..64 columns; rows padded to W = 32 or 64 FP32, 128 or 256 B): a warp owns a chunk and
//   splits into G = 128/W lane groups of W/4 lanes; group g takes slots g, g+G, ... of each part and
//   lane q of a group the float4 of columns 4q..4q+3, so one gather instruction moves G rows.
//   Single column (the plain form): a lane owns a slot; part sums by K-lane butterflies, vertex sums by
//   a segmented warp scan.
// Stop test: d/(1-d) * ||Y_{k+1}-Y_k||_1 <= tol * ||Y_{k+1}||_1 over all columns, reduced in FP64
// (FP32 per-chunk partials, FP64 per lane and across the grid); everything else is FP32.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.hpp"

namespace eeg {
namespace {

constexpr uint32_t PPR_SLOTS = 128;  // slots per work chunk
constexpr uint32_t PPR_GROUP = 32;   // hub chunks per first-level group
constexpr uint32_t PPR_W = 64;       // widest row of the batched form (FP32 columns)
constexpr int PPR_TPB = 256;
constexpr uint32_t NONE = 0xFFFFFFFFu;
constexpr unsigned FULL = 0xFFFFFFFFu;

struct Chunk {
    uint32_t p0, p1;  // parts [p0, p1)
    uint32_t hub;     // hub table index, or NONE
    uint32_t idx;     // index of this chunk within its hub
};
struct Hub {
    uint32_t v;       // vertex
    uint32_t first;   // first partial slot
    uint32_t count;   // chunks
    uint32_t gfirst;  // first group
};

// Device tables of one direction.
struct DirTab {
    const uint32_t* __restrict__ vowner;
    const uint32_t* __restrict__ vcol;
    const float* __restrict__ w;  // normalised weight of each slot
    const Chunk* __restrict__ chunk;
    uint32_t nchunks;
    const Hub* __restrict__ hub;
    uint32_t* garrive;  // arrivals per group (monotone over the sweeps of one launch)
    uint32_t* harrive;  // group completions per hub
    float* partial;     // hub chunk partials (slots x width)
    float* gpartial;    // group partials (groups x width)
};

struct SolveArgs {
    DirTab g;
    uint32_t n;
    const float* __restrict__ b;  // n x width source rows
    float scale_b;                // 1-d (forward) or 1 (adjoint)
    float d;
    float* y0;
    float* y1;
    PRCtrl* ctrl;
    uint32_t max_iters;
    double tol;
    uint64_t timeout_ns;
};

struct GradArgs {
    DirTab g;               // forward direction
    const float* __restrict__ X;
    const float* __restrict__ L;
    float d;
    float* gslot;           // dLoss/dW per forward slot
    float* r;               // sum_v dLoss/dW_uv W_uv per vertex
    uint32_t accumulate;
};

// ------------------------------------------------------------------ small helpers
__device__ __forceinline__ float4 f4(float v) { return make_float4(v, v, v, v); }
__device__ __forceinline__ void fma4(float4& acc, float w, const float4& x) {
    acc.x = fmaf(w, x.x, acc.x);
    acc.y = fmaf(w, x.y, acc.y);
    acc.z = fmaf(w, x.z, acc.z);
    acc.w = fmaf(w, x.w, acc.w);
}
__device__ __forceinline__ float4 shfl_xor4(const float4& v, int o) {
    return make_float4(__shfl_xor_sync(FULL, v.x, o), __shfl_xor_sync(FULL, v.y, o), __shfl_xor_sync(FULL, v.z, o),
                       __shfl_xor_sync(FULL, v.w, o));
}
__device__ __forceinline__ float4 add4(const float4& a, const float4& b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 affine4(float d, const float4& acc, float sb, const float4& b) {
    return make_float4(fmaf(d, acc.x, sb * b.x), fmaf(d, acc.y, sb * b.y), fmaf(d, acc.z, sb * b.z),
                       fmaf(d, acc.w, sb * b.w));
}
__device__ __forceinline__ float l1diff4(const float4& a, const float4& b) {
    return fabsf(a.x - b.x) + fabsf(a.y - b.y) + fabsf(a.z - b.z) + fabsf(a.w - b.w);
}
__device__ __forceinline__ float l14(const float4& a) { return fabsf(a.x) + fabsf(a.y) + fabsf(a.z) + fabsf(a.w); }
__device__ __forceinline__ float dot4(const float4& a, const float4& b) {
    return fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, a.w * b.w)));
}
__device__ __forceinline__ uint32_t ld_nc(const uint32_t* p) { return __ldg(p); }

// Element j (run-time index) of a register array without local-memory indexing.
template <int N, typename T>
__device__ __forceinline__ T pick(const T (&a)[N], uint32_t j) {
    T r = a[0];
#pragma unroll
    for (int i = 1; i < N; ++i)
        if ((uint32_t)i == j) r = a[i];
    return r;
}

// Lane-group transpose reduction: each lane holds N values (one per slot of its group of NQ lanes);
// afterwards lane q holds the sum over the group's lanes of value index(q) (see red_index). log2(N)
// halving steps, then plain butterflies.
template <int N, int NQ>
__device__ __forceinline__ float tred(float (&v)[N], uint32_t q) {
    int n = N;
#pragma unroll
    for (int o = NQ / 2; o >= 1; o >>= 1) {
        if (n >= 2) {
            const bool up = (q & (uint32_t)o) != 0;
#pragma unroll
            for (int i = 0; i < N / 2; ++i) {
                if (i < n / 2) {
                    const float send = up ? v[i] : v[i + n / 2];
                    const float keep = up ? v[i + n / 2] : v[i];
                    v[i] = keep + __shfl_xor_sync(FULL, send, o);
                }
            }
            n >>= 1;
        } else {
            v[0] += __shfl_xor_sync(FULL, v[0], o);
        }
    }
    return v[0];
}
template <int N, int NQ>
__device__ __forceinline__ uint32_t red_index(uint32_t q) {
    uint32_t i = 0;
    int n = N;
#pragma unroll
    for (int o = NQ / 2; o >= 1; o >>= 1) {
        if (n >= 2) {
            if (q & (uint32_t)o) i += (uint32_t)(n / 2);
            n >>= 1;
        }
    }
    return i;
}

// Sum of a float4 over the warp's lane groups (lanes q, q+NQ, ...); every lane gets its q's total.
template <int NQ>
__device__ __forceinline__ float4 across_groups(float4 v) {
#pragma unroll
    for (int o = NQ; o < 32; o <<= 1) v = add4(v, shfl_xor4(v, o));
    return v;
}

// Compensated sum of partial rows [first, first+cnt) (NQ float4 each); lane groups take rows in turn;
// every lane of the warp returns the same float4 for its q.
template <int NQ>
__device__ float4 sum_rows(const float4* base, uint32_t first, uint32_t cnt, uint32_t grp, uint32_t q) {
    constexpr uint32_t G = 32 / NQ;
    float4 hi = f4(0.f), lo = f4(0.f);
    for (uint32_t i = grp; i < cnt; i += G) {
        const float4 p = __ldcg(base + (size_t)(first + i) * NQ + q);
        pair_add(hi.x, lo.x, p.x, 0.f);
        pair_add(hi.y, lo.y, p.y, 0.f);
        pair_add(hi.z, lo.z, p.z, 0.f);
        pair_add(hi.w, lo.w, p.w, 0.f);
    }
#pragma unroll
    for (int o = NQ; o < 32; o <<= 1) {
        const float4 ho = shfl_xor4(hi, o), lo2 = shfl_xor4(lo, o);
        pair_add(hi.x, lo.x, ho.x, lo2.x);
        pair_add(hi.y, lo.y, ho.y, lo2.y);
        pair_add(hi.z, lo.z, ho.z, lo2.z);
        pair_add(hi.w, lo.w, ho.w, lo2.w);
    }
    return hi;
}

// Slot j*G + grp of a part row (grp run-time, the array index compile-time: no local memory).
template <int G, int K>
__device__ __forceinline__ uint32_t group_slot(const uint32_t (&row)[K], int j, uint32_t grp) {
    uint32_t r = row[j * G];
#pragma unroll
    for (int g = 1; g < G; ++g)
        if (grp == (uint32_t)g) r = row[j * G + g];
    return r;
}

// Rows gathered per lane per step: 8, so U = 8/H parts per step (16/K at W = 64, 32/K at W = 32).
template <int K, int G>
struct RowStep {
    static constexpr int H = K / G;  // slots of a part per lane group
    static constexpr int U = 8 / H;  // parts per step
};

// Neighbour ids and weights of this lane group's slots (j*G + grp) of parts pp .. pp+U-1 of a chunk
// (NONE and 0 past its np parts). Two groups (W = 64): whole rows by 256-bit loads, then a selection;
// more groups: the group's slots one by one (the whole rows would take 2*U*K registers).
template <int K, int G>
__device__ __forceinline__ void load_group_slots(const DirTab& g, uint32_t p0, uint32_t pp, uint32_t np, uint32_t grp,
                                                 uint64_t pol, uint32_t (&colg)[RowStep<K, G>::U][K / G],
                                                 uint32_t (&wbg)[RowStep<K, G>::U][K / G]) {
    constexpr int U = RowStep<K, G>::U, H = K / G;
    if constexpr (G <= 2) {
        uint32_t col[U][K], wb[U][K];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (pp + u < np) {
                const size_t row = (size_t)(p0 + pp + u) * K;
                ld_part<K>(g.vcol + row, col[u], pol);
                ld_part<K>(reinterpret_cast<const uint32_t*>(g.w) + row, wb[u], pol);
            } else {
#pragma unroll
                for (int j = 0; j < K; ++j) {
                    col[u][j] = NONE;
                    wb[u][j] = 0u;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int j = 0; j < H; ++j) {
                colg[u][j] = group_slot<G>(col[u], j, grp);
                wbg[u][j] = group_slot<G>(wb[u], j, grp);
            }
    } else {
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int j = 0; j < H; ++j) {
                colg[u][j] = NONE;
                wbg[u][j] = 0u;
                if (pp + u < np) {
                    const size_t at = (size_t)(p0 + pp + u) * K + (size_t)(j * G) + grp;
                    colg[u][j] = ld_nc(g.vcol + at);
                    wbg[u][j] = __float_as_uint(__ldg(g.w + at));
                }
            }
    }
}
// Compensated sum of scalar partials [first, first+cnt); all lanes return the same value.
__device__ float sum_scalars(const float* base, uint32_t first, uint32_t cnt, uint32_t lane) {
    float hi = 0.f, lo = 0.f;
    for (uint32_t i = lane; i < cnt; i += 32) pair_add(hi, lo, __ldcg(base + first + i), 0.f);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const float h2 = __shfl_xor_sync(FULL, hi, o), l2 = __shfl_xor_sync(FULL, lo, o);
        pair_add(hi, lo, h2, l2);
    }
    return hi;
}

// Arrival at a counter; true in the warp that completes `target` arrivals. Warp-collective.
__device__ __forceinline__ bool arrive_last(uint32_t* ctr, uint32_t target, uint32_t lane) {
    uint32_t last = 0;
    if (lane == 0) {
        __threadfence();
        last = (atomicAdd(ctr, 1u) + 1u == target) ? 1u : 0u;
    }
    last = __shfl_sync(FULL, last, 0);
    if (last) __threadfence();
    return last != 0;
}

// Next chunk of this CTA's strided share of the chunk list (blockIdx.x + i * gridDim.x: CTAs get
// similar mixes of hub and leaf chunks), drawn by its warps through a shared counter so that no warp
// idles while another of the CTA still has chunks queued. NONE when the share is used up. Warp-collective.
__device__ __forceinline__ uint32_t next_chunk(uint32_t* ctr, uint32_t nchunks, uint32_t lane) {
    uint32_t i = 0;
    if (lane == 0) i = atomicAdd(ctr, 1u);
    i = __shfl_sync(FULL, i, 0);
    const uint64_t c = blockIdx.x + (uint64_t)i * gridDim.x;
    return c < nchunks ? (uint32_t)c : NONE;
}

// Hub chunk delivery, batched rows. `tot` is the chunk's row (same in every lane group). Returns true
// in the warp that completes the hub for this sweep (`mult` = sweeps completed including this one), with
// the hub's full row in `out` and its vertex in `v`. Warp-collective.
template <int NQ>
__device__ bool hub_rows(const DirTab& g, const Chunk& ch, const float4& tot, uint32_t mult, uint32_t lane,
                         float4& out, uint32_t& v) {
    const uint32_t grp = lane / NQ, q = lane % NQ;
    const Hub H = g.hub[ch.hub];
    float4* part = reinterpret_cast<float4*>(g.partial);
    float4* gpart = reinterpret_cast<float4*>(g.gpartial);
    if (grp == 0) {
        part[(size_t)(H.first + ch.idx) * NQ + q] = tot;
        __threadfence();
    }
    __syncwarp();
    const uint32_t gi = ch.idx / PPR_GROUP, g0 = gi * PPR_GROUP;
    const uint32_t gs = min(PPR_GROUP, H.count - g0);
    if (!arrive_last(&g.garrive[H.gfirst + gi], mult * gs, lane)) return false;
    const float4 s1 = sum_rows<NQ>(part, H.first + g0, gs, grp, q);
    const uint32_t ng = (H.count + PPR_GROUP - 1) / PPR_GROUP;
    v = H.v;
    if (ng == 1) {
        out = s1;
        return true;
    }
    if (grp == 0) {
        gpart[(size_t)(H.gfirst + gi) * NQ + q] = s1;
        __threadfence();
    }
    __syncwarp();
    if (!arrive_last(&g.harrive[ch.hub], mult * ng, lane)) return false;
    out = sum_rows<NQ>(gpart, H.gfirst, ng, grp, q);
    return true;
}
// Same for one scalar per chunk.
__device__ bool hub_scalar(const DirTab& g, const Chunk& ch, float tot, uint32_t mult, uint32_t lane, float& out,
                           uint32_t& v) {
    const Hub H = g.hub[ch.hub];
    if (lane == 0) {
        g.partial[H.first + ch.idx] = tot;
        __threadfence();
    }
    __syncwarp();
    const uint32_t gi = ch.idx / PPR_GROUP, g0 = gi * PPR_GROUP;
    const uint32_t gs = min(PPR_GROUP, H.count - g0);
    if (!arrive_last(&g.garrive[H.gfirst + gi], mult * gs, lane)) return false;
    const float s1 = sum_scalars(g.partial, H.first + g0, gs, lane);
    const uint32_t ng = (H.count + PPR_GROUP - 1) / PPR_GROUP;
    v = H.v;
    if (ng == 1) {
        out = s1;
        return true;
    }
    if (lane == 0) {
        g.gpartial[H.gfirst + gi] = s1;
        __threadfence();
    }
    __syncwarp();
    if (!arrive_last(&g.harrive[ch.hub], mult * ng, lane)) return false;
    out = sum_scalars(g.gpartial, H.gfirst, ng, lane);
    return true;
}

// End of a sweep: reduce the residual / norm, barrier, stop test. Returns 0 = continue, 1 = converged,
// 2 = grid aborting.
__device__ __forceinline__ int end_sweep(const SolveArgs& a, uint32_t s, double dr, double dn, uint32_t& epoch) {
    PRCtrl* ctrl = a.ctrl;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        dr += __shfl_down_sync(FULL, dr, off);
        dn += __shfl_down_sync(FULL, dn, off);
    }
    if ((threadIdx.x & 31u) == 0 && (dr != 0.0 || dn != 0.0)) {
        atomicAdd(&ctrl->resid[s % 3], dr);
        atomicAdd(&ctrl->norm[s % 3], dn);
    }
    if (!grid_barrier(&ctrl->bw, epoch, a.timeout_ns)) return 2;
    __shared__ double s_rn[2];  // one read per CTA instead of one per warp
    if (threadIdx.x == 0) {
        s_rn[0] = __ldcg(&ctrl->resid[s % 3]);
        s_rn[1] = __ldcg(&ctrl->norm[s % 3]);
    }
    __syncthreads();
    const double resid = s_rn[0], norm = s_rn[1];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // slot (s+2)%3 was last read before barrier s and is next accumulated after barrier s+1
        ctrl->resid[(s + 2) % 3] = 0.0;
        ctrl->norm[(s + 2) % 3] = 0.0;
        ctrl->last_resid = resid;
        ctrl->last_norm = norm;
    }
    return ((double)a.d / (1.0 - (double)a.d) * resid <= a.tol * norm) ? 1 : 0;
}

// ------------------------------------------------------------------ batched rows: solve
template <int NQ>
__device__ __forceinline__ void flush_row(const SolveArgs& a, float4* out, uint32_t v, float4 acc, const float4& bv,
                                          const float4& ov, uint32_t grp, uint32_t q, float& rr, float& nn) {
    acc = across_groups<NQ>(acc);
    const float4 y = affine4(a.d, acc, a.scale_b, bv);
    if (grp == 0) {
        out[(size_t)v * NQ + q] = y;
        rr += l1diff4(y, ov);
        nn += l14(y);
    }
}

// 3 CTAs per SM (<= 85 registers, a few spilled): the solve is latency-bound, and 24 warps per SM
// instead of 16 measured 1.3x faster on R-MAT s20 x 64 columns. NQ = W/4 lanes per row.
template <int K, int NQ>
__global__ void __launch_bounds__(PPR_TPB, 3) k_ppr_rows(SolveArgs a) {
    constexpr int G = 32 / NQ;               // lane groups (rows per gather instruction)
    constexpr int H = K / G;                 // slots per group per part
    constexpr int U = RowStep<K, G>::U;      // parts per step: 8 row gathers in flight per lane
    static_assert(H >= 1 && H <= 8, "K must be at least the number of lane groups");
    const uint32_t lane = threadIdx.x & 31u, grp = lane / NQ, q = lane % NQ;
    __shared__ uint32_t s_next[2];  // per sweep (alternating): next of this CTA's chunks
    if (threadIdx.x == 0) s_next[0] = s_next[1] = 0u;
    __syncthreads();
    const uint64_t pol = l2_evict_first_policy();
    const float4* b = reinterpret_cast<const float4*>(a.b);
    uint32_t epoch = 0, s = 0;
    bool conv = false;
    {
        float4* y0 = reinterpret_cast<float4*>(a.y0);
        float4* y1 = reinterpret_cast<float4*>(a.y1);
        const uint64_t tot = (uint64_t)a.n * NQ;
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot;
             i += (uint64_t)gridDim.x * blockDim.x) {
            const float4 v = b[i];
            const float4 y = make_float4(a.scale_b * v.x, a.scale_b * v.y, a.scale_b * v.z, a.scale_b * v.w);
            y0[i] = y;
            y1[i] = y;
        }
    }
    if (!grid_barrier(&a.ctrl->bw, epoch, a.timeout_ns)) goto finish;
    for (; s < a.max_iters; ++s) {
        const float4* in = reinterpret_cast<const float4*>((s & 1u) ? a.y1 : a.y0);
        float4* out = reinterpret_cast<float4*>((s & 1u) ? a.y0 : a.y1);
        double dr = 0.0, dn = 0.0;
        if (threadIdx.x == 0) s_next[(s + 1u) & 1u] = 0u;  // next sweep's; ordered by the sweep's grid barrier
        for (uint32_t c; (c = next_chunk(&s_next[s & 1u], a.g.nchunks, lane)) != NONE;) {
            const Chunk ch = a.g.chunk[c];
            const uint32_t np = ch.p1 - ch.p0;
            const uint32_t own_l = lane < np ? ld_nc(a.g.vowner + ch.p0 + lane) : NONE;
            uint32_t cur = __shfl_sync(FULL, own_l, 0);
            float4 bv = b[(size_t)cur * NQ + q];
            float4 ov = in[(size_t)cur * NQ + q];
            float4 acc = f4(0.f);
            float rr = 0.f, nn = 0.f;
            for (uint32_t pp = 0; pp < np; pp += U) {
                uint32_t colg[U][H], wbg[U][H];
                load_group_slots<K, G>(a.g, ch.p0, pp, np, grp, pol, colg, wbg);
                float4 xv[U][H];
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int j = 0; j < H; ++j) {
                        const uint32_t id = colg[u][j];
                        xv[u][j] = id != NONE ? in[(size_t)id * NQ + q] : f4(0.f);
                    }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (pp + u < np) {
                        const uint32_t o = __shfl_sync(FULL, own_l, pp + u);
                        if (o != cur) {
                            flush_row<NQ>(a, out, cur, acc, bv, ov, grp, q, rr, nn);
                            acc = f4(0.f);
                            cur = o;
                            bv = b[(size_t)cur * NQ + q];
                            ov = in[(size_t)cur * NQ + q];
                        }
#pragma unroll
                        for (int j = 0; j < H; ++j) fma4(acc, __uint_as_float(wbg[u][j]), xv[u][j]);
                    }
                }
            }
            if (ch.hub == NONE) {
                flush_row<NQ>(a, out, cur, acc, bv, ov, grp, q, rr, nn);
            } else {
                const float4 tot = across_groups<NQ>(acc);
                float4 full;
                uint32_t v;
                if (hub_rows<NQ>(a.g, ch, tot, s + 1, lane, full, v)) {
                    const float4 y = affine4(a.d, full, a.scale_b, b[(size_t)v * NQ + q]);
                    if (grp == 0) {
                        const float4 o = in[(size_t)v * NQ + q];
                        out[(size_t)v * NQ + q] = y;
                        rr += l1diff4(y, o);
                        nn += l14(y);
                    }
                }
            }
            dr += (double)rr;
            dn += (double)nn;
        }
        const int st = end_sweep(a, s, dr, dn, epoch);
        if (st == 2) goto finish;
        if (st == 1) {
            ++s;
            conv = true;
            break;
        }
    }
    if (!conv && blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&a.ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_ITER_CAP);
finish:
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctrl->iterations = s;
}

// ------------------------------------------------------------------ single column: solve
template <int K>
__global__ void __launch_bounds__(PPR_TPB, 4) k_ppr_scalar(SolveArgs a) {
    constexpr int PPS = 32 / K;                   // parts per 32-slot step
    constexpr int STEPS = (int)PPR_SLOTS / 32;    // steps per chunk
    const uint32_t lane = threadIdx.x & 31u;
    __shared__ uint32_t s_next[2];  // per sweep (alternating): next of this CTA's chunks
    if (threadIdx.x == 0) s_next[0] = s_next[1] = 0u;
    __syncthreads();
    const float* b = a.b;
    uint32_t epoch = 0, s = 0;
    bool conv = false;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float y = a.scale_b * b[i];
        a.y0[i] = y;
        a.y1[i] = y;
    }
    if (!grid_barrier(&a.ctrl->bw, epoch, a.timeout_ns)) goto finish;
    for (; s < a.max_iters; ++s) {
        const float* in = (s & 1u) ? a.y1 : a.y0;
        float* out = (s & 1u) ? a.y0 : a.y1;
        double dr = 0.0, dn = 0.0;
        if (threadIdx.x == 0) s_next[(s + 1u) & 1u] = 0u;  // next sweep's; ordered by the sweep's grid barrier
        for (uint32_t c; (c = next_chunk(&s_next[s & 1u], a.g.nchunks, lane)) != NONE;) {
            const Chunk ch = a.g.chunk[c];
            const uint32_t np = ch.p1 - ch.p0;
            const uint32_t nsl = np * K;
            const size_t base = (size_t)ch.p0 * K;
            const uint32_t own_l = lane < np ? ld_nc(a.g.vowner + ch.p0 + lane) : NONE;
            uint32_t col[STEPS];
            float wv[STEPS], xv[STEPS];
#pragma unroll
            for (int st = 0; st < STEPS; ++st) {
                const uint32_t idx = (uint32_t)st * 32u + lane;
                col[st] = idx < nsl ? ld_nc(a.g.vcol + base + idx) : NONE;
                wv[st] = idx < nsl ? __ldg(a.g.w + base + idx) : 0.f;
            }
#pragma unroll
            for (int st = 0; st < STEPS; ++st) xv[st] = col[st] != NONE ? in[col[st]] : 0.f;
            float psum = 0.f;
#pragma unroll
            for (int st = 0; st < STEPS; ++st) {
                if ((uint32_t)st * 32u < nsl) {
                    float v = wv[st] * xv[st];
#pragma unroll
                    for (int o = K / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
#pragma unroll
                    for (int i = 0; i < PPS; ++i) {
                        const float t = __shfl_sync(FULL, v, i * K);
                        if (lane == (uint32_t)(st * PPS + i)) psum = t;
                    }
                }
            }
            // vertex sums: segmented inclusive scan over the part lanes
            const uint32_t prev = __shfl_up_sync(FULL, own_l, 1);
            const bool head = lane == 0 || own_l != prev;
            const uint32_t hm = __ballot_sync(FULL, head);
            const uint32_t start = 31u - __clz(hm & (((lane == 31u) ? 0u : (2u << lane)) - 1u));
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float t = __shfl_up_sync(FULL, psum, o);
                if (lane >= (uint32_t)o && lane - (uint32_t)o >= start) psum += t;
            }
            float rr = 0.f, nn = 0.f;
            if (ch.hub == NONE) {
                const uint32_t next = __shfl_down_sync(FULL, own_l, 1);
                const bool lastl = lane < np && (lane == np - 1 || next != own_l);
                if (lastl) {
                    const float y = fmaf(a.d, psum, a.scale_b * b[own_l]);
                    rr += fabsf(y - in[own_l]);
                    nn += fabsf(y);
                    out[own_l] = y;
                }
            } else {
                const float tot = __shfl_sync(FULL, psum, np - 1);
                float full;
                uint32_t v;
                if (hub_scalar(a.g, ch, tot, s + 1, lane, full, v) && lane == 0) {
                    const float y = fmaf(a.d, full, a.scale_b * b[v]);
                    rr += fabsf(y - in[v]);
                    nn += fabsf(y);
                    out[v] = y;
                }
            }
            dr += (double)rr;
            dn += (double)nn;
        }
        const int st = end_sweep(a, s, dr, dn, epoch);
        if (st == 2) goto finish;
        if (st == 1) {
            ++s;
            conv = true;
            break;
        }
    }
    if (!conv && blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&a.ctrl->bw.status, (uint32_t)DEV_OK, (uint32_t)DEV_ITER_CAP);
finish:
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctrl->iterations = s;
}

// ------------------------------------------------------------------ gradients
// Batched rows: g_uv = d <X_u, L_v> per forward slot; r_u = sum_v g_uv W_uv per vertex.
template <int K, int NQ>
__global__ void __launch_bounds__(PPR_TPB, 2) k_ppr_grad_rows(GradArgs a) {
    constexpr int G = 32 / NQ;
    constexpr int H = K / G;
    constexpr int U = RowStep<K, G>::U;
    static_assert(H >= 1 && H <= NQ, "K must be at least the number of lane groups");
    const uint32_t lane = threadIdx.x & 31u, grp = lane / NQ, q = lane % NQ;
    __shared__ uint32_t s_next[2];  // per sweep (alternating): next of this CTA's chunks
    if (threadIdx.x == 0) s_next[0] = s_next[1] = 0u;
    __syncthreads();
    const uint64_t pol = l2_evict_first_policy();
    const float4* X = reinterpret_cast<const float4*>(a.X);
    const float4* L = reinterpret_cast<const float4*>(a.L);
    const uint32_t ri = red_index<H, NQ>(q);
    const uint32_t jme = (uint32_t)G * ri + grp;               // slot this lane reports after the reduction
    const bool writer = (q & (uint32_t)(NQ / H - 1)) == 0u;    // one lane per reduced value
    for (uint32_t c; (c = next_chunk(&s_next[0], a.g.nchunks, lane)) != NONE;) {
        const Chunk ch = a.g.chunk[c];
        const uint32_t np = ch.p1 - ch.p0;
        const uint32_t own_l = lane < np ? ld_nc(a.g.vowner + ch.p0 + lane) : NONE;
        uint32_t cur = __shfl_sync(FULL, own_l, 0);
        float4 xu = X[(size_t)cur * NQ + q];
        float racc = 0.f;
        for (uint32_t pp = 0; pp < np; pp += U) {
            uint32_t colg[U][H], wbg[U][H];
            load_group_slots<K, G>(a.g, ch.p0, pp, np, grp, pol, colg, wbg);
            float4 lv[U][H];
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int j = 0; j < H; ++j) {
                    const uint32_t id = colg[u][j];
                    lv[u][j] = id != NONE ? L[(size_t)id * NQ + q] : f4(0.f);
                }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (pp + u < np) {
                    const uint32_t o = __shfl_sync(FULL, own_l, pp + u);
                    if (o != cur) {
                        float t = racc;
#pragma unroll
                        for (int off = 16; off >= 1; off >>= 1) t += __shfl_xor_sync(FULL, t, off);
                        if (lane == 0) a.r[cur] = a.accumulate ? a.r[cur] + t : t;
                        racc = 0.f;
                        cur = o;
                        xu = X[(size_t)cur * NQ + q];
                    }
                    float dv[H];
#pragma unroll
                    for (int j = 0; j < H; ++j) dv[j] = dot4(xu, lv[u][j]);
                    const float dsum = tred<H, NQ>(dv, q);
                    const uint32_t id = pick<H>(colg[u], ri);  // slot jme of the part
                    if (writer && id != NONE) {
                        const float g = a.d * dsum;
                        const size_t slot = (size_t)(ch.p0 + pp + u) * K + jme;
                        a.gslot[slot] = a.accumulate ? a.gslot[slot] + g : g;
                        racc = fmaf(g, __uint_as_float(pick<H>(wbg[u], ri)), racc);
                    }
                }
            }
        }
        float t = racc;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) t += __shfl_xor_sync(FULL, t, off);
        if (ch.hub == NONE) {
            if (lane == 0) a.r[cur] = a.accumulate ? a.r[cur] + t : t;
        } else {
            float full;
            uint32_t v;
            if (hub_scalar(a.g, ch, t, 1u, lane, full, v) && lane == 0) a.r[v] = a.accumulate ? a.r[v] + full : full;
        }
    }
}

// Single column: the same per slot, X and L scalars.
template <int K>
__global__ void __launch_bounds__(PPR_TPB, 4) k_ppr_grad_scalar(GradArgs a) {
    constexpr int PPS = 32 / K;
    constexpr int STEPS = (int)PPR_SLOTS / 32;
    const uint32_t lane = threadIdx.x & 31u;
    __shared__ uint32_t s_next[2];  // per sweep (alternating): next of this CTA's chunks
    if (threadIdx.x == 0) s_next[0] = s_next[1] = 0u;
    __syncthreads();
    for (uint32_t c; (c = next_chunk(&s_next[0], a.g.nchunks, lane)) != NONE;) {
        const Chunk ch = a.g.chunk[c];
        const uint32_t np = ch.p1 - ch.p0;
        const uint32_t nsl = np * K;
        const size_t base = (size_t)ch.p0 * K;
        const uint32_t own_l = lane < np ? ld_nc(a.g.vowner + ch.p0 + lane) : NONE;
        uint32_t col[STEPS];
        float wv[STEPS], gv[STEPS];
#pragma unroll
        for (int st = 0; st < STEPS; ++st) {
            const uint32_t idx = (uint32_t)st * 32u + lane;
            col[st] = idx < nsl ? ld_nc(a.g.vcol + base + idx) : NONE;
            wv[st] = idx < nsl ? __ldg(a.g.w + base + idx) : 0.f;
        }
#pragma unroll
        for (int st = 0; st < STEPS; ++st) {
            const uint32_t o = __shfl_sync(FULL, own_l, st * PPS + (int)(lane / K));
            gv[st] = 0.f;
            if (col[st] != NONE) {
                gv[st] = a.d * (a.X[o] * a.L[col[st]]);
                const size_t slot = base + (uint32_t)st * 32u + lane;
                a.gslot[slot] = a.accumulate ? a.gslot[slot] + gv[st] : gv[st];
            }
        }
        float psum = 0.f;
#pragma unroll
        for (int st = 0; st < STEPS; ++st) {
            if ((uint32_t)st * 32u < nsl) {
                float v = gv[st] * wv[st];
#pragma unroll
                for (int o = K / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
#pragma unroll
                for (int i = 0; i < PPS; ++i) {
                    const float t = __shfl_sync(FULL, v, i * K);
                    if (lane == (uint32_t)(st * PPS + i)) psum = t;
                }
            }
        }
        const uint32_t prev = __shfl_up_sync(FULL, own_l, 1);
        const bool head = lane == 0 || own_l != prev;
        const uint32_t hm = __ballot_sync(FULL, head);
        const uint32_t start = 31u - __clz(hm & (((lane == 31u) ? 0u : (2u << lane)) - 1u));
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float t = __shfl_up_sync(FULL, psum, o);
            if (lane >= (uint32_t)o && lane - (uint32_t)o >= start) psum += t;
        }
        if (ch.hub == NONE) {
            const uint32_t next = __shfl_down_sync(FULL, own_l, 1);
            if (lane < np && (lane == np - 1 || next != own_l))
                a.r[own_l] = a.accumulate ? a.r[own_l] + psum : psum;
        } else {
            const float tot = __shfl_sync(FULL, psum, np - 1);
            float full;
            uint32_t v;
            if (hub_scalar(a.g, ch, tot, 1u, lane, full, v) && lane == 0) a.r[v] = a.accumulate ? a.r[v] + full : full;
        }
    }
}

// Per-edge outputs in input edge order.
__global__ void k_ppr_scatter(uint64_t nslots, uint32_t K, const uint32_t* __restrict__ veid,
                              const uint32_t* __restrict__ vowner, const float* __restrict__ gslot,
                              const float* __restrict__ r, const float* __restrict__ s, float* dwn, float* dw) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = veid[i];
        if (e == NONE) continue;
        const float g = gslot[i];
        if (dwn) dwn[e] = g;
        if (dw) {
            const uint32_t u = vowner[i / K];
            const float su = s[u];
            dw[e] = su > 0.f ? (g - r[u]) / su : 0.f;
        }
    }
}

// out = (1-d) L  (dLoss/dT)
__global__ void k_ppr_scale(uint64_t count, float f, const float* __restrict__ in, float* __restrict__ out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = f * in[i];
}

// ------------------------------------------------------------------ weights
// s_u = sum of u's raw out-weights (warp per vertex, fixed order); flags negative / non-finite weights.
__global__ void k_ppr_out_sums(uint32_t n, uint32_t K, const uint32_t* __restrict__ vstart,
                               const uint32_t* __restrict__ veid, const float* __restrict__ w, float* __restrict__ s,
                               uint32_t* bad) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t v = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += nw) {
        const size_t a0 = (size_t)vstart[v] * K, a1 = (size_t)vstart[v + 1] * K;
        float acc = 0.f;
        uint32_t b = 0;
        for (size_t i = a0 + lane; i < a1; i += 32) {
            const uint32_t e = veid[i];
            if (e != NONE) {
                const float x = w[e];
                if (!(x >= 0.f) || !isfinite(x)) b = 1;
                acc += x;
            }
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
        if (__any_sync(FULL, b) && lane == 0) atomicOr(bad, 1u);
        if (lane == 0) s[v] = acc;
    }
}
// Normalised weight per slot. Forward: the slot's source is the part owner; transposed: the slot's
// neighbour.
__global__ void k_ppr_norm(uint64_t nslots, uint32_t K, int transposed, const uint32_t* __restrict__ veid,
                           const uint32_t* __restrict__ vowner, const uint32_t* __restrict__ vcol,
                           const float* __restrict__ w, const float* __restrict__ s, float* __restrict__ wn) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = veid[i];
        float r = 0.f;
        if (e != NONE) {
            const uint32_t u = transposed ? vcol[i] : vowner[i / K];
            const float su = s[u];
            r = su > 0.f ? w[e] / su : 0.f;
        }
        wn[i] = r;
    }
}

unsigned grid_1d(uint64_t work, int device) {
    const uint64_t cap = (uint64_t)sm_count(device) * 8;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((work + PPR_TPB - 1) / PPR_TPB, cap));
}

}  // namespace

// Host-held device tables of one direction.
struct PPRDir {
    Chunk* chunk = nullptr;
    uint32_t nchunks = 0;
    Hub* hub = nullptr;
    uint32_t nhubs = 0, nslots = 0, ngroups = 0;
    uint32_t* garrive = nullptr;
    uint32_t* harrive = nullptr;
    float* partial = nullptr;
    float* gpartial = nullptr;
    float* w = nullptr;  // normalised weight per slot
};

}  // namespace eeg

struct eeg_ppr {
    eeg_vgraph* vg = nullptr;
    uint32_t C = 1, W = 1;
    eeg::PPRDir fwd, rev;
    float* w_raw = nullptr;  // m
    float* s = nullptr;      // n
    uint32_t* bad = nullptr;
    float* Y[2] = {nullptr, nullptr};  // forward iterates
    float* Lb[2] = {nullptr, nullptr}; // adjoint iterates
    float* b = nullptr;                // staged input rows (n x W)
    float* gslot = nullptr;            // forward slots
    float* r = nullptr;                // n
    float* stage_m = nullptr;          // 2m: host-bound edge outputs
    float* stage_nw = nullptr;         // n x W: host-bound / repacked row outputs
    eeg::PRCtrl* ctrl = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int xi = -1;  // Y buffer holding X after the last forward
    bool have_w = false, have_g = false;
    uint64_t bytes = 0;
};

namespace eeg {
namespace {

eeg_status ppr_alloc(eeg_ppr* p, void** ptr, size_t bytes) {
    EEG_TRY(vg_alloc(p->vg, ptr, bytes));
    p->bytes += bytes;
    return EEG_OK;
}

void free_pdir(eeg_ppr* p, PPRDir& d) {
    vg_free(p->vg, d.chunk);
    vg_free(p->vg, d.hub);
    vg_free(p->vg, d.garrive);
    vg_free(p->vg, d.harrive);
    vg_free(p->vg, d.partial);
    vg_free(p->vg, d.gpartial);
    vg_free(p->vg, d.w);
    d = PPRDir{};
}

// Cut one direction's parts into chunks (host; from vstart).
eeg_status build_chunks(eeg_ppr* p, const VDir& vd, PPRDir& d) {
    eeg_vgraph* vg = p->vg;
    const uint32_t n = vg->n, K = vg->K;
    const uint32_t CH = PPR_SLOTS / K;
    std::vector<uint32_t> vs((size_t)n + 1);
    EEG_CUDA(cudaMemcpy(vs.data(), vd.vstart, sizeof(uint32_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost));
    std::vector<Chunk> ch;
    std::vector<Hub> hubs;
    ch.reserve((size_t)(vd.P / CH) + 16);
    uint32_t slots = 0, groups = 0;
    uint32_t v = 0;
    while (v < n) {
        const uint32_t np = vs[v + 1] - vs[v];
        if (np == 0) {
            ++v;
            continue;
        }
        if (np > CH) {
            const uint32_t count = (np + CH - 1) / CH;
            const uint32_t h = (uint32_t)hubs.size();
            hubs.push_back(Hub{v, slots, count, groups});
            for (uint32_t i = 0; i < count; ++i)
                ch.push_back(Chunk{vs[v] + i * CH, std::min(vs[v] + (i + 1) * CH, vs[v + 1]), h, i});
            slots += count;
            groups += (count + PPR_GROUP - 1) / PPR_GROUP;
            ++v;
            continue;
        }
        const uint32_t p0 = vs[v];
        uint32_t p1 = vs[v + 1];
        ++v;
        while (v < n && vs[v + 1] - vs[v] <= CH && vs[v + 1] - p0 <= CH) {
            p1 = vs[v + 1];
            ++v;
        }
        ch.push_back(Chunk{p0, p1, NONE, 0});
    }
    d.nchunks = (uint32_t)ch.size();
    d.nhubs = (uint32_t)hubs.size();
    d.nslots = slots;
    d.ngroups = groups;
    EEG_TRY(ppr_alloc(p, (void**)&d.chunk, sizeof(Chunk) * std::max<size_t>(ch.size(), 1)));
    EEG_TRY(ppr_alloc(p, (void**)&d.hub, sizeof(Hub) * std::max<size_t>(hubs.size(), 1)));
    EEG_TRY(ppr_alloc(p, (void**)&d.garrive, sizeof(uint32_t) * std::max<uint32_t>(groups, 1)));
    EEG_TRY(ppr_alloc(p, (void**)&d.harrive, sizeof(uint32_t) * std::max<uint32_t>(d.nhubs, 1)));
    EEG_TRY(ppr_alloc(p, (void**)&d.partial, sizeof(float) * p->W * std::max<uint32_t>(slots, 1)));
    EEG_TRY(ppr_alloc(p, (void**)&d.gpartial, sizeof(float) * p->W * std::max<uint32_t>(groups, 1)));
    EEG_TRY(ppr_alloc(p, (void**)&d.w, sizeof(float) * std::max<size_t>((size_t)vd.P * K, 4)));
    if (!ch.empty())
        EEG_CUDA(cudaMemcpy(d.chunk, ch.data(), sizeof(Chunk) * ch.size(), cudaMemcpyHostToDevice));
    if (!hubs.empty())
        EEG_CUDA(cudaMemcpy(d.hub, hubs.data(), sizeof(Hub) * hubs.size(), cudaMemcpyHostToDevice));
    return EEG_OK;
}

DirTab tab(const VDir& vd, const PPRDir& d) {
    DirTab t{};
    t.vowner = vd.vowner;
    t.vcol = vd.vcol;
    t.w = d.w;
    t.chunk = d.chunk;
    t.nchunks = d.nchunks;
    t.hub = d.hub;
    t.garrive = d.garrive;
    t.harrive = d.harrive;
    t.partial = d.partial;
    t.gpartial = d.gpartial;
    return t;
}

eeg_status reset_counters(const PPRDir& d, cudaStream_t st) {
    EEG_CUDA(cudaMemsetAsync(d.garrive, 0, sizeof(uint32_t) * std::max<uint32_t>(d.ngroups, 1), st));
    EEG_CUDA(cudaMemsetAsync(d.harrive, 0, sizeof(uint32_t) * std::max<uint32_t>(d.nhubs, 1), st));
    return EEG_OK;
}

template <typename Kern>
eeg_status launch_coop(Kern kern, void* arg, int device, uint32_t bps, uint64_t work_warps, cudaStream_t st) {
    int per_sm = 0;
    EEG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PPR_TPB, 0));
    if (per_sm <= 0) {
        set_last_error("personalised PageRank kernel does not fit on an SM");
        return EEG_ERR_CUDA;
    }
    if (bps > 0 && (int)bps < per_sm) per_sm = (int)bps;
    uint64_t blocks = (uint64_t)per_sm * sm_count(device);
    const uint64_t need = (work_warps * 32 + PPR_TPB - 1) / PPR_TPB;
    if (need < blocks) blocks = std::max<uint64_t>(need, 1);
    void* params[] = {arg};
    EEG_CUDA(cudaLaunchCooperativeKernel((const void*)kern, dim3((unsigned)blocks), dim3(PPR_TPB), params, 0, st));
    return EEG_OK;
}

template <int K>
eeg_status launch_solve(eeg_ppr* p, SolveArgs& a, uint32_t bps, cudaStream_t st) {
    const uint64_t work = std::max<uint64_t>(a.g.nchunks, ((uint64_t)a.n * 16 + 31) / 32);
    if (p->W == 1) return launch_coop(k_ppr_scalar<K>, &a, p->vg->device, bps, work, st);
    if (p->W == 32) return launch_coop(k_ppr_rows<K, 8>, &a, p->vg->device, bps, work, st);
    return launch_coop(k_ppr_rows<K, 16>, &a, p->vg->device, bps, work, st);
}

template <int K>
eeg_status launch_grad(eeg_ppr* p, GradArgs& a, cudaStream_t st) {
    const int dev = p->vg->device;
    const uint64_t cap = (uint64_t)sm_count(dev) * (p->W == 1 ? 4 : 2) * (PPR_TPB / 32);
    const uint64_t warps = std::max<uint64_t>(1, std::min<uint64_t>(a.g.nchunks, cap));
    const unsigned blocks = (unsigned)((warps * 32 + PPR_TPB - 1) / PPR_TPB);
    if (p->W == 1)
        k_ppr_grad_scalar<K><<<blocks, PPR_TPB, 0, st>>>(a);
    else if (p->W == 32)
        k_ppr_grad_rows<K, 8><<<blocks, PPR_TPB, 0, st>>>(a);
    else
        k_ppr_grad_rows<K, 16><<<blocks, PPR_TPB, 0, st>>>(a);
    EEG_CUDA(cudaGetLastError());
    return EEG_OK;
}

// Source rows for a solve: the caller's array when it already has the internal layout, else staged.
eeg_status stage_rows(eeg_ppr* p, const float* in, int on_device, cudaStream_t st, const float** out) {
    const uint32_t n = p->vg->n;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (on_device && p->C == p->W && ((uintptr_t)in & 15u) == 0) {
        *out = in;
        return EEG_OK;
    }
    if (p->C == p->W)
        EEG_CUDA(cudaMemcpyAsync(p->b, in, sizeof(float) * (size_t)n * p->W, kind, st));
    else
        EEG_CUDA(cudaMemcpy2DAsync(p->b, sizeof(float) * p->W, in, sizeof(float) * p->C, sizeof(float) * p->C, n, kind, st));
    *out = p->b;
    return EEG_OK;
}

eeg_status unstage_rows(eeg_ppr* p, const float* src, float* dst, int on_device, cudaStream_t st) {
    const uint32_t n = p->vg->n;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (p->C == p->W)
        EEG_CUDA(cudaMemcpyAsync(dst, src, sizeof(float) * (size_t)n * p->W, kind, st));
    else
        EEG_CUDA(cudaMemcpy2DAsync(dst, sizeof(float) * p->C, src, sizeof(float) * p->W, sizeof(float) * p->C, n, kind, st));
    return EEG_OK;
}

eeg_status solve(eeg_ppr* p, bool adjoint, const float* bsrc, const eeg_options& o, cudaStream_t st,
                 eeg_result* res, int* which) {
    eeg_vgraph* vg = p->vg;
    const VDir& vd = adjoint ? vg->fwd : vg->rev;
    PPRDir& d = adjoint ? p->fwd : p->rev;
    float** Y = adjoint ? p->Lb : p->Y;
    const float damping = o.pr_damping > 0.f ? o.pr_damping : 0.85f;
    SolveArgs a{};
    a.g = tab(vd, d);
    a.n = vg->n;
    a.b = bsrc;
    a.scale_b = adjoint ? 1.0f : 1.0f - damping;
    a.d = damping;
    a.y0 = Y[0];
    a.y1 = Y[1];
    a.ctrl = p->ctrl;
    a.max_iters = o.max_iterations ? o.max_iterations : 10000u;
    a.tol = o.pr_tolerance > 0.f ? (double)o.pr_tolerance : 1e-7;
    a.timeout_ns = wait_limit_ns(o);
    EEG_CUDA(cudaMemsetAsync(p->ctrl, 0, sizeof(PRCtrl), st));
    EEG_TRY(reset_counters(d, st));
    switch (vg->K) {
        case 4: EEG_TRY(launch_solve<4>(p, a, o.blocks_per_sm, st)); break;
        case 8: EEG_TRY(launch_solve<8>(p, a, o.blocks_per_sm, st)); break;
        case 16: EEG_TRY(launch_solve<16>(p, a, o.blocks_per_sm, st)); break;
        default: set_last_error("K must be 4, 8 or 16"); return EEG_ERR_UNSUPPORTED;
    }
    PRCtrl hc;
    EEG_CUDA(cudaMemcpyAsync(&hc, p->ctrl, sizeof(PRCtrl), cudaMemcpyDeviceToHost, st));
    EEG_CUDA(cudaStreamSynchronize(st));
    *which = (int)(hc.iterations & 1u);
    const double m = (double)vg->m, n = (double)vg->n;
    res->iterations += hc.iterations;
    res->pr_residual = hc.last_resid;
    res->pr_l1_norm = hc.last_norm;
    res->edges_scanned += (uint64_t)hc.iterations * vg->m;
    res->algorithmic_bytes += (double)hc.iterations * (8.0 * m + (double)p->W * (4.0 * m + 8.0 * n));
    res->launches += 1;
    if (hc.bw.status == DEV_TIMEOUT) {
        set_last_error("grid barrier wait exceeded the timeout");
        return EEG_ERR_TIMEOUT;
    }
    if (hc.bw.status == DEV_ITER_CAP) {
        set_last_error("personalised PageRank did not reach the tolerance within the sweep cap");
        return EEG_ERR_ITER_CAP;
    }
    return EEG_OK;
}

}  // namespace
}  // namespace eeg

using namespace eeg;

extern "C" {

EEG_API eeg_status eeg_ppr_create(eeg_vgraph* vg, uint32_t columns, eeg_ppr** out) {
    if (!vg || !out) {
        set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    *out = nullptr;
    if (columns == 0 || columns > PPR_W) {
        set_last_error("columns must be in [1, 64]");
        return EEG_ERR_INVALID;
    }
    if (!vg->fwd_parts) {
        set_last_error("personalised PageRank needs the forward parts (not EEG_VG_REVERSE_ONLY)");
        return EEG_ERR_INVALID;
    }
    if (!vg->has_rev || vg->rev_alias || !(vg->flags & EEG_VG_EDGE_IDS) || !vg->fwd.veid || !vg->rev.veid) {
        set_last_error("personalised PageRank needs a graph built with EEG_VG_REVERSE | EEG_VG_EDGE_IDS");
        return EEG_ERR_INVALID;
    }
    if (vg->n == 0) {
        set_last_error("empty graph");
        return EEG_ERR_INVALID;
    }
    EEG_CUDA(cudaSetDevice(vg->device));
    eeg_ppr* p = new eeg_ppr();
    p->vg = vg;
    p->C = columns;
    p->W = columns == 1 ? 1u : (columns <= 32 ? 32u : PPR_W);  // row width: 128-B rows up to 32 columns
    const size_t n = vg->n, rows = n * p->W;
    eeg_status s = EEG_OK;
    auto run = [&]() -> eeg_status {
        EEG_TRY(build_chunks(p, vg->fwd, p->fwd));
        EEG_TRY(build_chunks(p, vg->rev, p->rev));
        EEG_TRY(ppr_alloc(p, (void**)&p->w_raw, sizeof(float) * std::max<uint64_t>(vg->m, 1)));
        EEG_TRY(ppr_alloc(p, (void**)&p->s, sizeof(float) * n));
        EEG_TRY(ppr_alloc(p, (void**)&p->bad, sizeof(uint32_t)));
        for (int i = 0; i < 2; ++i) {
            EEG_TRY(ppr_alloc(p, (void**)&p->Y[i], sizeof(float) * rows));
            EEG_TRY(ppr_alloc(p, (void**)&p->Lb[i], sizeof(float) * rows));
        }
        EEG_TRY(ppr_alloc(p, (void**)&p->b, sizeof(float) * rows));
        EEG_CUDA(cudaMemset(p->b, 0, sizeof(float) * rows));  // padding columns stay zero
        EEG_TRY(ppr_alloc(p, (void**)&p->gslot, sizeof(float) * std::max<size_t>((size_t)vg->fwd.P * vg->K, 4)));
        EEG_TRY(ppr_alloc(p, (void**)&p->r, sizeof(float) * n));
        EEG_CUDA(cudaMalloc((void**)&p->ctrl, sizeof(PRCtrl)));
        EEG_CUDA(cudaEventCreate(&p->ev[0]));
        EEG_CUDA(cudaEventCreate(&p->ev[1]));
        return EEG_OK;
    };
    s = run();
    if (s != EEG_OK) {
        eeg_ppr_destroy(p);
        return s;
    }
    *out = p;
    return EEG_OK;
}

EEG_API eeg_status eeg_ppr_set_weights(eeg_ppr* p, const float* w, int on_device) {
    if (!p || (!w && p->vg->m > 0)) {
        set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    eeg_vgraph* vg = p->vg;
    EEG_CUDA(cudaSetDevice(vg->device));
    const uint32_t K = vg->K;
    if (vg->m > 0)
        EEG_CUDA(cudaMemcpy(p->w_raw, w, sizeof(float) * vg->m, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    EEG_CUDA(cudaMemset(p->bad, 0, sizeof(uint32_t)));
    k_ppr_out_sums<<<grid_1d((uint64_t)vg->n * 32, vg->device), PPR_TPB>>>(vg->n, K, vg->fwd.vstart, vg->fwd.veid,
                                                                           p->w_raw, p->s, p->bad);
    const uint64_t fs = (uint64_t)vg->fwd.P * K, rs = (uint64_t)vg->rev.P * K;
    if (fs)
        k_ppr_norm<<<grid_1d(fs, vg->device), PPR_TPB>>>(fs, K, 0, vg->fwd.veid, vg->fwd.vowner, vg->fwd.vcol, p->w_raw,
                                                         p->s, p->fwd.w);
    if (rs)
        k_ppr_norm<<<grid_1d(rs, vg->device), PPR_TPB>>>(rs, K, 1, vg->rev.veid, vg->rev.vowner, vg->rev.vcol, p->w_raw,
                                                         p->s, p->rev.w);
    EEG_CUDA(cudaGetLastError());
    uint32_t bad = 0;
    EEG_CUDA(cudaMemcpy(&bad, p->bad, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (bad) {
        p->have_w = false;
        set_last_error("edge weights must be finite and >= 0");
        return EEG_ERR_INVALID;
    }
    p->have_w = true;
    p->xi = -1;
    return EEG_OK;
}

EEG_API eeg_status eeg_ppr_forward(eeg_ppr* p, const float* teleport, int in_on_device, float* x_out,
                                   int out_on_device, const eeg_options* opts, void* stream, eeg_result* res) {
    if (!p || !teleport) {
        set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    if (!p->have_w) {
        set_last_error("set the edge weights first (eeg_ppr_set_weights)");
        return EEG_ERR_INVALID;
    }
    eeg_options o;
    eeg_options_init(&o);
    if (opts) o = *opts;
    cudaStream_t st = (cudaStream_t)stream;
    EEG_CUDA(cudaSetDevice(p->vg->device));
    eeg_result r;
    memset(&r, 0, sizeof(r));
    p->xi = -1;
    const float* bsrc = nullptr;
    EEG_CUDA(cudaEventRecord(p->ev[0], st));
    EEG_TRY(stage_rows(p, teleport, in_on_device, st, &bsrc));
    int which = 0;
    eeg_status s = solve(p, false, bsrc, o, st, &r, &which);
    if (s != EEG_OK && s != EEG_ERR_ITER_CAP) return s;
    p->xi = which;
    if (x_out) EEG_TRY(unstage_rows(p, p->Y[which], x_out, out_on_device, st));
    EEG_CUDA(cudaEventRecord(p->ev[1], st));
    EEG_CUDA(cudaEventSynchronize(p->ev[1]));
    float ms = 0.f;
    EEG_CUDA(cudaEventElapsedTime(&ms, p->ev[0], p->ev[1]));
    r.kernel_ms = ms;
    r.reached_vertices = p->vg->n;
    r.reached_edges = p->vg->m;
    r.gteps = ms > 0 ? (double)r.iterations * (double)p->vg->m / (ms * 1e-3) / 1e9 : 0.0;
    if (res) *res = r;
    return s;
}

EEG_API eeg_status eeg_ppr_adjoint(eeg_ppr* p, const float* dl_dx, int in_on_device, float* dl_dteleport,
                                   float* dl_dw, float* dl_dwn, int out_on_device, int accumulate,
                                   const eeg_options* opts, void* stream, eeg_result* res) {
    if (!p || !dl_dx) {
        set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    if (p->xi < 0) {
        set_last_error("run eeg_ppr_forward first");
        return EEG_ERR_INVALID;
    }
    eeg_options o;
    eeg_options_init(&o);
    if (opts) o = *opts;
    eeg_vgraph* vg = p->vg;
    cudaStream_t st = (cudaStream_t)stream;
    EEG_CUDA(cudaSetDevice(vg->device));
    const float damping = o.pr_damping > 0.f ? o.pr_damping : 0.85f;
    eeg_result r;
    memset(&r, 0, sizeof(r));
    const float* bsrc = nullptr;
    EEG_CUDA(cudaEventRecord(p->ev[0], st));
    EEG_TRY(stage_rows(p, dl_dx, in_on_device, st, &bsrc));
    int which = 0;
    eeg_status s = solve(p, true, bsrc, o, st, &r, &which);
    if (s != EEG_OK && s != EEG_ERR_ITER_CAP) return s;
    const float* L = p->Lb[which];
    // edge gradients
    GradArgs g{};
    g.g = tab(vg->fwd, p->fwd);
    g.X = p->Y[p->xi];
    g.L = L;
    g.d = damping;
    g.gslot = p->gslot;
    g.r = p->r;
    g.accumulate = (accumulate && p->have_g) ? 1u : 0u;
    EEG_TRY(reset_counters(p->fwd, st));
    switch (vg->K) {
        case 4: EEG_TRY(launch_grad<4>(p, g, st)); break;
        case 8: EEG_TRY(launch_grad<8>(p, g, st)); break;
        case 16: EEG_TRY(launch_grad<16>(p, g, st)); break;
        default: set_last_error("K must be 4, 8 or 16"); return EEG_ERR_UNSUPPORTED;
    }
    p->have_g = true;
    r.launches += 1;
    const uint64_t fs = (uint64_t)vg->fwd.P * vg->K;
    if ((dl_dw || dl_dwn) && fs) {
        float* dwn = dl_dwn;
        float* dw = dl_dw;
        if (!out_on_device) {
            if (!p->stage_m) EEG_TRY(ppr_alloc(p, (void**)&p->stage_m, sizeof(float) * 2 * std::max<uint64_t>(vg->m, 1)));
            dwn = dl_dwn ? p->stage_m : nullptr;
            dw = dl_dw ? p->stage_m + vg->m : nullptr;
        }
        k_ppr_scatter<<<grid_1d(fs, vg->device), PPR_TPB, 0, st>>>(fs, vg->K, vg->fwd.veid, vg->fwd.vowner, p->gslot,
                                                                   p->r, p->s, dwn, dw);
        EEG_CUDA(cudaGetLastError());
        r.launches += 1;
        if (!out_on_device) {
            if (dl_dwn) EEG_CUDA(cudaMemcpyAsync(dl_dwn, dwn, sizeof(float) * vg->m, cudaMemcpyDeviceToHost, st));
            if (dl_dw) EEG_CUDA(cudaMemcpyAsync(dl_dw, dw, sizeof(float) * vg->m, cudaMemcpyDeviceToHost, st));
        }
    }
    if (dl_dteleport) {
        const uint64_t cnt = (uint64_t)vg->n * p->W;
        const bool direct = out_on_device && p->C == p->W;
        if (!direct && !p->stage_nw) EEG_TRY(ppr_alloc(p, (void**)&p->stage_nw, sizeof(float) * cnt));
        float* dst = direct ? dl_dteleport : p->stage_nw;
        k_ppr_scale<<<grid_1d(cnt, vg->device), PPR_TPB, 0, st>>>(cnt, 1.0f - damping, L, dst);
        EEG_CUDA(cudaGetLastError());
        r.launches += 1;
        if (!direct) EEG_TRY(unstage_rows(p, dst, dl_dteleport, out_on_device, st));
    }
    EEG_CUDA(cudaEventRecord(p->ev[1], st));
    EEG_CUDA(cudaEventSynchronize(p->ev[1]));
    float ms = 0.f;
    EEG_CUDA(cudaEventElapsedTime(&ms, p->ev[0], p->ev[1]));
    r.kernel_ms = ms;
    r.reached_vertices = vg->n;
    r.reached_edges = vg->m;
    // gradient pass: per edge 8 B (target + weight) + 4 B gradient + one gathered row of the adjoint
    r.algorithmic_bytes += (double)vg->m * (12.0 + 4.0 * p->W) + (double)vg->n * 4.0 * p->W;
    r.gteps = ms > 0 ? (double)r.iterations * (double)vg->m / (ms * 1e-3) / 1e9 : 0.0;
    if (res) *res = r;
    return s;
}

EEG_API void eeg_ppr_destroy(eeg_ppr* p) {
    if (!p) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(p->vg->device);
    cudaDeviceSynchronize();  // no kernel may still use the arrays
    free_pdir(p, p->fwd);
    free_pdir(p, p->rev);
    eeg_vgraph* vg = p->vg;
    vg_free(vg, p->w_raw);
    vg_free(vg, p->s);
    vg_free(vg, p->bad);
    for (int i = 0; i < 2; ++i) {
        vg_free(vg, p->Y[i]);
        vg_free(vg, p->Lb[i]);
    }
    vg_free(vg, p->b);
    vg_free(vg, p->gslot);
    vg_free(vg, p->r);
    vg_free(vg, p->stage_m);
    vg_free(vg, p->stage_nw);
    if (p->ctrl) cudaFree(p->ctrl);
    if (p->ev[0]) cudaEventDestroy(p->ev[0]);
    if (p->ev[1]) cudaEventDestroy(p->ev[1]);
    cudaSetDevice(prev);
    delete p;
}

}  // extern "C"
