// common.cuh -- shared device/host helpers for the EEGraph GB300 kernels.
//
// Device side: acquire/relaxed loads, the global timer, a bounded grid barrier for persistent
// cooperative kernels (no unbounded spin: a wait that outlives its limit records EEG status
// TIMEOUT in the control block and every CTA leaves), and CTA-wide scans.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/eegraph_c.h"

namespace eeg {

constexpr uint32_t INF = 0xFFFFFFFEu;      // DIST_INFINITY = UINT_MAX - 1 (reference include/globals.hpp:32)
constexpr uint32_t NO_EDGE = 0xFFFFFFFFu;  // unused slot of a part (padding up to K)

enum Op : int { OP_BFS = 0, OP_SSSP = 1, OP_SSWP = 2, OP_CC = 3 };

// Device status codes written into control blocks.
enum DevStatus : uint32_t { DEV_OK = 0, DEV_TIMEOUT = 1, DEV_ITER_CAP = 2, DEV_BAD_INPUT = 3, DEV_OVERFLOW = 4 };

// ------------------------------------------------------------------ host error plumbing
void set_last_error(const std::string& msg);
eeg_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define EEG_CUDA(call)                                                        \
    do {                                                                      \
        cudaError_t _e = (call);                                              \
        if (_e != cudaSuccess) return ::eeg::cuda_fail(_e, #call, __FILE__, __LINE__); \
    } while (0)

#define EEG_TRY(call)                        \
    do {                                     \
        eeg_status _s = (call);              \
        if (_s != EEG_OK) return _s;         \
    } while (0)

// Control words shared by every persistent kernel (first fields of each control block).
// A line of its own: pollers never share it with the round counters that working CTAs update
// (R-MAT s22: SSSP 0.706 -> 0.700 ms, CC 1.197 -> 1.188, 4096^2 grid SSSP 27.9 -> 27.5 ms).
struct alignas(128) BarrierWords {
    uint32_t arrive;  // monotone arrival counter (wrap-safe compare)
    uint32_t abort;   // set when any CTA gave up; everyone leaves at the next barrier
    uint32_t status;  // DevStatus (first error wins)
    uint32_t pad[29];
};

#ifdef __CUDACC__
// ------------------------------------------------------------------ device helpers
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// {p[0], p[1]} in one acquire load (p 8-byte aligned)
__device__ __forceinline__ uint2 ld_acquire_v2(const uint32_t* p) {
    uint2 v;
    asm volatile("ld.acquire.gpu.global.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p) : "memory");
    return v;
}
// release-ordered reduction: the writes this thread has made or observed come before the add
__device__ __forceinline__ void red_release_add(uint32_t* p, uint32_t v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Streaming loads for edge arrays that are read once per expansion: bypass L1 and mark the lines
// evict-first in L2 so that the per-vertex value arrays stay resident. sm_100+ has 256-bit global
// loads (v8.b32, 32-byte aligned): one load fetches a whole 8-slot part, i.e. one DRAM sector.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint4 ld_stream_u4(const uint32_t* p, uint64_t pol) {
    uint4 v;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void ld_stream_u8(const uint32_t* p, uint32_t* o) {
    asm volatile("ld.global.nc.L1::no_allocate.L2::evict_first.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(o[0]), "=r"(o[1]), "=r"(o[2]), "=r"(o[3]), "=r"(o[4]), "=r"(o[5]), "=r"(o[6]), "=r"(o[7])
                 : "l"(p));
}
// Load one K-slot part row (K in {4, 8, 16}; row start aligned to 4*K bytes).
template <int K>
__device__ __forceinline__ void ld_part(const uint32_t* p, uint32_t (&o)[K], uint64_t pol) {
    if constexpr (K == 4) {
        const uint4 v = ld_stream_u4(p, pol);
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    } else {
#pragma unroll
        for (int i = 0; i < K; i += 8) ld_stream_u8(p + i, o + i);
    }
}

// Grid-wide barrier for a cooperative launch. `epoch` is a per-CTA counter kept by the caller.
// Returns false when the grid is aborting (timeout elsewhere or here).
__device__ __forceinline__ bool grid_barrier(BarrierWords* bw, uint32_t& epoch, uint64_t timeout_ns) {
    __shared__ uint32_t s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        epoch += 1;
        const uint32_t target = epoch * gridDim.x;
        __threadfence();
        atomicAdd(&bw->arrive, 1u);
        uint32_t ok = 1;
        const uint64_t t0 = global_timer_ns();  // the wait is measured from this CTA's arrival
        uint32_t spins = 0;
        while (true) {
            uint32_t cur = ld_acquire(&bw->arrive);
            if ((int32_t)(cur - target) >= 0) break;
            if (ld_relaxed(&bw->abort)) { ok = 0; break; }
            __nanosleep(32);
            if ((++spins & 7u) == 0) {
                const uint64_t now = global_timer_ns();
                if (now - t0 > timeout_ns) {
                    atomicCAS(&bw->status, (uint32_t)DEV_OK, (uint32_t)DEV_TIMEOUT);
                    atomicExch(&bw->abort, 1u);
                    ok = 0;
                    break;
                }
            }
        }
        if (ok && ld_relaxed(&bw->abort)) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// The same barrier for grids whose CTAs arrive together (PageRank's balanced sweeps): the arrival
// itself releases the CTA's writes (ordered before this thread by the __syncthreads), and each spin is
// one acquire load of the arrivals and the abort word together, so the last arrival is seen one L2
// round trip sooner (R-MAT s22 PageRank, 93 barriers: 17.35 -> 17.10 ms). Where CTAs finish at
// different times the faster polling slowed the CTAs still working (SSSP 0.700 -> 0.719 ms), so the
// traversals keep grid_barrier.
__device__ __forceinline__ bool grid_barrier_sync(BarrierWords* bw, uint32_t& epoch, uint64_t timeout_ns) {
    __shared__ uint32_t s_ok2;
    __syncthreads();
    if (threadIdx.x == 0) {
        epoch += 1;
        const uint32_t target = epoch * gridDim.x;
        red_release_add(&bw->arrive, 1u);
        uint32_t ok = 1;
        const uint64_t t0 = global_timer_ns();
        uint32_t spins = 0;
        while (true) {
            const uint2 w = ld_acquire_v2(&bw->arrive);  // {arrive, abort}
            if (w.y) { ok = 0; break; }
            if ((int32_t)(w.x - target) >= 0) break;
            __nanosleep(32);
            if ((++spins & 7u) == 0) {
                const uint64_t now = global_timer_ns();
                if (now - t0 > timeout_ns) {
                    atomicCAS(&bw->status, (uint32_t)DEV_OK, (uint32_t)DEV_TIMEOUT);
                    atomicExch(&bw->abort, 1u);
                    ok = 0;
                    break;
                }
            }
        }
        s_ok2 = ok;
    }
    __syncthreads();
    return s_ok2 != 0;
}

// Knuth's TwoSum: s + e == a + b exactly (round-to-nearest FP32).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}
// (h1,l1) + (h2,l2) -> normalised pair (compensated FP32 summation)
__device__ __forceinline__ void pair_add(float& h1, float& l1, float h2, float l2) {
    float s, e;
    two_sum(h1, h2, s, e);
    const float t = __fadd_rn(__fadd_rn(l1, l2), e);
    h1 = __fadd_rn(s, t);
    l1 = __fsub_rn(t, __fsub_rn(h1, s));
}

// Exclusive CTA-wide sum scan of one uint32 per thread. `s_warp` needs 33 entries.
// Returns the exclusive prefix; *total receives the CTA sum (all threads).
__device__ __forceinline__ uint32_t block_exclusive_sum(uint32_t x, uint32_t* s_warp, uint32_t* total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t nwarps = blockDim.x >> 5;
    uint32_t inc = x;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= (uint32_t)off) inc += y;
    }
    __syncthreads();
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < nwarps) ? s_warp[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, off);
            if (lane >= (uint32_t)off) wi += y;
        }
        if (lane < nwarps) s_warp[lane] = wi - w;  // exclusive warp offsets
        if (lane == nwarps - 1) s_warp[32] = wi;   // total
    }
    __syncthreads();
    uint32_t res = s_warp[warp] + inc - x;
    *total = s_warp[32];
    __syncthreads();
    return res;
}
#endif  // __CUDACC__

// ------------------------------------------------------------------ device-wide scans (builder)
// out[i] = op-prefix of in; inclusive or exclusive; op = add or max. n < 2^32.
enum ScanOp { SCAN_ADD = 0, SCAN_MAX = 1 };
eeg_status device_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, bool inclusive, ScanOp op,
                           uint32_t* tmp_partials, cudaStream_t st);
uint64_t device_scan_tmp_words(uint64_t n);

int sm_count(int device);

}  // namespace eeg
