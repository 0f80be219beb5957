// Edge-balanced frontier expansion shared by the push-style kernels (SSSP,
// CC hooking sweeps): the frontier queue's out-degrees are prefix-summed and
// a persistent grid walks the flattened edge list in tiles, so a hub vertex
// is spread over many CTAs instead of serialising one warp.
#pragma once

#include "gbx_internal.cuh"

namespace gbx {

constexpr int kExpThreads = 256;
constexpr int kExpItems = 4;
constexpr uint32_t kExpTile = kExpThreads * kExpItems;

__device__ __forceinline__ uint32_t upper_index(const uint32_t *pre, uint32_t lo, uint32_t hi,
                                                uint32_t i) {
    // largest f in [lo, hi] with pre[f] <= i
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(pre + mid) <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Visitor: __device__ void operator()(uint32_t v, uint32_t e, uint32_t u, bool active)
//          is called by every thread of a warp together (active = the lane
//          has an edge), so it may use warp collectives.
//          __device__ void finish() -- once per thread at the end.
template <class Visitor>
__global__ void __launch_bounds__(kExpThreads)
    expand_kernel(const uint32_t *__restrict__ q, const uint32_t *__restrict__ pre, uint32_t qlen,
                  const uint32_t *__restrict__ total_edges, const uint32_t *__restrict__ off,
                  const uint32_t *__restrict__ dest, Visitor vis) {
    __shared__ uint32_t s_range[2];
    const uint32_t M = *total_edges;
    for (uint64_t base = (uint64_t)blockIdx.x * kExpTile; base < M; base += (uint64_t)gridDim.x * kExpTile) {
        uint64_t tile_end = base + kExpTile < M ? base + kExpTile : (uint64_t)M;
        if (threadIdx.x < 2) {
            uint32_t target = threadIdx.x == 0 ? (uint32_t)base : (uint32_t)tile_end - 1;
            s_range[threadIdx.x] = upper_index(pre, 0, qlen - 1, target);
        }
        __syncthreads();
        const uint32_t flo = s_range[0], fhi = s_range[1];
#pragma unroll
        for (int k = 0; k < kExpItems; ++k) {
            uint64_t i = base + (uint64_t)k * kExpThreads + threadIdx.x;
            uint32_t v = 0, e = 0, u = 0;
            bool active = i < M;
            if (active) {
                uint32_t f = upper_index(pre, flo, fhi, (uint32_t)i);
                v = __ldg(q + f);
                e = __ldg(off + v) + ((uint32_t)i - __ldg(pre + f));
                u = __ldg(dest + e);
            }
            vis(v, e, u, active);
        }
        __syncthreads();
    }
    vis.finish();
}

__global__ void gather_queue_degrees_kernel(const uint32_t *q, uint32_t qlen, const uint32_t *deg,
                                            uint32_t *out);

// warp-aggregated append of `x` when `push` (all lanes call together)
__device__ __forceinline__ void warp_append(uint32_t *queue, uint32_t *len, uint32_t x, bool push) {
    unsigned m = __ballot_sync(0xffffffffu, push);
    if (!m) return;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t leader = __ffs(m) - 1;
    uint32_t basepos = 0;
    if (lane == leader) basepos = atomicAdd(len, (uint32_t)__popc(m));
    basepos = __shfl_sync(0xffffffffu, basepos, leader);
    if (push) queue[basepos + __popc(m & ((1u << lane) - 1u))] = x;
}

// Prefix-sum the degrees of q[0..qlen) into pre/total and launch the expansion.
template <class Visitor>
inline int expand_frontier(const uint32_t *q, uint32_t qlen, const uint32_t *off, const uint32_t *dest,
                           const uint32_t *deg, uint32_t *degs_tmp, uint32_t *pre, uint32_t *total,
                           Visitor vis, cudaStream_t s) {
    if (qlen == 0) return GBX_OK;
    unsigned g = ceil_div(qlen, 256);
    unsigned cap = (unsigned)num_sms() * 8;
    gather_queue_degrees_kernel<<<g < cap ? g : cap, 256, 0, s>>>(q, qlen, deg, degs_tmp);
    GBX_LAUNCH_CHECK();
    GBX_TRY(exclusive_scan_u32(degs_tmp, pre, qlen, s, total));
    expand_kernel<Visitor><<<num_sms() * 8, kExpThreads, 0, s>>>(q, pre, qlen, total, off, dest, vis);
    GBX_LAUNCH_CHECK();
    return GBX_OK;
}

}  // namespace gbx
