// Persistent cooperative kernels: a grid barrier with a bounded wait and the
// launch helper that sizes the grid to what is co-resident.
//
// The barrier is one monotonic 64-bit arrival counter: at its n-th barrier
// each CTA's thread 0 adds 1 with release semantics (no reply awaited) and
// polls the counter with acquire loads until it reaches n * gridDim.x. The
// __syncthreads on either side extends the ordering to the whole CTA. Nobody
// resets or re-arms anything, so a barrier costs one arrival plus one poll
// round trip (about half the latency of a count-and-generation barrier, whose
// last arrival must reset the count and then publish the generation). The
// kernels are launched with cudaLaunchCooperativeKernel, which guarantees
// that every CTA is resident, so the wait always ends; it is still capped
// (kBarrierSpinLimit polls, about two seconds): on expiry the CTA raises the
// error word and every CTA leaves the kernel at its next barrier, so the host
// sees GBX_ERR_DEVICE_TIMEOUT instead of a hung device.
#pragma once

#include "gbx_internal.cuh"

namespace gbx {

struct GridSync {
    unsigned long long arrived;  // total arrivals since launch (zeroed by the host)
    unsigned error;              // 1 = a barrier wait expired
    unsigned pad;
};

constexpr unsigned kBarrierSpinLimit = 1u << 22;

// this CTA's arrival target for its next barrier (set by grid_barrier_init)
__shared__ unsigned long long s_grid_target;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Once at kernel start, before the first grid_barrier (whose leading
// __syncthreads orders it).
__device__ __forceinline__ void grid_barrier_init() {
    if (threadIdx.x == 0) s_grid_target = 0;
}

// Returns false when the grid must stop (a wait expired somewhere).
__device__ __forceinline__ bool grid_barrier(GridSync *gs) {
    __shared__ unsigned s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned long long target = s_grid_target + gridDim.x;
        s_grid_target = target;
        asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(&gs->arrived) : "memory");
        unsigned ok = 1, spins = 0;
        while (ld_acquire_u64(&gs->arrived) < target) {
            if (++spins > kBarrierSpinLimit) {
                atomicExch(&gs->error, 1u);
                break;
            }
            __nanosleep(32);
        }
        if (ld_acquire_u32(&gs->error)) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// After a grid barrier: the first warp copies the step counters *src (a
// struct of 32-bit words) into the CTA's shared *dst, and the CTA waits for
// it. The other warps then read shared memory instead of sending the same
// few L2 lines thousands of requests per step. The barrier's acquire (by
// thread 0) and its closing __syncthreads order the loads after the other
// CTAs' counter updates.
template <class T>
__device__ __forceinline__ void fetch_counters(const T *src, T *dst) {
    static_assert(sizeof(T) % 4 == 0 && sizeof(T) / 4 <= 32, "counters are at most 32 words");
    if (threadIdx.x < sizeof(T) / 4)
        reinterpret_cast<uint32_t *>(dst)[threadIdx.x] = __ldcg(reinterpret_cast<const uint32_t *>(src) + threadIdx.x);
    __syncthreads();
}

// Per-warp staging of queue appends in shared memory: lanes append with
// ballot ranks into the warp's buffer, and the warp reserves space in the
// global queue with one atomic per kWarpQueueCap/2..kWarpQueueCap entries
// instead of one per ballot round (a single global length counter is
// otherwise hammered by every warp of the grid).
constexpr uint32_t kWarpQueueCap = 128;

struct WarpQueue {
    uint32_t *buf;  // kWarpQueueCap entries of shared memory owned by this warp
    uint32_t n;     // fill, identical in all lanes
    __device__ __forceinline__ explicit WarpQueue(uint32_t *b) : buf(b), n(0) {}
    __device__ __forceinline__ void flush(uint32_t *queue, unsigned *len) {
        if (n == 0) return;
        __syncwarp();
        const uint32_t lane = threadIdx.x & 31;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(len, n);
        base = __shfl_sync(0xffffffffu, base, 0);
        for (uint32_t i = lane; i < n; i += 32) queue[base + i] = buf[i];
        __syncwarp();
        n = 0;
    }
    // all lanes call together
    __device__ __forceinline__ void push(uint32_t x, bool p, uint32_t *queue, unsigned *len) {
        const unsigned m = __ballot_sync(0xffffffffu, p);
        if (!m) return;
        const uint32_t lane = threadIdx.x & 31;
        if (p) buf[n + __popc(m & ((1u << lane) - 1u))] = x;
        n += __popc(m);
        if (n > kWarpQueueCap - 32) flush(queue, len);
    }
};

// Work-unit dealer: a warp's first unit is its global warp index (no atomic),
// later ones come from the cursor, offset by the number of warps, so steps
// with little work cost no atomics at all. The cursor increment for the next
// unit is issued when a unit is handed out and its reply is only read at the
// next take(), so its latency overlaps the unit's work.
struct UnitDealer {
    unsigned *cursor;
    uint32_t ticket;  // lane 0: reply of the increment in flight
    uint32_t nwarps;
    bool first;
    __device__ __forceinline__ UnitDealer(unsigned *c)
        : cursor(c), ticket(0), nwarps((gridDim.x * blockDim.x) >> 5), first(true) {}
    __device__ __forceinline__ uint32_t take(uint32_t units) {
        uint32_t u;
        if (first) {
            u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
            first = false;
        } else {
            u = nwarps + __shfl_sync(0xffffffffu, ticket, 0);
        }
        if (u < units && (threadIdx.x & 31) == 0) ticket = atomicAdd(cursor, 1u);
        return u;
    }
};

// Owner of work chunk c in a list whose entry h owns chunks [hc[h], hc[h+1])
// (hc strictly increasing, hc[0] = 0): the last h in [0, n) with hc[h] <= c,
// searched 32 ways at a time by the whole warp -- log32(n) rounds of one
// load per lane instead of log2(n) dependent loads. All lanes call together
// and get the same answer.
__device__ __forceinline__ uint32_t warp_chunk_owner(const uint32_t *hc, uint32_t n, uint32_t c) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t lo = 0, hi = n;  // answer in [lo, hi); hc[lo] <= c
    while (hi - lo > 1) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t idx = lo + lane * step;
        const bool ok = idx < hi && __ldcg(hc + idx) <= c;
        const unsigned m = __ballot_sync(0xffffffffu, ok);  // lane 0 always holds
        lo += (31u - __clz(m)) * step;
        hi = min(lo + step, hi);
    }
    return lo;
}

// Largest co-resident grid for `kernel` with `threads` per CTA. `cache`
// (one per call site, indexed by device) keeps the answer after the first
// occupancy query.
template <class K>
inline int coop_grid(K kernel, int threads, size_t smem, int *grid, int (*cache)[64] = nullptr) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cache && dev >= 0 && dev < 64 && (*cache)[dev] > 0) {
        *grid = (*cache)[dev];
        return GBX_OK;
    }
    int per_sm = 0;
    GBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
    GBX_REQUIRE(per_sm > 0, GBX_ERR_CUDA, "kernel cannot be resident");
    *grid = per_sm * num_sms();
    if (cache && dev >= 0 && dev < 64) (*cache)[dev] = *grid;
    return GBX_OK;
}

}  // namespace gbx
