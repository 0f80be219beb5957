// Persistent cooperative kernels: a grid barrier with a bounded wait and the
// launch helper that sizes the grid to what is co-resident.
//
// The barrier is a generation counter: each CTA's thread 0 reads the
// generation, arrives with an atomicAdd, and the last arrival resets the
// count and advances the generation; the others spin (with __nanosleep) until
// it moves. The kernels are launched with cudaLaunchCooperativeKernel, which
// guarantees that every CTA is resident, so the wait always ends; it is still
// capped (kBarrierSpinLimit, about two seconds): on expiry the CTA raises the
// error word and every CTA leaves the kernel at its next barrier, so the host
// sees GBX_ERR_DEVICE_TIMEOUT instead of a hung device.
#pragma once

#include "gbx_internal.cuh"

namespace gbx {

struct GridSync {
    unsigned count;
    unsigned gen;
    unsigned error;  // 1 = a barrier wait expired
    unsigned pad;
};

constexpr unsigned kBarrierSpinLimit = 1u << 25;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Returns false when the grid must stop (a wait expired somewhere).
__device__ __forceinline__ bool grid_barrier(GridSync *gs) {
    __shared__ unsigned s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned ok = 1;
        __threadfence();
        const unsigned my_gen = ld_acquire_u32(&gs->gen);
        const unsigned arrived = atomicAdd(&gs->count, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(&gs->count, 0u);
            __threadfence();
            atomicAdd(&gs->gen, 1u);
        } else {
            unsigned spins = 0;
            while (ld_acquire_u32(&gs->gen) == my_gen) {
                if (++spins > kBarrierSpinLimit) {
                    atomicExch(&gs->error, 1u);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (ld_acquire_u32(&gs->error)) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Largest co-resident grid for `kernel` with `threads` per CTA.
template <class K>
inline int coop_grid(K kernel, int threads, size_t smem, int *grid) {
    int per_sm = 0;
    GBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
    GBX_REQUIRE(per_sm > 0, GBX_ERR_CUDA, "kernel cannot be resident");
    *grid = per_sm * num_sms();
    return GBX_OK;
}

}  // namespace gbx
