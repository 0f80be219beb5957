// Device-wide exclusive prefix sums (reduce -> scan of partials -> downsweep).
// Each block covers kTile = 256 threads x 16 items; partial sums are scanned
// recursively. Used for CSR offsets, frontier expansion and compaction.
#include "gbx_internal.cuh"

namespace gbx {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

template <typename Out>
__device__ __forceinline__ Out block_exclusive_scan(Out v, Out *warp_tot, Out *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    Out incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        Out t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        Out w = lane < (kScanThreads / 32) ? warp_tot[lane] : Out(0);
        Out wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            Out t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < (kScanThreads / 32)) warp_tot[lane] = wi - w;
        if (lane == (kScanThreads / 32) - 1) *total = wi;
    }
    __syncthreads();
    return incl - v + warp_tot[wid];
}

template <typename In, typename Out>
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const In *in, Out *partials, uint32_t n) {
    __shared__ Out sh[32];
    uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    Out s = 0;
#pragma unroll 4
    for (int k = 0; k < kScanItems; ++k) {
        uint64_t i = base + (uint64_t)k * kScanThreads + threadIdx.x;
        if (i < n) s += (Out)in[i];
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

template <typename In, typename Out>
__global__ void __launch_bounds__(kScanThreads)
    scan_down_kernel(const In *in, Out *out, const Out *block_off, uint32_t n, Out *total_out) {
    __shared__ Out tile[kScanTile];
    __shared__ Out warp_tot[32];
    __shared__ Out tot;
    uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    for (int k = 0; k < kScanItems; ++k) {
        uint32_t j = k * kScanThreads + threadIdx.x;
        uint64_t i = base + j;
        tile[j] = i < n ? (Out)in[i] : Out(0);
    }
    __syncthreads();
    Out local[kScanItems];
    Out sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        local[k] = tile[threadIdx.x * kScanItems + k];
        sum += local[k];
    }
    Out pre = block_exclusive_scan(sum, warp_tot, &tot);
    Out off = (block_off ? block_off[blockIdx.x] : Out(0)) + pre;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        tile[threadIdx.x * kScanItems + k] = off;
        off += local[k];
    }
    __syncthreads();
    for (int k = 0; k < kScanItems; ++k) {
        uint32_t j = k * kScanThreads + threadIdx.x;
        uint64_t i = base + j;
        if (i < n) out[i] = tile[j];
    }
    if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        Out last = (block_off ? block_off[blockIdx.x] : Out(0)) + tot;
        *total_out = last;
    }
}

template <typename In, typename Out>
static int scan_impl(const In *in, Out *out, uint32_t n, cudaStream_t s, Out *total) {
    if (n == 0) {
        if (total) GBX_CUDA(cudaMemsetAsync(total, 0, sizeof(Out), s));
        return GBX_OK;
    }
    uint32_t blocks = (uint32_t)(((uint64_t)n + kScanTile - 1) / kScanTile);
    if (blocks == 1) {
        scan_down_kernel<In, Out><<<1, kScanThreads, 0, s>>>(in, out, nullptr, n, total);
        GBX_LAUNCH_CHECK();
        return GBX_OK;
    }
    DevBuf<Out> partials, offs;
    GBX_TRY(partials.alloc(blocks, s));
    GBX_TRY(offs.alloc(blocks, s));
    scan_reduce_kernel<In, Out><<<blocks, kScanThreads, 0, s>>>(in, partials.p, n);
    GBX_LAUNCH_CHECK();
    GBX_TRY((scan_impl<Out, Out>(partials.p, offs.p, blocks, s, (Out *)nullptr)));
    scan_down_kernel<In, Out><<<blocks, kScanThreads, 0, s>>>(in, out, offs.p, n, total);
    GBX_LAUNCH_CHECK();
    return GBX_OK;
}

int exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, cudaStream_t s,
                       uint32_t *total_dev) {
    return scan_impl<uint32_t, uint32_t>(in, out, n, s, total_dev);
}

int exclusive_scan_u64(const uint32_t *in, uint64_t *out, uint32_t n, cudaStream_t s) {
    return scan_impl<uint32_t, uint64_t>(in, out, n, s, (uint64_t *)nullptr);
}

}  // namespace gbx
