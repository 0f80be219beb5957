// Stable LSD radix sort of (uint32 key, uint32 value) pairs, 8 bits per pass,
// used by the CSR build (edges by destination then source, like the
// reference's radixSortEdgesBySourceAndDestination, radixsort.c:285-339) and
// by the degree reordering (radixSortEdgesByDegree, reorder.c:223-269).
//
// Per pass: (1) each 4096-item tile histograms its digits into a digit-major
// table, (2) the table is prefix-summed, so entry (d, t) is the global start
// of tile t's digit-d items, (3) each tile ranks its items stably -- warps own
// 512 consecutive items, processed 32 at a time with __match_any_sync peer
// groups and per-warp digit counters, then a per-digit prefix over warps --
// and scatters keys and values.
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;  // 4096
constexpr uint32_t kRadix = 256;

__global__ void __launch_bounds__(kSortThreads)
    radix_hist_kernel(const uint32_t *__restrict__ keys, uint32_t n, int shift, uint32_t tiles,
                      uint32_t *hist) {
    __shared__ uint32_t h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; ++k) {
        uint64_t i = base + (uint64_t)k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[(uint64_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads)
    radix_scatter_kernel(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                         uint32_t n, int shift, uint32_t tiles, const uint32_t *__restrict__ offs,
                         uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out) {
    __shared__ uint32_t whist[kSortWarps][kRadix];
    __shared__ uint32_t tile_off[kRadix];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < (int)(kSortWarps * kRadix); d += kSortThreads) (&whist[0][0])[d] = 0;
    tile_off[threadIdx.x] = offs[(uint64_t)threadIdx.x * tiles + blockIdx.x];
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kSortTile + (uint64_t)wid * (kSortItems * 32);
    uint32_t k_reg[kSortItems], v_reg[kSortItems], r_reg[kSortItems];
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        uint64_t i = base + (uint64_t)r * 32 + lane;
        bool valid = i < n;
        uint32_t key = valid ? keys[i] : 0u;
        uint32_t d = valid ? ((key >> shift) & 0xFFu) : kRadix;  // invalid lanes form their own group
        k_reg[r] = key;
        v_reg[r] = valid ? vals[i] : 0u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = 0;
        if (valid) before = whist[wid][d];
        __syncwarp();
        uint32_t rank = before + __popc(peers & lt);
        if (valid && (__ffs(peers) - 1) == (int)lane) whist[wid][d] = before + __popc(peers);
        __syncwarp();
        r_reg[r] = valid ? rank : 0xFFFFFFFFu;
    }
    __syncthreads();
    // per-digit exclusive prefix over warps
    {
        uint32_t d = threadIdx.x, run = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            uint32_t c = whist[w][d];
            whist[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        if (r_reg[r] == 0xFFFFFFFFu) continue;
        uint32_t d = (k_reg[r] >> shift) & 0xFFu;
        uint32_t pos = tile_off[d] + whist[wid][d] + r_reg[r];
        keys_out[pos] = k_reg[r];
        vals_out[pos] = v_reg[r];
    }
}

int radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t n, int bits, cudaStream_t s) {
    if (n <= 1 || bits <= 0) return GBX_OK;
    const uint32_t tiles = (uint32_t)(((uint64_t)n + kSortTile - 1) / kSortTile);
    DevBuf<uint32_t> k2, v2, hist, offs;
    GBX_TRY(k2.alloc(n, s));
    GBX_TRY(v2.alloc(n, s));
    GBX_TRY(hist.alloc((size_t)kRadix * tiles, s));
    GBX_TRY(offs.alloc((size_t)kRadix * tiles, s));
    GBX_REQUIRE((uint64_t)kRadix * tiles < 0xFFFFFFFFull, GBX_ERR_INVALID, "sort too large");
    uint32_t *ka = keys, *va = vals, *kb = k2.p, *vb = v2.p;
    int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        radix_hist_kernel<<<tiles, kSortThreads, 0, s>>>(ka, n, shift, tiles, hist.p);
        GBX_LAUNCH_CHECK();
        GBX_TRY(exclusive_scan_u32(hist.p, offs.p, kRadix * tiles, s, nullptr));
        radix_scatter_kernel<<<tiles, kSortThreads, 0, s>>>(ka, va, n, shift, tiles, offs.p, kb, vb);
        GBX_LAUNCH_CHECK();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys) {
        GBX_CUDA(cudaMemcpyAsync(keys, ka, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
        GBX_CUDA(cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    }
    return GBX_OK;
}

}  // namespace gbx
