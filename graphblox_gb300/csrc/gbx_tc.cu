// Triangle count (the reference's triangleCountPullGraphCSR,
// triangleCount.c:254-334): on a (src,dst)-sorted CSR,
//   total = sum over edges u->v with v <= u,
//           over w in N(v) with w <= v, of [w in N(u)].
// On a symmetric, deduplicated, loop-free graph this counts each triangle
// once (w < v < u); after degree reordering (highest degree = id 0) it is the
// degree-ordered DAG count.
//
// One warp per vertex u. N(u)'s prefix of ids <= u is staged in shared
// memory (when it fits) for the membership binary searches. The warp walks
// the v's of that prefix 32 at a time: each lane takes one v and finds the
// length of N(v)'s prefix of ids <= v; a warp scan flattens the (v, w) pairs
// so all 32 lanes stay busy on uneven lists, each lane mapping its pair back
// to (v, w) with a shuffle binary search, as in the pull engine.
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {

constexpr int kTcThreads = 256;
constexpr int kTcWarps = kTcThreads / 32;
constexpr uint32_t kTcStage = 1024;  // ids of N(u) staged per warp

// number of elements <= x in sorted a[0..n)
__device__ __forceinline__ uint32_t count_le(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool contains(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        uint32_t m = a[mid];
        if (m < x) lo = mid + 1; else hi = mid;
    }
    return lo < n && a[lo] == x;
}

__global__ void __launch_bounds__(kTcThreads)
    tc_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest, uint32_t V,
              unsigned long long *total) {
    __shared__ uint32_t stage[kTcWarps][kTcStage];
    __shared__ unsigned long long sred[32];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long count = 0;
    for (uint32_t u = gw; u < V; u += nw) {
        const uint32_t bu = off[u], du = off[u + 1] - bu;
        if (du == 0) continue;
        const uint32_t *nu = dest + bu;
        uint32_t pu = 0;
        if (lane == 0) pu = count_le(nu, du, u);
        pu = __shfl_sync(0xffffffffu, pu, 0);
        if (pu == 0) continue;
        const uint32_t *su = nu;
        if (pu <= kTcStage) {
            for (uint32_t i = lane; i < pu; i += 32) stage[wid][i] = nu[i];
            __syncwarp();
            su = stage[wid];
        }
        for (uint32_t a0 = 0; a0 < pu; a0 += 32) {
            uint32_t a = a0 + lane;
            uint32_t bv = 0, pv = 0;
            if (a < pu) {
                uint32_t v = su[a];
                bv = off[v];
                uint32_t dv = off[v + 1] - bv;
                pv = count_le(dest + bv, dv, v);
            }
            uint32_t incl = pv;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += t;
            }
            uint32_t excl = incl - pv;
            uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
            for (uint32_t i0 = 0; i0 < tot; i0 += 32) {
                uint32_t i = i0 + lane;
                uint32_t k = 0;
#pragma unroll
                for (uint32_t step = 16; step > 0; step >>= 1) {
                    uint32_t cand = k + step;
                    uint32_t pc = __shfl_sync(0xffffffffu, excl, cand);
                    if (pc <= i) k = cand;
                }
                uint32_t pk = __shfl_sync(0xffffffffu, excl, k);
                uint32_t bk = __shfl_sync(0xffffffffu, bv, k);
                if (i < tot) {
                    uint32_t w = __ldg(dest + bk + (i - pk));
                    if (contains(su, pu, w)) count++;
                }
            }
        }
        __syncwarp();
    }
    count = block_sum(count, sred);
    if (threadIdx.x == 0 && count) atomicAdd(total, count);
}

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_tc(gbx_graph *g, uint64_t *total, void *stream) {
    clear_error();
    GBX_REQUIRE(g && total, GBX_ERR_INVALID, "graph or total is NULL");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf<unsigned long long> d;
    GBX_TRY(d.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(d.p, 0, 8, s));
    unsigned grid = std::min<unsigned>(ceil_div((uint64_t)g->V * 32, kTcThreads), (unsigned)num_sms() * 8);
    tc_kernel<<<grid, kTcThreads, 0, s>>>(g->offsets, g->dest, g->V, d.p);
    GBX_LAUNCH_CHECK();
    unsigned long long h = 0;
    if (is_device_ptr(total)) {
        GBX_CUDA(cudaMemcpyAsync(total, d.p, 8, cudaMemcpyDeviceToDevice, s));
        return GBX_OK;
    }
    GBX_CUDA(cudaMemcpyAsync(&h, d.p, 8, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    *total = h;
    return GBX_OK;
}
