// Triangle count (the reference's triangleCountPullGraphCSR,
// triangleCount.c:254-334): on a (src,dst)-sorted CSR,
//   total = sum over edges u->v with v <= u,
//           over w in N(v) with w <= v, of [w in N(u)].
// On a symmetric, deduplicated, loop-free graph this counts each triangle
// once (w < v < u); after degree reordering (highest degree = id 0) it is the
// degree-ordered DAG count.
//
// Let N+(x) = N(x) ∩ [0, x], a prefix of the sorted row (its length is cached
// per graph in low_count). Every w of N+(v) is <= v, so the reference's term
// for the pair (u, v) is the number of w in N+(v) that are in N+(u).
//
// Rows without repeated neighbours (checked once per graph): N+(u) is put in
// an open-addressing hash table in shared memory, then the N+(v) lists of all
// v in N+(u) are streamed with consecutive lanes on consecutive elements
// (coalesced) and each element costs one or two shared-memory probes. Work
// is flattened over 32 v's at a time so short lists do not idle lanes; each
// lane walks its item -> v mapping forward through a per-warp prefix table.
//   light u (|N+(u)| <= kTcLightMax): one warp per u, a per-warp table;
//   heavy u: one CTA per u, one table per CTA, warps split the v's.
// Rows with repeated neighbours keep the reference's multiplicities with a
// binary search of N+(u) in global memory per element of N+(v).
#include <algorithm>
#include <vector>

#include "gbx_internal.cuh"

namespace gbx {

constexpr int kTcThreads = 256;
constexpr int kTcWarps = kTcThreads / 32;
constexpr uint32_t kTcLightMax = 512;       // |N+(u)| handled by one warp
constexpr uint32_t kTcWarpSlots = 1024;     // hash slots per warp (light)
constexpr uint32_t kTcHeavyMax = 4096;      // |N+(u)| handled with a CTA table
constexpr uint32_t kTcCtaSlots = 8192;      // hash slots per CTA (heavy)
constexpr uint32_t kEmptySlot = 0xFFFFFFFFu;

// number of elements <= x in sorted a[0..n)
__device__ __forceinline__ uint32_t count_le(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= x) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool sorted_contains(const uint32_t *a, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < x) lo = mid + 1; else hi = mid;
    }
    return lo < n && __ldg(a + lo) == x;
}

__device__ __forceinline__ uint32_t hash_slot(uint32_t x, uint32_t mask) {
    return (x * 0x9E3779B1u >> 7) & mask;
}

__device__ __forceinline__ void hash_insert(uint32_t *table, uint32_t mask, uint32_t x) {
    uint32_t h = hash_slot(x, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        uint32_t old = atomicCAS(table + h, kEmptySlot, x);
        if (old == kEmptySlot || old == x) return;
        h = (h + 1) & mask;
    }
}

__device__ __forceinline__ bool hash_contains(const uint32_t *table, uint32_t mask, uint32_t x) {
    uint32_t h = hash_slot(x, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        uint32_t t = table[h];
        if (t == x) return true;
        if (t == kEmptySlot) return false;
        h = (h + 1) & mask;
    }
    return false;
}

__device__ __forceinline__ uint32_t table_mask(uint32_t n, uint32_t max_slots) {
    uint32_t t = 64;
    while (t < 2 * n && t < max_slots) t <<= 1;
    return t - 1;
}

__global__ void tc_low_count_kernel(const uint32_t *off, const uint32_t *dest, uint32_t V, uint32_t *low) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        uint32_t b = off[v];
        low[v] = count_le(dest + b, off[v + 1] - b, v);
    }
}

// rows with a repeated neighbour (sorted rows: adjacent equal ids)
__global__ void tc_dup_check_kernel(const uint32_t *off, const uint32_t *dest, uint32_t V, unsigned *dups) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    bool found = false;
    for (uint32_t v = gw; v < V; v += nw) {
        uint32_t b = off[v], e = off[v + 1];
        for (uint32_t j = b + 1 + lane; j < e; j += 32)
            if (dest[j] == dest[j - 1]) found = true;
    }
    if (__any_sync(0xffffffffu, found) && lane == 0) atomicOr(dups, 1u);
}

// Stream N+(v) for the (up to 32) v's su[a0 .. a0+cnt) of one u and count the
// elements found by `member`. All lanes of the warp call this together.
template <class Member>
__device__ __forceinline__ unsigned long long stream_lists(const uint32_t *__restrict__ off,
                                                          const uint32_t *__restrict__ dest,
                                                          const uint32_t *__restrict__ low,
                                                          const uint32_t *nu, uint32_t a0, uint32_t cnt,
                                                          uint32_t *s_pre, uint32_t *s_base,
                                                          const Member &member) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t pv = 0, bv = 0;
    if (lane < cnt) {
        uint32_t v = __ldg(nu + a0 + lane);
        pv = __ldg(low + v);
        bv = __ldg(off + v);
    }
    uint32_t incl = pv;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    s_pre[lane] = incl - pv;
    s_base[lane] = bv;
    if (lane == 31) s_pre[32] = incl;
    __syncwarp();
    const uint32_t tot = s_pre[32];
    unsigned long long count = 0;
    uint32_t k = 0;  // owner row of this lane's current item, advanced monotonically
    for (uint32_t i0 = 0; i0 < tot; i0 += 128) {
        uint32_t w[4];
        bool ok[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint32_t i = i0 + q * 32 + lane;
            ok[q] = i < tot;
            w[q] = 0;
            if (ok[q]) {
                while (s_pre[k + 1] <= i) ++k;
                w[q] = __ldg(dest + s_base[k] + (i - s_pre[k]));
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (ok[q] && member(w[q])) count++;
    }
    __syncwarp();
    return count;
}

struct HashMember {
    const uint32_t *table;
    uint32_t mask;
    __device__ __forceinline__ bool operator()(uint32_t w) const { return hash_contains(table, mask, w); }
};

struct SortedMember {
    const uint32_t *list;
    uint32_t n;
    __device__ __forceinline__ bool operator()(uint32_t w) const { return sorted_contains(list, n, w); }
};

__global__ void __launch_bounds__(kTcThreads)
    tc_hash_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest,
                   const uint32_t *__restrict__ low, const uint32_t *__restrict__ heavy, uint32_t n_heavy,
                   uint32_t V, unsigned long long *total) {
    __shared__ uint32_t table[kTcCtaSlots];  // CTA table, or kTcWarps per-warp tables
    __shared__ uint32_t s_pre[kTcWarps][33];
    __shared__ uint32_t s_base[kTcWarps][32];
    __shared__ unsigned long long sred[32];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long count = 0;
    if (blockIdx.x < n_heavy) {
        // ---- heavy u: one CTA, one table
        const uint32_t u = heavy[blockIdx.x];
        const uint32_t pu = low[u];
        const uint32_t *nu = dest + off[u];
        if (pu <= kTcHeavyMax) {
            const uint32_t mask = table_mask(pu, kTcCtaSlots);
            for (uint32_t i = threadIdx.x; i <= mask; i += blockDim.x) table[i] = kEmptySlot;
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < pu; i += blockDim.x) hash_insert(table, mask, __ldg(nu + i));
            __syncthreads();
            HashMember m{table, mask};
            for (uint32_t a0 = wid * 32; a0 < pu; a0 += kTcWarps * 32)
                count += stream_lists(off, dest, low, nu, a0, min(32u, pu - a0), s_pre[wid], s_base[wid], m);
        } else {
            SortedMember m{nu, pu};
            for (uint32_t a0 = wid * 32; a0 < pu; a0 += kTcWarps * 32)
                count += stream_lists(off, dest, low, nu, a0, min(32u, pu - a0), s_pre[wid], s_base[wid], m);
        }
    } else {
        // ---- light u: one warp per u, per-warp table
        uint32_t *wt = table + wid * kTcWarpSlots;
        const uint32_t nwarps = (gridDim.x - n_heavy) * kTcWarps;
        for (uint32_t u = (blockIdx.x - n_heavy) * kTcWarps + wid; u < V; u += nwarps) {
            const uint32_t pu = __ldg(low + u);
            if (pu == 0 || pu > kTcLightMax) continue;
            const uint32_t *nu = dest + __ldg(off + u);
            const uint32_t mask = table_mask(pu, kTcWarpSlots);
            for (uint32_t i = lane; i <= mask; i += 32) wt[i] = kEmptySlot;
            __syncwarp();
            for (uint32_t i = lane; i < pu; i += 32) hash_insert(wt, mask, __ldg(nu + i));
            __syncwarp();
            HashMember m{wt, mask};
            for (uint32_t a0 = 0; a0 < pu; a0 += 32)
                count += stream_lists(off, dest, low, nu, a0, min(32u, pu - a0), s_pre[wid], s_base[wid], m);
        }
    }
    count = block_sum(count, sred);
    if (threadIdx.x == 0 && count) atomicAdd(total, count);
}

// Rows with repeated neighbours: the reference's multiplicities. For each
// v in N+(u) (with repeats), each w in N+(v) (with repeats) counts when w is
// in N(u); a binary search of N+(u) decides it.
__global__ void __launch_bounds__(kTcThreads)
    tc_multiset_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest,
                       const uint32_t *__restrict__ low, uint32_t V, unsigned long long *total) {
    __shared__ uint32_t s_pre[kTcWarps][33];
    __shared__ uint32_t s_base[kTcWarps][32];
    __shared__ unsigned long long sred[32];
    const uint32_t wid = threadIdx.x >> 5;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long count = 0;
    for (uint32_t u = gw; u < V; u += nw) {
        const uint32_t pu = __ldg(low + u);
        if (pu == 0) continue;
        const uint32_t *nu = dest + __ldg(off + u);
        SortedMember m{nu, pu};
        for (uint32_t a0 = 0; a0 < pu; a0 += 32)
            count += stream_lists(off, dest, low, nu, a0, min(32u, pu - a0), s_pre[wid], s_base[wid], m);
    }
    count = block_sum(count, sred);
    if (threadIdx.x == 0 && count) atomicAdd(total, count);
}

__global__ void tc_heavy_flags_kernel(const uint32_t *low, uint32_t V, uint32_t *flag) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        flag[v] = low[v] > kTcLightMax ? 1u : 0u;
}

__global__ void tc_scatter_kernel(const uint32_t *flag, const uint32_t *pos, uint32_t V, uint32_t *out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        if (flag[v]) out[pos[v]] = v;
}

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_tc(gbx_graph *g, uint64_t *total, void *stream) {
    clear_error();
    GBX_REQUIRE(g && total, GBX_ERR_INVALID, "graph or total is NULL");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    DevBuf<unsigned long long> d;
    GBX_TRY(d.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(d.p, 0, 8, s));
    const unsigned grid = std::min<unsigned>(ceil_div(V, 256), (unsigned)num_sms() * 8);
    const unsigned wgrid = std::min<unsigned>(ceil_div((uint64_t)V * 32, kTcThreads), (unsigned)num_sms() * 6);
    if (g->simple_rows < 0) {
        DevBuf<unsigned> dup;
        GBX_TRY(dup.alloc(1, s));
        GBX_CUDA(cudaMemsetAsync(dup.p, 0, 4, s));
        tc_dup_check_kernel<<<wgrid, kTcThreads, 0, s>>>(g->offsets, g->dest, V, dup.p);
        GBX_LAUNCH_CHECK();
        unsigned h = 0;
        GBX_CUDA(cudaMemcpyAsync(&h, dup.p, 4, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        g->simple_rows = h ? 0 : 1;
    }
    if (!g->low_count) {
        uint32_t *low = nullptr;
        GBX_CUDA(cudaMalloc(&low, (size_t)V * 4));
        tc_low_count_kernel<<<grid, 256, 0, s>>>(g->offsets, g->dest, V, low);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            cudaFree(low);
            return cuda_fail(e, "tc_low_count_kernel", __FILE__, __LINE__);
        }
        g->low_count = low;
    }
    if (g->simple_rows == 1) {
        // u whose N+(u) is too long for a warp table get a CTA each (ascending ids)
        DevBuf<uint32_t> flag, pos, tot, heavy;
        GBX_TRY(flag.alloc(V, s));
        GBX_TRY(pos.alloc(V, s));
        GBX_TRY(tot.alloc(1, s));
        tc_heavy_flags_kernel<<<grid, 256, 0, s>>>(g->low_count, V, flag.p);
        GBX_LAUNCH_CHECK();
        GBX_TRY(exclusive_scan_u32(flag.p, pos.p, V, s, tot.p));
        uint32_t n_heavy = 0;
        GBX_CUDA(cudaMemcpyAsync(&n_heavy, tot.p, 4, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        GBX_TRY(heavy.alloc(n_heavy ? n_heavy : 1, s));
        tc_scatter_kernel<<<grid, 256, 0, s>>>(flag.p, pos.p, V, heavy.p);
        GBX_LAUNCH_CHECK();
        tc_hash_kernel<<<n_heavy + wgrid, kTcThreads, 0, s>>>(g->offsets, g->dest, g->low_count, heavy.p,
                                                              n_heavy, V, d.p);
        GBX_LAUNCH_CHECK();
    } else {
        tc_multiset_kernel<<<wgrid, kTcThreads, 0, s>>>(g->offsets, g->dest, g->low_count, V, d.p);
        GBX_LAUNCH_CHECK();
    }
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
