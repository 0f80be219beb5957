// Pull engine: for every row v of a CSR, sum a per-edge term over the row's
// edges and hand the sum to a per-row epilogue. Shared by PageRank pull,
// SpMV and the personalised-PageRank forward/adjoint.
//
// Rows are split by degree once per graph (gbx_gather_plan):
//   light  (deg <= kLightMax): groups of 32 consecutive rows per warp. The
//          warp streams the group's edges with consecutive lanes on
//          consecutive edges (coalesced index loads, one gather each) into
//          shared memory, then lane k sums row k from shared memory and runs
//          the epilogue, so per-row writes are coalesced too.
//   medium (kLightMax < deg <= heavy_min): one warp per row, Kahan-compensated
//          per-lane sums, shuffle reduction.
//   heavy  (deg > heavy_min): one CTA per row, Kahan per thread, block tree.
// One launch covers all three classes: heavy CTAs first, then medium, then
// light, selected by blockIdx.
#pragma once

#include "gbx_internal.cuh"

struct gbx_gather_plan {
    uint32_t V = 0;
    uint32_t heavy_min = 0;
    uint32_t n_medium = 0;
    uint32_t n_heavy = 0;
    uint32_t *medium_rows = nullptr;  // device
    uint32_t *heavy_rows = nullptr;   // device
};

namespace gbx {

constexpr int kGatherThreads = 256;
constexpr int kGatherWarps = kGatherThreads / 32;
constexpr uint32_t kLightMax = 32;
constexpr uint32_t kLightBuf = 32 * kLightMax;  // floats per warp

// Kahan-compensated running sum
struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        float y = __fsub_rn(x, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ float value() const { return s; }
};

struct GatherGeometry {
    uint32_t heavy_blocks;
    uint32_t medium_blocks;
    uint32_t light_blocks;
    uint32_t total() const { return heavy_blocks + medium_blocks + light_blocks; }
};

inline GatherGeometry gather_geometry(const gbx_gather_plan &p) {
    GatherGeometry g;
    g.heavy_blocks = p.n_heavy;
    g.medium_blocks = (p.n_medium + kGatherWarps - 1) / kGatherWarps;
    uint32_t groups = (p.V + 31) / 32;
    g.light_blocks = (groups + kGatherWarps - 1) / kGatherWarps;
    return g;
}

// Term:  __device__ float operator()(uint32_t e) const   -- value of edge e
// Epi:   __device__ void operator()(uint32_t v, float sum)  -- per-row epilogue
//        __device__ void block_finish()                       -- once per CTA, all threads
template <class Term, class Epi>
__device__ __forceinline__ void gather_rows_kernel_body(const uint32_t *__restrict__ off, uint32_t V,
                                                        const gbx_gather_plan &plan,
                                                        const GatherGeometry &geo, const Term &term,
                                                        Epi &epi) {
    __shared__ float sbuf[kGatherWarps][kLightBuf];
    __shared__ float sred[32];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t bid = blockIdx.x;
    if (bid < geo.heavy_blocks) {
        // ---- one CTA per heavy row
        uint32_t v = plan.heavy_rows[bid];
        uint32_t b = off[v], e = off[v + 1];
        Kahan k;
        for (uint32_t j = b + threadIdx.x; j < e; j += blockDim.x) k.add(term(j));
        float s = block_sum(k.value(), sred);
        if (threadIdx.x == 0) epi(v, s);
    } else if (bid < geo.heavy_blocks + geo.medium_blocks) {
        // ---- one warp per medium row
        uint32_t idx = (bid - geo.heavy_blocks) * kGatherWarps + wid;
        if (idx < plan.n_medium) {
            uint32_t v = plan.medium_rows[idx];
            uint32_t b = off[v], e = off[v + 1];
            Kahan k;
            for (uint32_t j = b + lane; j < e; j += 32) k.add(term(j));
            float s = warp_sum(k.value());
            if (lane == 0) epi(v, s);
        }
    } else {
        // ---- 32 consecutive light rows per warp
        uint32_t group = (bid - geo.heavy_blocks - geo.medium_blocks) * kGatherWarps + wid;
        uint32_t v = group * 32 + lane;
        uint32_t b = 0, d = 0;
        if (v < V) {
            b = off[v];
            d = off[v + 1] - b;
        }
        uint32_t dl = d <= kLightMax ? d : 0;
        uint32_t incl = dl;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += t;
        }
        uint32_t excl = incl - dl;
        uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        float *buf = sbuf[wid];
        for (uint32_t i0 = 0; i0 < total; i0 += 32) {
            uint32_t i = i0 + lane;
            // last row k whose exclusive prefix is <= i (shuffle binary search)
            uint32_t k = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1) {
                uint32_t cand = k + step;
                uint32_t pc = __shfl_sync(0xffffffffu, excl, cand);
                if (pc <= i) k = cand;
            }
            uint32_t pk = __shfl_sync(0xffffffffu, excl, k);
            uint32_t bk = __shfl_sync(0xffffffffu, b, k);
            if (i < total) buf[i] = term(bk + (i - pk));
        }
        __syncwarp();
        if (v < V && d <= kLightMax) {
            float s = 0.f;
            for (uint32_t j = 0; j < d; ++j) s = __fadd_rn(s, buf[excl + j]);
            epi(v, s);
        }
    }
    epi.block_finish();
}

template <class Term, class Epi>
__global__ void __launch_bounds__(kGatherThreads)
    gather_rows_kernel(const uint32_t *__restrict__ off, uint32_t V, gbx_gather_plan plan,
                       GatherGeometry geo, Term term, Epi epi) {
    gather_rows_kernel_body(off, V, plan, geo, term, epi);
}

template <class Term, class Epi>
inline int launch_gather(const uint32_t *off, uint32_t V, const gbx_gather_plan &plan, Term term,
                         Epi epi, cudaStream_t s) {
    GatherGeometry geo = gather_geometry(plan);
    if (geo.total() == 0) return GBX_OK;
    gather_rows_kernel<Term, Epi><<<geo.total(), kGatherThreads, 0, s>>>(off, V, plan, geo, term, epi);
    GBX_LAUNCH_CHECK();
    return GBX_OK;
}

}  // namespace gbx
