// Pull engine: for every row v of a CSR, sum a per-edge term over the row's
// edges and hand the sum to a per-row epilogue. Shared by PageRank pull,
// SpMV and the personalised-PageRank forward/adjoint.
//
// Rows are split by degree once per graph (gbx_gather_plan):
//   light  (deg <= kLightMax): groups of 32 consecutive rows per warp. The
//          warp streams the group's edges with consecutive lanes on
//          consecutive edges (coalesced index loads) into shared memory, then
//          lane k sums row k from shared memory and runs the epilogue, so the
//          per-row writes are coalesced too.
//   medium (kLightMax < deg <= heavy_min): one warp per row, Kahan sums.
//   heavy  (deg > heavy_min): the row is cut into chunks of kHeavyChunk edges,
//          one CTA per chunk. Each CTA writes its partial sum; the CTA that
//          finishes a row last (atomic ticket after a __threadfence) adds the
//          partials in chunk order -- deterministic -- runs the epilogue and
//          re-arms the ticket for the next launch. No CTA ever waits.
// Every class issues its index loads for several edges before the dependent
// gathers (kUnroll in flight per thread): the sweep is latency-bound unless
// each SM keeps hundreds of loads outstanding.
// One launch covers all classes: heavy chunks first, then medium, then light.
#pragma once

#include "gbx_internal.cuh"

struct gbx_gather_plan {
    uint32_t V = 0;
    uint32_t heavy_min = 0;
    uint32_t n_medium = 0;
    uint32_t n_heavy = 0;
    uint32_t n_chunks = 0;             // heavy chunks in total
    uint32_t *medium_rows = nullptr;   // device [n_medium]
    uint32_t *heavy_rows = nullptr;    // device [n_heavy]
    uint32_t *chunk_heavy = nullptr;   // device [n_chunks]: heavy index of each chunk
    uint32_t *heavy_first = nullptr;   // device [n_heavy+1]: first chunk of each heavy row
    float *partials = nullptr;         // device [n_chunks]
    unsigned *tickets = nullptr;       // device [n_heavy], zero between launches
};

namespace gbx {

constexpr int kGatherThreads = 256;
constexpr int kGatherWarps = kGatherThreads / 32;
constexpr uint32_t kLightMax = 32;
constexpr uint32_t kLightBuf = 256;  // shared-memory window (floats) per warp
constexpr int kUnroll = 4;
constexpr uint32_t kHeavyChunk = kGatherThreads * 16;  // edges per heavy CTA

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
    __host__ __device__ uint32_t total() const { return heavy_blocks + medium_blocks + light_blocks; }
};

inline GatherGeometry gather_geometry(const gbx_gather_plan &p) {
    GatherGeometry g;
    g.heavy_blocks = p.n_chunks;
    g.medium_blocks = (p.n_medium + kGatherWarps - 1) / kGatherWarps;
    uint32_t groups = (p.V + 31) / 32;
    g.light_blocks = (groups + kGatherWarps - 1) / kGatherWarps;
    return g;
}

// Term:  __device__ uint32_t src_of(uint32_t e) const     -- first (index) load of edge e
//        __device__ float value(uint32_t e, uint32_t u) const -- dependent gather -> edge value
// Epi:   __device__ void operator()(uint32_t v, float sum)  -- per-row epilogue
//        __device__ void block_finish()                      -- once per CTA, all threads
template <class Term, class Epi>
__device__ __forceinline__ void gather_unit(const uint32_t *__restrict__ off, uint32_t V,
                                            const gbx_gather_plan &plan, const GatherGeometry &geo,
                                            const Term &term, Epi &epi, const uint32_t bid) {
    __shared__ float sbuf[kGatherWarps][kLightBuf];
    __shared__ float sred[32];
    __shared__ bool s_last;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (bid < geo.heavy_blocks) {
        // ---- one CTA per chunk of a heavy row
        const uint32_t h = plan.chunk_heavy[bid];
        const uint32_t v = plan.heavy_rows[h];
        const uint32_t first = plan.heavy_first[h];
        const uint32_t nchunks = plan.heavy_first[h + 1] - first;
        const uint32_t rb = off[v], re = off[v + 1];
        const uint32_t cb = rb + (bid - first) * kHeavyChunk;
        const uint32_t ce = min(cb + kHeavyChunk, re);
        Kahan k;
        for (uint32_t j0 = cb + threadIdx.x; j0 < ce; j0 += kGatherThreads * kUnroll) {
            uint32_t u[kUnroll];
#pragma unroll
            for (int q = 0; q < kUnroll; ++q) {
                uint32_t j = j0 + q * kGatherThreads;
                u[q] = j < ce ? term.src_of(j) : 0u;
            }
#pragma unroll
            for (int q = 0; q < kUnroll; ++q) {
                uint32_t j = j0 + q * kGatherThreads;
                if (j < ce) k.add(term.value(j, u[q]));
            }
        }
        float s = block_sum(k.value(), sred);
        if (nchunks == 1) {
            if (threadIdx.x == 0) epi(v, s);
        } else {
            if (threadIdx.x == 0) {
                plan.partials[bid] = s;
                __threadfence();
                unsigned t = atomicAdd(plan.tickets + h, 1u);
                s_last = (t == nchunks - 1);
            }
            __syncthreads();
            if (s_last && threadIdx.x == 0) {
                __threadfence();
                float tot = 0.f;
                for (uint32_t c = 0; c < nchunks; ++c)
                    tot = __fadd_rn(tot, *(volatile float *)(plan.partials + first + c));
                epi(v, tot);
                plan.tickets[h] = 0;  // re-arm for the next launch
            }
        }
    } else if (bid < geo.heavy_blocks + geo.medium_blocks) {
        // ---- one warp per medium row
        uint32_t idx = (bid - geo.heavy_blocks) * kGatherWarps + wid;
        if (idx < plan.n_medium) {
            uint32_t v = plan.medium_rows[idx];
            uint32_t b = off[v], e = off[v + 1];
            Kahan k;
            for (uint32_t j0 = b + lane; j0 < e; j0 += 32 * kUnroll) {
                uint32_t u[kUnroll];
#pragma unroll
                for (int q = 0; q < kUnroll; ++q) {
                    uint32_t j = j0 + q * 32;
                    u[q] = j < e ? term.src_of(j) : 0u;
                }
#pragma unroll
                for (int q = 0; q < kUnroll; ++q) {
                    uint32_t j = j0 + q * 32;
                    if (j < e) k.add(term.value(j, u[q]));
                }
            }
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
        const uint32_t excl = incl - dl;
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        float *buf = sbuf[wid];
        // the group's edges pass through shared memory in windows of kLightBuf;
        // each lane adds its row's part of every window, in edge order
        float s = 0.f;
        for (uint32_t w0 = 0; w0 < total; w0 += kLightBuf) {
            const uint32_t wend = min(w0 + kLightBuf, total);
            for (uint32_t i0 = w0; i0 < wend; i0 += 32 * kUnroll) {
                uint32_t e[kUnroll], u[kUnroll];
#pragma unroll
                for (int q = 0; q < kUnroll; ++q) {
                    uint32_t i = i0 + q * 32 + lane;
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
                    e[q] = bk + (i - pk);
                    u[q] = i < wend ? term.src_of(e[q]) : 0u;
                }
#pragma unroll
                for (int q = 0; q < kUnroll; ++q) {
                    uint32_t i = i0 + q * 32 + lane;
                    if (i < wend) buf[i - w0] = term.value(e[q], u[q]);
                }
            }
            __syncwarp();
            const uint32_t lo = max(excl, w0), hi = min(excl + dl, wend);
            for (uint32_t j = lo; j < hi; ++j) s = __fadd_rn(s, buf[j - w0]);
            __syncwarp();
        }
        if (v < V && d <= kLightMax) epi(v, s);
    }
}

// Work units (heavy chunks, medium warps, light groups) are dealt to a
// resident grid of kGatherBlocksPerSM CTAs per SM in unit order.
constexpr int kGatherBlocksPerSM = 6;

template <class Term, class Epi>
__device__ __forceinline__ void gather_rows_kernel_body(const uint32_t *__restrict__ off, uint32_t V,
                                                        const gbx_gather_plan &plan,
                                                        const GatherGeometry &geo, const Term &term,
                                                        Epi &epi) {
    const uint32_t units = geo.total();
    for (uint32_t bid = blockIdx.x; bid < units; bid += gridDim.x) gather_unit(off, V, plan, geo, term, epi, bid);
    epi.block_finish();
}

inline unsigned gather_grid(const GatherGeometry &geo) {
    const unsigned cap = (unsigned)num_sms() * kGatherBlocksPerSM;
    return geo.total() < cap ? geo.total() : cap;
}

template <class Term, class Epi>
__global__ void __launch_bounds__(kGatherThreads, kGatherBlocksPerSM)
    gather_rows_kernel(const uint32_t *__restrict__ off, uint32_t V, gbx_gather_plan plan,
                       GatherGeometry geo, Term term, Epi epi) {
    gather_rows_kernel_body(off, V, plan, geo, term, epi);
}

template <class Term, class Epi>
inline int launch_gather(const uint32_t *off, uint32_t V, const gbx_gather_plan &plan, Term term,
                         Epi epi, cudaStream_t s) {
    GatherGeometry geo = gather_geometry(plan);
    if (geo.total() == 0) return GBX_OK;
    gather_rows_kernel<Term, Epi><<<gather_grid(geo), kGatherThreads, 0, s>>>(off, V, plan, geo, term, epi);
    GBX_LAUNCH_CHECK();
    return GBX_OK;
}

}  // namespace gbx
