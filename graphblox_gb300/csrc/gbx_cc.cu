// Connected components (the reference's connectedComponentsGraphCSR,
// connectedComponents.c:268-629). Every variant hooks roots high->low only
// and compresses fully, so components[v] is the smallest vertex id of v's
// component -- identical labels to the reference for all three variants.
//
//  1 Afforest (default, :379-535): two neighbour rounds linking v with its
//    r-th neighbour, compress, sample 1024 vertices' labels in one CTA
//    (bitonic sort in shared memory, first most frequent label), then link
//    the remaining edges of every vertex outside that component (plus all
//    in-edges when the inverse CSR is present, as the DIRECTED build does).
//  0 Shiloach-Vishkin sweeps (:293-377): hook on roots, compress, repeat.
//  2 label propagation (:537-629): atomicMin both ways until stable.
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
    return *(const volatile uint32_t *)p;
}

// linkNodes (connectedComponents.c:177-196)
__device__ __forceinline__ void cc_link(uint32_t u, uint32_t v, uint32_t *comp) {
    uint32_t p1 = ld_volatile(comp + u);
    uint32_t p2 = ld_volatile(comp + v);
    for (int guard = 0; p1 != p2 && guard < (1 << 20); ++guard) {
        uint32_t high = p1 > p2 ? p1 : p2;
        uint32_t low = p1 + (p2 - high);
        uint32_t phigh = ld_volatile(comp + high);
        if (phigh == low) break;
        if (phigh == high && atomicCAS(comp + high, high, low) == high) break;
        p1 = ld_volatile(comp + ld_volatile(comp + high));
        p2 = ld_volatile(comp + low);
    }
}

__global__ void cc_init_kernel(uint32_t *comp, uint32_t V) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        comp[v] = v;
}

// compressNodes (connectedComponents.c:199-210)
__global__ void cc_compress_kernel(uint32_t *comp, uint32_t V) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        uint32_t c = comp[v];
        uint32_t cc = ld_volatile(comp + c);
        while (c != cc) {
            c = cc;
            cc = ld_volatile(comp + c);
        }
        comp[v] = c;
    }
}

__global__ void cc_neighbor_round_kernel(const uint32_t *off, const uint32_t *dest, uint32_t *comp,
                                         uint32_t V, uint32_t r) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        uint32_t b = off[v], e = off[v + 1];
        if (b + r < e) cc_link(v, dest[b + r], comp);
    }
}

// most frequent label among `ns` sampled vertices; first maximum in key order
__global__ void __launch_bounds__(1024) cc_sample_kernel(const uint32_t *comp, uint32_t V, uint32_t ns,
                                                         uint64_t seed, uint32_t *out) {
    __shared__ uint32_t key[1024];
    __shared__ uint32_t runlen[1024];
    uint32_t t = threadIdx.x;
    uint64_t x = seed + 0x9E3779B97F4A7C15ull * (t + 1);
    x ^= x >> 30; x *= 0xBF58476D1CE4E5B9ull; x ^= x >> 27; x *= 0x94D049BB133111EBull; x ^= x >> 31;
    key[t] = t < ns ? comp[(uint32_t)(x % V)] : 0xFFFFFFFFu;
    __syncthreads();
    for (uint32_t k = 2; k <= 1024; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            uint32_t p = t ^ j;
            if (p > t) {
                uint32_t a = key[t], b = key[p];
                bool up = (t & k) == 0;
                if ((a > b) == up) { key[t] = b; key[p] = a; }
            }
            __syncthreads();
        }
    }
    // run length at each run start
    uint32_t me = key[t];
    bool start = (t == 0) || key[t - 1] != me;
    uint32_t len = 0;
    if (start && me != 0xFFFFFFFFu) {
        uint32_t j = t;
        while (j < 1024 && key[j] == me) ++j;
        len = j - t;
    }
    runlen[t] = len;
    __syncthreads();
    if (t == 0) {
        uint32_t best = 0, bestc = 0;
        for (uint32_t i = 0; i < 1024; ++i)
            if (runlen[i] > bestc) { bestc = runlen[i]; best = key[i]; }
        *out = best;
    }
}

// Afforest final link: warp per vertex over edges from index `skip_first`.
__global__ void cc_final_link_kernel(const uint32_t *off, const uint32_t *dest, const uint32_t *ioff,
                                     const uint32_t *isrc, uint32_t *comp, uint32_t V,
                                     uint32_t skip_first, const uint32_t *skip_label) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t skip = *skip_label;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = gw; v < V; v += nw) {
        if (ld_volatile(comp + v) == skip) continue;
        uint32_t b = off[v], e = off[v + 1];
        for (uint32_t j = b + skip_first + lane; j < e; j += 32) cc_link(v, dest[j], comp);
        if (ioff) {
            uint32_t ib = ioff[v], ie = ioff[v + 1];
            for (uint32_t j = ib + lane; j < ie; j += 32) cc_link(v, isrc[j], comp);
        }
    }
}

// Shiloach-Vishkin hooking sweep: hook the higher root under the lower one
__global__ void cc_sv_hook_kernel(const uint32_t *off, const uint32_t *dest, uint32_t *comp,
                                  uint32_t V, unsigned *change) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    bool changed = false;
    for (uint32_t v = gw; v < V; v += nw) {
        uint32_t b = off[v], e = off[v + 1];
        for (uint32_t j = b + lane; j < e; j += 32) {
            uint32_t u = dest[j];
            uint32_t cs = ld_volatile(comp + v), cd = ld_volatile(comp + u);
            if (cs == cd) continue;
            uint32_t high = cs > cd ? cs : cd, low = cs + (cd - high);
            if (ld_volatile(comp + high) == high && atomicCAS(comp + high, high, low) == high)
                changed = true;
        }
    }
    if (__any_sync(0xffffffffu, changed) && lane == 0) atomicOr(change, 1u);
}

// label propagation: min label across every edge, both directions
__global__ void cc_lp_kernel(const uint32_t *off, const uint32_t *dest, uint32_t *comp, uint32_t V,
                             unsigned *change) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    bool changed = false;
    for (uint32_t v = gw; v < V; v += nw) {
        uint32_t b = off[v], e = off[v + 1];
        for (uint32_t j = b + lane; j < e; j += 32) {
            uint32_t u = dest[j];
            uint32_t cv = ld_volatile(comp + v), cu = ld_volatile(comp + u);
            if (cv < cu) changed |= atomicMin(comp + u, cv) > cv;
            else if (cu < cv) changed |= atomicMin(comp + v, cu) > cu;
        }
    }
    if (__any_sync(0xffffffffu, changed) && lane == 0) atomicOr(change, 1u);
}

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_cc(gbx_graph *g, int variant, uint32_t *components, uint32_t *iterations,
                      void *stream) {
    clear_error();
    GBX_REQUIRE(g && components, GBX_ERR_INVALID, "graph or components is NULL");
    GBX_REQUIRE(variant >= 0 && variant <= 2, GBX_ERR_INVALID, "variant must be 0, 1 or 2");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    OutArray<uint32_t> out;
    GBX_TRY(out.bind(components, V, s));
    uint32_t *comp = out.d;
    const unsigned grid = std::min<unsigned>(ceil_div(V, 256), (unsigned)num_sms() * 8);
    const unsigned wgrid = std::min<unsigned>(ceil_div((uint64_t)V * 32, 256), (unsigned)num_sms() * 16);
    cc_init_kernel<<<grid, 256, 0, s>>>(comp, V);
    GBX_LAUNCH_CHECK();
    uint32_t iters = 0;
    DevBuf<unsigned> flag;
    GBX_TRY(flag.alloc(2, s));
    if (variant == 1) {
        const uint32_t rounds = 2;
        for (uint32_t r = 0; r < rounds; ++r) {
            cc_neighbor_round_kernel<<<grid, 256, 0, s>>>(g->offsets, g->dest, comp, V, r);
            GBX_LAUNCH_CHECK();
            cc_compress_kernel<<<grid, 256, 0, s>>>(comp, V);
            GBX_LAUNCH_CHECK();
        }
        uint32_t ns = V < 1024 ? V / 2 : 1024;
        if (ns == 0) ns = 1;
        cc_sample_kernel<<<1, 1024, 0, s>>>(comp, V, ns, 27491095ull, flag.p);
        GBX_LAUNCH_CHECK();
        cc_final_link_kernel<<<wgrid, 256, 0, s>>>(g->offsets, g->dest, g->in_offsets, g->in_src,
                                                   comp, V, rounds, flag.p);
        GBX_LAUNCH_CHECK();
        cc_compress_kernel<<<grid, 256, 0, s>>>(comp, V);
        GBX_LAUNCH_CHECK();
        iters = rounds;
    } else {
        const uint32_t cap = V + 2;  // each sweep merges at least one pair of trees
        unsigned h = 1;
        while (h) {
            GBX_REQUIRE(iters < cap, GBX_ERR_ITER_CAP, "CC sweep cap reached");
            GBX_CUDA(cudaMemsetAsync(flag.p, 0, 4, s));
            if (variant == 0) {
                // forward edges hook both endpoints' trees, so in-edges add nothing
                cc_sv_hook_kernel<<<wgrid, 256, 0, s>>>(g->offsets, g->dest, comp, V, flag.p);
                GBX_LAUNCH_CHECK();
                cc_compress_kernel<<<grid, 256, 0, s>>>(comp, V);
            } else {
                cc_lp_kernel<<<wgrid, 256, 0, s>>>(g->offsets, g->dest, comp, V, flag.p);
            }
            GBX_LAUNCH_CHECK();
            GBX_CUDA(cudaMemcpyAsync(&h, flag.p, 4, cudaMemcpyDeviceToHost, s));
            GBX_CUDA(cudaStreamSynchronize(s));
            iters++;
        }
    }
    GBX_TRY(out.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    if (iterations) *iterations = iters;
    return GBX_OK;
}
