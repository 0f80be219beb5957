// Pull PageRank in FP64: the reference's recurrence (pageRankPullGraphCSR,
// pageRank.c:245-368 -- ranks start at 1 - 0.85f, dangling mass dropped,
// final ranks divided by N) evaluated in double precision for exactly the
// requested number of iterations. It is the yardstick the FP32 results of
// gbx_pagerank_pull are measured against on graphs too large for a CPU
// restatement to run beside the benchmark (1.2e9 edges); it is not a faster
// or alternative PageRank.
//
// Each iteration is edge-parallel, so no row, however long, lands on one
// thread: a warp takes 8,192 consecutive pull edges, each lane 256 of them;
// a lane finds the row of its first edge by binary search over the offsets
// and walks its edges in order, summing contrib[src] in FP64 and adding the
// row's partial sum into sums[row] (FP64 atomics) whenever the row changes.
// An epilogue forms the new ranks and contributions and clears the sums.
// The atomics make the order of the partial sums of a split row vary from
// run to run, which moves a rank by a few FP64 ulps at most.
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {
namespace {

constexpr uint32_t kF64LaneEdges = 256;
constexpr uint32_t kF64WarpEdges = 32 * kF64LaneEdges;

// The FP32 recurrence's constants (0.85f and 1 - 0.85f, as the reference
// defines them), held exactly in FP64, so that the difference to the FP32
// ranks measures arithmetic rounding only.
__device__ __forceinline__ double f64_damp() { return (double)0.85f; }
__device__ __forceinline__ double f64_base() { return (double)(1.0f - 0.85f); }

__global__ void f64_init_kernel(const uint32_t *outdeg, uint32_t V, double *rank, double *contrib, double *sums) {
    const double base = f64_base();
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        rank[v] = base;
        const uint32_t d = outdeg[v];
        contrib[v] = d ? base / (double)d : 0.0;
        sums[v] = 0.0;
    }
}

__global__ void f64_gather_kernel(const uint32_t *__restrict__ poff, const uint32_t *__restrict__ psrc, uint32_t V,
                                  uint32_t E, const double *__restrict__ contrib, double *sums) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint64_t c0 = (uint64_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kF64WarpEdges; c0 < E;
         c0 += (uint64_t)nw * kF64WarpEdges) {
        const uint64_t j0 = c0 + (uint64_t)lane * kF64LaneEdges;
        if (j0 >= E) continue;
        const uint32_t j1 = (uint32_t)std::min<uint64_t>(j0 + kF64LaneEdges, E);
        uint32_t j = (uint32_t)j0;
        // last row r with poff[r] <= j (poff[0] = 0 <= j < E = poff[V])
        uint32_t lo = 0, hi = V - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (__ldg(poff + mid) <= j) lo = mid; else hi = mid - 1;
        }
        uint32_t r = lo, rend = __ldg(poff + r + 1);
        double acc = 0.0;
        for (; j < j1; ++j) {
            while (j >= rend) {  // rows that end before j (empty ones included)
                if (acc != 0.0) atomicAdd(sums + r, acc);
                acc = 0.0;
                ++r;
                rend = __ldg(poff + r + 1);
            }
            acc += __ldg(contrib + __ldg(psrc + j));
        }
        if (acc != 0.0) atomicAdd(sums + r, acc);
    }
}

__global__ void f64_update_kernel(const uint32_t *outdeg, uint32_t V, double *rank, double *contrib, double *sums) {
    const double damp = f64_damp(), base = f64_base();
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const double next = base + damp * sums[v];
        sums[v] = 0.0;
        rank[v] = next;
        const uint32_t d = outdeg[v];
        contrib[v] = d ? next / (double)d : 0.0;
    }
}

__global__ void f64_finish_kernel(const double *rank, uint32_t V, double *out) {
    const double n = (double)V;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) out[v] = rank[v] / n;
}

}  // namespace
}  // namespace gbx

using namespace gbx;

extern "C" int gbx_pagerank_pull_fp64(gbx_graph *g, uint32_t iterations, double *ranks, void *stream) {
    clear_error();
    GBX_REQUIRE(g, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(ranks, GBX_ERR_INVALID, "ranks is NULL");
    GBX_REQUIRE(g->V > 0, GBX_ERR_INVALID, "graph has no vertices");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V, E = g->E;
    DevBuf<double> rank, contrib, sums;
    GBX_TRY(rank.alloc(V, s));
    GBX_TRY(contrib.alloc(V, s));
    GBX_TRY(sums.alloc(V, s));
    OutArray<double> out;
    GBX_TRY(out.bind(ranks, V, s));
    const unsigned grid = std::min<unsigned>(ceil_div(V, 256), (unsigned)num_sms() * 8);
    f64_init_kernel<<<grid, 256, 0, s>>>(g->out_degree, V, rank.p, contrib.p, sums.p);
    GBX_LAUNCH_CHECK();
    const unsigned ggrid =
        std::min<unsigned>(ceil_div(ceil_div((uint64_t)E, kF64WarpEdges), 8), (unsigned)num_sms() * 16);
    for (uint32_t it = 0; it < iterations; ++it) {
        if (E) {
            f64_gather_kernel<<<std::max(ggrid, 1u), 256, 0, s>>>(g->pull_offsets(), g->pull_src(), V, E,
                                                                  contrib.p, sums.p);
            GBX_LAUNCH_CHECK();
        }
        f64_update_kernel<<<grid, 256, 0, s>>>(g->out_degree, V, rank.p, contrib.p, sums.p);
        GBX_LAUNCH_CHECK();
    }
    f64_finish_kernel<<<grid, 256, 0, s>>>(rank.p, V, out.d);
    GBX_LAUNCH_CHECK();
    GBX_TRY(out.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}
