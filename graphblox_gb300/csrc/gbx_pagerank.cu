// Pull PageRank (the reference's pageRankPullGraphCSR, pageRank.c:245-368).
//
// One fused kernel per iteration: for every vertex v the pull engine sums
// contrib[u] over v's in-edges, and the epilogue computes
//   next = base_pr + damp * sum           (base_pr = 1 - 0.85f, damp = 0.85f)
//   contrib_next[v] = next / outdeg(v)    (0 for dangling vertices)
//   |next - prev| -> FP64 error sum, active count (>= epsilon)
// so the reference's three V-sized passes (contrib, gather, update) become
// one sweep. Ranks and contributions ping-pong between two buffers.
//
// Iterations are launched back to back with no host round trip; iteration
// `it` returns immediately when iteration it-1 left no active vertex, which
// reproduces the reference's early exit (stats->iterations = the index of the
// iteration with no active vertex). A final kernel divides by N (:344-350).
// The loop (state reset, initial ranks, the iterations) is captured once per
// graph and (max_iterations, epsilon) as a CUDA graph on working memory kept
// with the graph, and replayed by every later call: one graph launch and the
// finishing kernel per call.
#include <algorithm>

#include "gbx_gather.cuh"

namespace gbx {

struct PrIterState {
    double err;
    unsigned active;
    unsigned pad;
};

struct PrTerm {
    const uint32_t *__restrict__ src;
    const float *__restrict__ contrib;
    // the in-edge stream is read once per iteration: evict-first, so it does
    // not push the gathered contributions out of L2
    __device__ __forceinline__ uint32_t src_of(uint32_t e) const { return __ldcs(src + e); }
    __device__ __forceinline__ float value(uint32_t, uint32_t u) const { return __ldg(contrib + u); }
};

struct PrEpi {
    const float *__restrict__ r_cur;
    float *__restrict__ r_next;
    float *__restrict__ contrib_next;
    const uint32_t *__restrict__ out_degree;
    PrIterState *state;  // this iteration's slot
    double epsilon;
    double inv_n;
    double err;
    unsigned active;
    bool reduce;  // accumulate the residual and the active count this iteration
    __device__ __forceinline__ void operator()(uint32_t v, float sum) {
        const float damp = 0.85f;
        const float base = 1.0f - 0.85f;
        float next = __fadd_rn(base, __fmul_rn(damp, sum));
        float prev = r_cur[v];
        r_next[v] = next;
        uint32_t d = out_degree[v];
        contrib_next[v] = d ? __fdiv_rn(next, (float)d) : 0.0f;
        if (reduce) {
            double e = (double)fabsf(__fsub_rn(next, prev));
            err += e * inv_n;
            active += (e >= epsilon) ? 1u : 0u;
        }
    }
    __device__ __forceinline__ void block_finish() {
        if (!reduce) return;
        __shared__ double sd[32];
        __shared__ unsigned su[32];
        double te = block_sum(err, sd);
        unsigned ta = block_sum(active, su);
        if (threadIdx.x == 0) {
            if (te != 0.0) atomicAdd(&state->err, te);
            if (ta) atomicAdd(&state->active, ta);
        }
    }
};

__global__ void pr_init_kernel(float *r, float *contrib, const uint32_t *out_degree, uint32_t V) {
    const float base = 1.0f - 0.85f;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        r[v] = base;
        uint32_t d = out_degree[v];
        contrib[v] = d ? __fdiv_rn(base, (float)d) : 0.0f;
    }
}

// Iteration `it`: skip when the previous iteration converged.
template <class Term, class Epi>
__global__ void __launch_bounds__(kGatherThreads, kGatherBlocksPerSM)
    pr_iteration_kernel(const uint32_t *__restrict__ off, uint32_t V, gbx_gather_plan plan,
                        GatherGeometry geo, Term term, Epi epi, const PrIterState *prev) {
    if (prev && prev->active == 0) return;
    gather_rows_kernel_body(off, V, plan, geo, term, epi);
}

// final ranks: pick the buffer holding the last executed iteration
__global__ void pr_finish_kernel(const float *r0, const float *r1, const PrIterState *st,
                                 uint32_t max_it, uint32_t can_stop, uint32_t V, float *out, uint32_t *iters_out,
                                 gbx_pr_result *res_dev) {
    __shared__ uint32_t s_k;
    if (threadIdx.x == 0) {
        uint32_t k = max_it;
        for (uint32_t i = 0; can_stop && i < max_it; ++i)
            if (st[i].active == 0) { k = i; break; }
        s_k = k;
    }
    __syncthreads();
    uint32_t k = s_k;
    uint32_t executed = k < max_it ? k + 1 : max_it;
    const float *r = (executed & 1u) ? r1 : r0;
    const float nf = (float)V;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        out[v] = __fdiv_rn(r[v], nf);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        res_dev->iterations = k;
        uint32_t last = executed ? executed - 1 : 0;
        res_dev->active_last = executed ? (can_stop ? st[last].active : V) : 0;
        res_dev->error_total = executed ? st[last].err : 0.0;
        if (iters_out) *iters_out = k;
    }
}

// Enqueue the iteration loop: state reset, initial ranks, max_it iterations.
static int pr_enqueue_loop(gbx_graph *g, const gbx_gather_plan &plan, uint32_t max_it, double epsilon, float *rbuf,
                           float *cbuf, PrIterState *st, cudaStream_t s, uint32_t *kernels) {
    const uint32_t V = g->V;
    float *r[2] = {rbuf, rbuf + V};
    float *c[2] = {cbuf, cbuf + V};
    GBX_CUDA(cudaMemsetAsync(st, 0, sizeof(PrIterState) * (max_it ? max_it : 1), s));
    const int grid = (int)std::min<uint64_t>((V + 255) / 256, (uint64_t)num_sms() * 8);
    pr_init_kernel<<<grid, 256, 0, s>>>(r[0], c[0], g->out_degree, V);
    GBX_LAUNCH_CHECK();
    const GatherGeometry geo = gather_geometry(plan);
    const double inv_n = 1.0 / (double)V;
    for (uint32_t it = 0; it < max_it; ++it) {
        const int a = it & 1, b = a ^ 1;
        PrTerm term{g->pull_src(), c[a]};
        // with epsilon = 0 every vertex stays active, so only the last
        // iteration's residual (reported as error_total) is reduced
        const bool reduce = epsilon > 0.0 || it + 1 == max_it;
        PrEpi epi{r[a], r[b], c[b], g->out_degree, st + it, epsilon, inv_n, 0.0, 0u, reduce};
        pr_iteration_kernel<PrTerm, PrEpi><<<gather_grid(geo), kGatherThreads, 0, s>>>(
            g->pull_offsets(), V, plan, geo, term, epi, (it && epsilon > 0.0) ? st + it - 1 : nullptr);
        GBX_LAUNCH_CHECK();
    }
    *kernels = 1 + max_it;
    return GBX_OK;
}

}  // namespace gbx

// Per-graph PageRank working memory and the iteration loop captured as a CUDA
// graph (re-captured when max_iterations or epsilon change). Calls on one
// graph object are serialised by the caller, as for every other entry point.
struct gbx_pr_cache {
    float *rbuf = nullptr, *cbuf = nullptr;  // 2V each: ping-pong ranks / contributions
    gbx::PrIterState *st = nullptr;
    gbx_pr_result *res = nullptr;
    uint32_t cap = 0;  // slots in st
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint32_t key_it = 0, kernels = 0;
    double key_eps = -1.0;
};

void gbx_free_pr_cache(gbx_pr_cache *c) {
    if (!c) return;
    if (c->exec) cudaGraphExecDestroy(c->exec);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    cudaFree(c->rbuf);
    cudaFree(c->cbuf);
    cudaFree(c->st);
    cudaFree(c->res);
    delete c;
}

using namespace gbx;

namespace {

int pr_cache(gbx_graph *g, uint32_t max_it, gbx_pr_cache **out) {
    gbx_pr_cache *c = g->pr_cache;
    if (!c) {
        c = new gbx_pr_cache();
        g->pr_cache = c;
        GBX_CUDA(cudaMalloc(&c->rbuf, sizeof(float) * 2 * (size_t)g->V));
        GBX_CUDA(cudaMalloc(&c->cbuf, sizeof(float) * 2 * (size_t)g->V));
        GBX_CUDA(cudaMalloc(&c->res, sizeof(gbx_pr_result)));
        GBX_CUDA(cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    }
    if (c->cap < std::max(max_it, 1u)) {
        if (c->exec) cudaGraphExecDestroy(c->exec);
        c->exec = nullptr;
        cudaFree(c->st);
        c->st = nullptr;
        c->cap = std::max(max_it, 64u);
        GBX_CUDA(cudaMalloc(&c->st, sizeof(PrIterState) * c->cap));
    }
    *out = c;
    return GBX_OK;
}

// (Re)capture the loop on the cache's own stream.
int pr_capture(gbx_graph *g, const gbx_gather_plan &plan, uint32_t max_it, double epsilon, gbx_pr_cache *c) {
    if (c->exec && c->key_it == max_it && c->key_eps == epsilon) return GBX_OK;
    if (c->exec) cudaGraphExecDestroy(c->exec);
    c->exec = nullptr;
    GBX_CUDA(cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
    uint32_t kernels = 0;
    const int st = pr_enqueue_loop(g, plan, max_it, epsilon, c->rbuf, c->cbuf, c->st, c->cap_stream, &kernels);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->cap_stream, &graph);
    if (st != GBX_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    GBX_CUDA(e);
    const cudaError_t ei = cudaGraphInstantiate(&c->exec, graph, 0);
    cudaGraphDestroy(graph);
    GBX_CUDA(ei);
    c->key_it = max_it;
    c->key_eps = epsilon;
    c->kernels = kernels;
    return GBX_OK;
}

}  // namespace

extern "C" int gbx_pagerank_pull(gbx_graph *g, uint32_t max_iterations, double epsilon,
                                 float *ranks, gbx_pr_result *result, void *stream) {
    clear_error();
    GBX_REQUIRE(g && ranks, GBX_ERR_INVALID, "graph or ranks is NULL");
    GBX_REQUIRE(epsilon >= 0.0, GBX_ERR_INVALID, "epsilon must be >= 0");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    gbx_gather_plan *plan = nullptr;
    GBX_TRY(get_pull_plan(g, s, &plan));
    OutArray<float> out;
    GBX_TRY(out.bind(ranks, V, s));
    gbx_pr_cache *c = nullptr;
    GBX_TRY(pr_cache(g, max_iterations, &c));
    GBX_TRY(pr_capture(g, *plan, max_iterations, epsilon, c));
    GBX_CUDA(cudaGraphLaunch(c->exec, s));
    for (uint32_t k = 0; k < c->kernels; ++k) note_launch();
    float *r[2] = {c->rbuf, c->rbuf + V};
    const int grid = (int)std::min<uint64_t>((V + 255) / 256, (uint64_t)num_sms() * 8);
    gbx_pr_result *res = c->res;
    pr_finish_kernel<<<grid, 256, 0, s>>>(r[0], r[1], c->st, max_iterations, epsilon > 0.0 ? 1u : 0u, V, out.d,
                                          nullptr, res);
    GBX_LAUNCH_CHECK();
    GBX_TRY(out.finish(s));
    gbx_pr_result hres;
    GBX_CUDA(cudaMemcpyAsync(&hres, res, sizeof(hres), cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    if (result) *result = hres;
    return GBX_OK;
}
