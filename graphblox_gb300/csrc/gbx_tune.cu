// Per-graph tuning knobs and the autotuner that sets them.
//
// Knobs (stored on the gbx_graph):
//   bfs_alpha   switch top-down -> bottom-up when the frontier's edges exceed
//               unexplored edges / alpha (the reference fixes 15, BFS.c:374)
//   bfs_beta    stay bottom-up while the frontier exceeds V / beta (18)
//   sssp_delta  bucket width of the near/far schedule
//   pull_heavy_min  in-degree above which the pull engine (PR, SpMV) cuts a
//               row into CTA-sized chunks (rows of 33 up to it get a warp)
// SSSP distances are the same for every setting, and PR/SpMV sums only change
// their FP32 summation order (within the 1e-6 relative L1 bound). BFS levels,
// processed_nodes and iteration are the same for every bfs_alpha / bfs_beta
// when the pull CSR is the inverse of the forward CSR (or the graph is
// symmetric); without an inverse CSR the reference pulls over out-edges, and
// on an asymmetric graph its levels then depend on the direction schedule, so
// gbx_autotune leaves the BFS thresholds at the reference's values there.
// gbx_autotune times candidates on sample sources of the graph itself with
// CUDA events and keeps the fastest.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gbx_internal.cuh"

using namespace gbx;

extern "C" int gbx_graph_set_tuning(gbx_graph *g, const char *key, double value) {
    clear_error();
    GBX_REQUIRE(g && key, GBX_ERR_INVALID, "graph or key is NULL");
    GBX_REQUIRE(value >= 0.0 && value < 4294967296.0, GBX_ERR_INVALID, "value out of range");
    const uint32_t v = (uint32_t)value;
    if (!strcmp(key, "bfs_alpha")) {
        GBX_REQUIRE(v >= 1, GBX_ERR_INVALID, "bfs_alpha must be >= 1");
        g->bfs_alpha = v;
    } else if (!strcmp(key, "bfs_beta")) {
        GBX_REQUIRE(v >= 1, GBX_ERR_INVALID, "bfs_beta must be >= 1");
        g->bfs_beta = v;
    } else if (!strcmp(key, "sssp_delta")) {
        g->sssp_delta = v;
    } else if (!strcmp(key, "pull_heavy_min")) {
        GBX_REQUIRE(v >= 64, GBX_ERR_INVALID, "pull_heavy_min must be >= 64");
        if (v != g->pull_heavy_min) {
            // the pull plans and PageRank's captured loop embed the old classes
            cudaDeviceSynchronize();
            free_plan(g->plan_fwd);
            free_plan(g->plan_inv);
            g->plan_fwd = g->plan_inv = nullptr;
            gbx_free_pr_cache(g->pr_cache);
            g->pr_cache = nullptr;
            g->pull_heavy_min = v;
        }
    } else {
        GBX_REQUIRE(false, GBX_ERR_INVALID, "unknown tuning key '%s'", key);
    }
    return GBX_OK;
}

extern "C" int gbx_graph_get_tuning(const gbx_graph *g, const char *key, double *value) {
    clear_error();
    GBX_REQUIRE(g && key && value, GBX_ERR_INVALID, "NULL argument");
    if (!strcmp(key, "bfs_alpha")) *value = g->bfs_alpha;
    else if (!strcmp(key, "bfs_beta")) *value = g->bfs_beta;
    else if (!strcmp(key, "sssp_delta")) *value = g->sssp_delta;
    else if (!strcmp(key, "pull_heavy_min")) *value = g->pull_heavy_min;
    else GBX_REQUIRE(false, GBX_ERR_INVALID, "unknown tuning key '%s'", key);
    return GBX_OK;
}

namespace {

// sample sources: vertices with out-degree > 0 picked by a fixed hash
int sample_sources(gbx_graph *g, uint32_t n, cudaStream_t s, std::vector<uint32_t> *out) {
    std::vector<uint32_t> deg(g->V);
    GBX_CUDA(cudaMemcpyAsync(deg.data(), g->out_degree, (size_t)g->V * 4, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    uint64_t x = 0x9E3779B97F4A7C15ull;
    for (uint32_t tries = 0; out->size() < n && tries < 64 * n + 1024; ++tries) {
        x ^= x >> 12;
        x ^= x << 25;
        x ^= x >> 27;
        uint32_t v = (uint32_t)((x * 2685821657736338717ull) >> 32) % g->V;
        if (deg[v] > 0) out->push_back(v);
    }
    if (out->empty()) out->push_back(0);
    return GBX_OK;
}

template <class F>
int time_ms(F f, cudaStream_t s, float *ms) {
    cudaEvent_t a, b;
    GBX_CUDA(cudaEventCreate(&a));
    GBX_CUDA(cudaEventCreate(&b));
    GBX_CUDA(cudaEventRecord(a, s));
    int st = f();
    GBX_CUDA(cudaEventRecord(b, s));
    GBX_CUDA(cudaEventSynchronize(b));
    GBX_CUDA(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return st;
}

}  // namespace

extern "C" int gbx_autotune(gbx_graph *g, uint32_t flags, uint32_t num_samples, void *stream) {
    clear_error();
    GBX_REQUIRE(g, GBX_ERR_INVALID, "graph is NULL");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    if (num_samples == 0) num_samples = 4;
    DevBuf<uint32_t> out;
    GBX_TRY(out.alloc(g->V, s));
    if ((flags & 1u) && g->has_inverse()) {
        // a traversal's cost depends strongly on its source, so every
        // candidate runs the same (at least 16) sources, twice, and keeps its
        // faster pass
        std::vector<uint32_t> bsrc;
        GBX_TRY(sample_sources(g, std::max<uint32_t>(num_samples, 16), s, &bsrc));
        const uint32_t cands[] = {4, 15, 64, 256, 1024, 4096};
        float best = 1e30f;
        uint32_t best_a = g->bfs_alpha;
        for (uint32_t c : cands) {
            g->bfs_alpha = c;
            GBX_TRY(gbx_bfs(g, bsrc[0], 2, out.p, nullptr, nullptr, stream));  // warm
            float ms = 1e30f;
            for (int pass = 0; pass < 2; ++pass) {
                float t = 0.f;
                GBX_TRY(time_ms([&]() {
                    for (uint32_t v : bsrc) GBX_TRY(gbx_bfs(g, v, 2, out.p, nullptr, nullptr, stream));
                    return GBX_OK;
                }, s, &t));
                ms = std::min(ms, t);
            }
            if (trace_enabled()) fprintf(stderr, "| autotune bfs_alpha %-4u | %9.3f ms |\n", c, ms);
            if (ms < best) {
                best = ms;
                best_a = c;
            }
        }
        g->bfs_alpha = best_a;
    }
    if (flags & 2u) {
        const uint32_t cands_w[] = {64, 96, 128, 192, 256, 512, 1024, 4096};
        const uint32_t cands_u[] = {1, 2, 4};
        const uint32_t *cands = g->weight ? cands_w : cands_u;
        const int nc = g->weight ? 8 : 3;
        float best = 1e30f;
        uint32_t best_d = g->sssp_delta;
        // as for alpha: the same (at least 16) sources for every candidate,
        // twice, keeping the faster pass
        std::vector<uint32_t> ssrc;
        GBX_TRY(sample_sources(g, std::max<uint32_t>(num_samples, 16), s, &ssrc));
        for (int i = 0; i < nc; ++i) {
            GBX_TRY(gbx_sssp(g, ssrc[0], cands[i], out.p, nullptr, stream));  // warm
            float ms = 1e30f;
            for (int pass = 0; pass < 2; ++pass) {
                float t = 0.f;
                GBX_TRY(time_ms([&]() {
                    for (uint32_t v : ssrc) GBX_TRY(gbx_sssp(g, v, cands[i], out.p, nullptr, stream));
                    return GBX_OK;
                }, s, &t));
                ms = std::min(ms, t);
            }
            if (trace_enabled()) fprintf(stderr, "| autotune sssp_delta %-4u | %9.3f ms |\n", cands[i], ms);
            if (ms < best) {
                best = ms;
                best_d = cands[i];
            }
        }
        g->sssp_delta = best_d;
    }
    if (flags & 4u) {
        // pull-engine row classes, timed on pull PageRank iterations
        const uint32_t cands[] = {1024, 4096, 16384};
        DevBuf<float> ranks;
        GBX_TRY(ranks.alloc(g->V, s));
        float best = 1e30f;
        uint32_t best_h = g->pull_heavy_min;
        for (uint32_t c : cands) {
            GBX_TRY(gbx_graph_set_tuning(g, "pull_heavy_min", c));
            GBX_TRY(gbx_pagerank_pull(g, 5, 0.0, ranks.p, nullptr, stream));  // builds the plan, captures
            float ms = 0.f;
            GBX_TRY(time_ms([&]() { return gbx_pagerank_pull(g, 5, 0.0, ranks.p, nullptr, stream); }, s, &ms));
            if (trace_enabled()) fprintf(stderr, "| autotune pull_heavy_min %-5u | %9.3f ms |\n", c, ms);
            if (ms < best) {
                best = ms;
                best_h = c;
            }
        }
        GBX_TRY(gbx_graph_set_tuning(g, "pull_heavy_min", best_h));
    }
    return GBX_OK;
}
