// Chung-Lu power-law graphs with local windows, generated on the device (no
// reference counterpart: the reference reads edge lists from files).
//
// Vertex i has weight w_i = (i + i0)^(-1/(gamma-1)), scaled so the weights
// sum to the edge count; i0 is chosen on the host so the largest expected
// degree is about sqrt(E) (the structural cut-off). Edge e draws, from a
// counter-based stream keyed by (seed, e):
//   source       ~ w (Walker/Vose alias table: one uniform index + one coin)
//   destination  with probability local_fraction: uniform inside the
//                source's window of `window` consecutive ids; otherwise ~ w.
// So out-degrees follow a power law with exponent gamma and mean E/V, and
// local_fraction of the edges stay inside window-aligned id blocks. The
// output depends only on (V, E, gamma, window, local_fraction, seed).
#include <algorithm>
#include <cmath>
#include <vector>

#include "gbx_internal.cuh"

namespace gbx {

__host__ __device__ __forceinline__ uint64_t cl_mix64(uint64_t z) {
    // splitmix64 finaliser (Steele, Lea, Flood 2014)
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint32_t cl_below(uint64_t r, uint32_t n) {
    // uniform in [0, n) from the high 32 bits of r (multiply-shift)
    return (uint32_t)(((r >> 32) * (uint64_t)n) >> 32);
}

__device__ __forceinline__ uint32_t cl_alias(const float *__restrict__ prob, const uint32_t *__restrict__ alias,
                                             uint32_t V, uint64_t r) {
    const uint32_t i = cl_below(r, V);
    const float coin = (float)(uint32_t)(r & 0xFFFFFFu) * (1.0f / 16777216.0f);
    return coin < __ldg(prob + i) ? i : __ldg(alias + i);
}

__global__ void chung_lu_kernel(const float *__restrict__ prob, const uint32_t *__restrict__ alias, uint32_t V,
                                uint64_t E, uint32_t window, uint32_t local_thr, uint64_t key, uint32_t *src,
                                uint32_t *dst) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) {
        uint64_t x = key ^ (e * 0x9E3779B97F4A7C15ull);
        const uint64_t r0 = cl_mix64(x += 0x9E3779B97F4A7C15ull);
        const uint64_t r1 = cl_mix64(x += 0x9E3779B97F4A7C15ull);
        const uint64_t r2 = cl_mix64(x += 0x9E3779B97F4A7C15ull);
        const uint32_t s = cl_alias(prob, alias, V, r0);
        uint32_t d;
        if ((uint32_t)(r1 & 0xFFFFFFFFu) < local_thr) {
            const uint32_t base = s - s % window;
            d = base + cl_below(r2, min(window, V - base));
        } else {
            d = cl_alias(prob, alias, V, r2);
        }
        src[e] = s;
        dst[e] = d;
    }
}

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_generate_chung_lu(uint32_t num_vertices, uint64_t num_edges, double exponent, uint32_t window,
                                     double local_fraction, uint64_t seed, uint32_t *src, uint32_t *dst,
                                     void *stream) {
    clear_error();
    GBX_REQUIRE(src && dst, GBX_ERR_INVALID, "src or dst is NULL");
    GBX_REQUIRE(num_vertices >= 2 && num_vertices <= (1u << 30), GBX_ERR_INVALID, "num_vertices must be 2..2^30");
    GBX_REQUIRE(exponent > 2.0 && exponent < 10.0, GBX_ERR_INVALID, "exponent must be in (2, 10)");
    GBX_REQUIRE(window >= 1, GBX_ERR_INVALID, "window must be >= 1");
    GBX_REQUIRE(local_fraction >= 0.0 && local_fraction <= 1.0, GBX_ERR_INVALID, "local_fraction must be in [0, 1]");
    GBX_REQUIRE(num_edges < (1ull << 32), GBX_ERR_INVALID, "num_edges must be below 2^32");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = num_vertices;
    const double beta = 1.0 / (exponent - 1.0);
    const double E = (double)num_edges;
    // i0: largest expected degree about sqrt(E)
    auto max_weight = [&](double i0) {
        double sum = 0.0;
        for (uint32_t i = 0; i < V; i += std::max(1u, V / 65536)) sum += std::pow(i + i0, -beta) * std::max(1u, V / 65536);
        return E * std::pow(i0, -beta) / sum;
    };
    double lo = 1.0, hi = (double)V;
    const double target = std::max(2.0, std::sqrt(E));
    for (int it = 0; it < 60; ++it) {
        const double mid = std::sqrt(lo * hi);
        if (max_weight(mid) > target) lo = mid; else hi = mid;
    }
    const double i0 = hi;
    // Vose alias table over w_i / mean
    std::vector<double> p(V);
    double sum = 0.0;
    for (uint32_t i = 0; i < V; ++i) sum += (p[i] = std::pow(i + i0, -beta));
    for (uint32_t i = 0; i < V; ++i) p[i] = p[i] * V / sum;
    std::vector<float> prob(V);
    std::vector<uint32_t> alias(V);
    std::vector<uint32_t> small, large;
    small.reserve(V);
    large.reserve(V);
    for (uint32_t i = 0; i < V; ++i) (p[i] < 1.0 ? small : large).push_back(i);
    while (!small.empty() && !large.empty()) {
        const uint32_t l = small.back(), g = large.back();
        small.pop_back();
        prob[l] = (float)p[l];
        alias[l] = g;
        p[g] = (p[g] + p[l]) - 1.0;
        if (p[g] < 1.0) {
            large.pop_back();
            small.push_back(g);
        }
    }
    for (uint32_t i : large) { prob[i] = 1.0f; alias[i] = i; }
    for (uint32_t i : small) { prob[i] = 1.0f; alias[i] = i; }
    DevBuf<float> dprob;
    DevBuf<uint32_t> dalias;
    GBX_TRY(dprob.alloc(V, s));
    GBX_TRY(dalias.alloc(V, s));
    GBX_CUDA(cudaMemcpyAsync(dprob.p, prob.data(), 4 * (size_t)V, cudaMemcpyHostToDevice, s));
    GBX_CUDA(cudaMemcpyAsync(dalias.p, alias.data(), 4 * (size_t)V, cudaMemcpyHostToDevice, s));
    OutArray<uint32_t> os, od;
    GBX_TRY(os.bind(src, num_edges, s));
    GBX_TRY(od.bind(dst, num_edges, s));
    const uint32_t local_thr = (uint32_t)std::min(4294967295.0, std::floor(local_fraction * 4294967296.0));
    const uint64_t key = cl_mix64(seed * 0xD1B54A32D192ED03ull + 0x9E3779B97F4A7C15ull);
    if (num_edges) {
        chung_lu_kernel<<<(unsigned)num_sms() * 8, 256, 0, s>>>(dprob.p, dalias.p, V, num_edges, window, local_thr,
                                                                key, os.d, od.d);
        GBX_LAUNCH_CHECK();
    }
    GBX_TRY(os.finish(s));
    GBX_TRY(od.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}
