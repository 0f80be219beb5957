// Pull PageRank for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: hosts whose own allocator has taken
// all device memory at start-up (a serving process or a framework's caching
// pool), and real-time hosts that must not grow the CUDA heap once they are
// running, since an allocation may block or fail at any time there.
// gbx_pagerank_pull allocates its working buffers (stream-ordered) and builds
// a per-graph degree plan; this variant allocates nothing. Its working memory
// is one file-scope __device__ array, g_pr_scratch, sized for graphs of at
// most kNoAllocMaxVertices vertices and kNoAllocMaxIterations iterations
// (about 64 MiB, held by every GPU that loads the library until the process
// exits). The caller passes the pull CSR, the out-degrees and the output, all
// in device memory.
//
// In host code the name g_pr_scratch is only a host-side stand-in for the
// device array; its device address is looked up with cudaGetSymbolAddress
// once per device, on the first call made with that device current (a lookup
// that failed is retried by the next call), so that first call does the
// set-up. Every call reuses the same array and keeps the previous call's
// contents; the iteration counters are cleared at the start of each call. Calls that overlap on the
// GPU (two streams, or two host threads) race on the array: serialise them.
// With a non-NULL result the call copies the result to the host and
// synchronises the stream before it returns.
//
// The computation is the reference's pageRankPullGraphCSR recurrence
// (pageRank.c:245-368), as in gbx_pagerank_pull, with a plan-free row mapping:
// each warp owns 32 consecutive rows; rows of up to 32 edges go through a
// shared-memory window, longer rows are summed by the whole warp in turn.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "gbx_internal.cuh"

namespace gbx {
namespace {

constexpr uint32_t kNoAllocMaxVertices = 1u << 22;  // 4,194,304
constexpr uint32_t kNoAllocMaxIterations = 1024;
constexpr int kNaThreads = 256;
constexpr int kNaWarps = kNaThreads / 32;
constexpr uint32_t kNaWindow = 256;

struct NaIter {
    double err;
    unsigned active;
    unsigned pad;
};

struct NaScratch {
    float r[2][kNoAllocMaxVertices];
    float c[2][kNoAllocMaxVertices];
    NaIter it[kNoAllocMaxIterations];
    gbx_pr_result res;
};

static __device__ __align__(256) NaScratch g_pr_scratch;

// Device address of g_pr_scratch per device; only a successful lookup is kept.
static std::mutex g_na_mutex;
static NaScratch *g_na_ptr[64] = {};

__device__ __forceinline__ float na_warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void na_init_kernel(NaScratch *sc, const uint32_t *outdeg, uint32_t V, uint32_t n_it) {
    const float base = 1.0f - 0.85f;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        sc->r[0][v] = base;
        uint32_t d = outdeg[v];
        sc->c[0][v] = d ? __fdiv_rn(base, (float)d) : 0.0f;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_it; i += gridDim.x * blockDim.x) {
        sc->it[i].err = 0.0;
        sc->it[i].active = 0;
    }
}

__global__ void __launch_bounds__(kNaThreads)
    na_iteration_kernel(NaScratch *sc, const uint32_t *__restrict__ off, const uint32_t *__restrict__ src,
                        const uint32_t *__restrict__ outdeg, uint32_t V, uint32_t it, double epsilon,
                        int check_prev, int reduce) {
    __shared__ float win[kNaWarps][kNaWindow];
    __shared__ double s_err[kNaWarps];
    __shared__ unsigned s_act[kNaWarps];
    if (check_prev && sc->it[it - 1].active == 0) return;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t a = it & 1, b = a ^ 1;
    const float *contrib = sc->c[a];
    const float damp = 0.85f, base = 1.0f - 0.85f;
    const double inv_n = 1.0 / (double)V;
    double err = 0.0;
    unsigned active = 0;
    const uint32_t groups = (V + 31) / 32;
    for (uint32_t g = blockIdx.x * kNaWarps + wid; g < groups; g += gridDim.x * kNaWarps) {
        const uint32_t v = g * 32 + lane;
        uint32_t rb = 0, d = 0;
        if (v < V) {
            rb = off[v];
            d = off[v + 1] - rb;
        }
        const uint32_t dl = d <= 32 ? d : 0;
        uint32_t incl = dl;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += t;
        }
        const uint32_t excl = incl - dl, total = __shfl_sync(0xffffffffu, incl, 31);
        float s = 0.f;
        for (uint32_t w0 = 0; w0 < total; w0 += kNaWindow) {
            const uint32_t wend = min(w0 + kNaWindow, total);
            for (uint32_t i0 = w0; i0 < wend; i0 += 32) {
                const uint32_t i = i0 + lane;
                uint32_t k = 0;
#pragma unroll
                for (uint32_t step = 16; step > 0; step >>= 1) {
                    uint32_t cand = k + step;
                    if (__shfl_sync(0xffffffffu, excl, cand) <= i) k = cand;
                }
                const uint32_t pk = __shfl_sync(0xffffffffu, excl, k);
                const uint32_t bk = __shfl_sync(0xffffffffu, rb, k);
                if (i < wend) win[wid][i - w0] = __ldg(contrib + __ldg(src + bk + (i - pk)));
            }
            __syncwarp();
            const uint32_t lo = max(excl, w0), hi = min(excl + dl, wend);
            for (uint32_t j = lo; j < hi; ++j) s = __fadd_rn(s, win[wid][j - w0]);
            __syncwarp();
        }
        // rows longer than 32 edges: the whole warp, one row at a time
        unsigned longs = __ballot_sync(0xffffffffu, d > 32);
        while (longs) {
            const uint32_t owner = __ffs(longs) - 1;
            longs &= longs - 1;
            const uint32_t ob = __shfl_sync(0xffffffffu, rb, owner);
            const uint32_t od = __shfl_sync(0xffffffffu, d, owner);
            float part = 0.f, comp = 0.f;  // Kahan
            for (uint32_t j = lane; j < od; j += 32) {
                float y = __fsub_rn(__ldg(contrib + __ldg(src + ob + j)), comp);
                float t = __fadd_rn(part, y);
                comp = __fsub_rn(__fsub_rn(t, part), y);
                part = t;
            }
            const float tot = na_warp_sum(part);
            if (lane == owner) s = tot;
        }
        if (v < V) {
            const float next = __fadd_rn(base, __fmul_rn(damp, s));
            const float prev = sc->r[a][v];
            sc->r[b][v] = next;
            const uint32_t od = outdeg[v];
            sc->c[b][v] = od ? __fdiv_rn(next, (float)od) : 0.0f;
            if (reduce) {
                const double e = (double)fabsf(__fsub_rn(next, prev));
                err += e * inv_n;
                active += (e >= epsilon) ? 1u : 0u;
            }
        }
    }
    if (!reduce) return;
    for (int o = 16; o > 0; o >>= 1) {
        err += __shfl_xor_sync(0xffffffffu, err, o);
        active += __shfl_xor_sync(0xffffffffu, active, o);
    }
    if (lane == 0) {
        s_err[wid] = err;
        s_act[wid] = active;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double te = 0.0;
        unsigned ta = 0;
        for (int w = 0; w < kNaWarps; ++w) {
            te += s_err[w];
            ta += s_act[w];
        }
        if (te != 0.0) atomicAdd(&sc->it[it].err, te);
        if (ta) atomicAdd(&sc->it[it].active, ta);
    }
}

__global__ void na_finish_kernel(NaScratch *sc, uint32_t max_it, uint32_t can_stop, uint32_t V, float *out) {
    __shared__ uint32_t s_k;
    if (threadIdx.x == 0) {
        uint32_t k = max_it;
        for (uint32_t i = 0; can_stop && i < max_it; ++i)
            if (sc->it[i].active == 0) { k = i; break; }
        s_k = k;
    }
    __syncthreads();
    const uint32_t k = s_k;
    const uint32_t executed = k < max_it ? k + 1 : max_it;
    const float *r = sc->r[executed & 1u];
    const float nf = (float)V;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        out[v] = __fdiv_rn(r[v], nf);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint32_t last = executed ? executed - 1 : 0;
        sc->res.iterations = k;
        sc->res.active_last = executed ? (can_stop ? sc->it[last].active : V) : 0;
        sc->res.error_total = executed ? sc->it[last].err : 0.0;
    }
}

// Device address of g_pr_scratch on the current device (set-up on first use;
// a failed lookup leaves the slot empty, so a later call tries again).
int scratch_for_current_device(NaScratch **out) {
    int dev = 0;
    GBX_CUDA(cudaGetDevice(&dev));
    GBX_REQUIRE(dev >= 0 && dev < 64, GBX_ERR_INVALID, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_pr_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_pr_scratch)", __FILE__, __LINE__);
        GBX_REQUIRE(p != nullptr, GBX_ERR_CUDA, "no device address for the PageRank scratch array");
        g_na_ptr[dev] = (NaScratch *)p;
    }
    *out = g_na_ptr[dev];
    return GBX_OK;
}

}  // namespace
}  // namespace gbx

using namespace gbx;

extern "C" int gbx_pagerank_pull_noalloc(uint32_t num_vertices, const uint32_t *pull_offsets,
                                         const uint32_t *pull_src, const uint32_t *out_degree,
                                         uint32_t max_iterations, double epsilon, float *ranks,
                                         gbx_pr_result *result, void *stream) {
    clear_error();
    GBX_REQUIRE(num_vertices > 0, GBX_ERR_INVALID, "num_vertices must be > 0");
    GBX_REQUIRE(num_vertices <= kNoAllocMaxVertices, GBX_ERR_INVALID,
                "gbx_pagerank_pull_noalloc handles at most %u vertices (got %u); use gbx_pagerank_pull",
                kNoAllocMaxVertices, num_vertices);
    GBX_REQUIRE(max_iterations <= kNoAllocMaxIterations, GBX_ERR_INVALID,
                "gbx_pagerank_pull_noalloc runs at most %u iterations (got %u)", kNoAllocMaxIterations,
                max_iterations);
    GBX_REQUIRE(epsilon >= 0.0, GBX_ERR_INVALID, "epsilon must be >= 0");
    GBX_REQUIRE(pull_offsets && pull_src && out_degree && ranks, GBX_ERR_INVALID, "NULL array argument");
    GBX_TRY(ensure_device());
    GBX_REQUIRE(is_device_ptr(pull_offsets) && is_device_ptr(pull_src) && is_device_ptr(out_degree) &&
                    is_device_ptr(ranks),
                GBX_ERR_INVALID, "gbx_pagerank_pull_noalloc takes device memory only");
    NaScratch *sc = nullptr;
    GBX_TRY(scratch_for_current_device(&sc));
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = num_vertices;
    const unsigned grid = std::min<unsigned>(ceil_div(V, 256), (unsigned)num_sms() * 8);
    na_init_kernel<<<grid, 256, 0, s>>>(sc, out_degree, V, max_iterations);
    GBX_LAUNCH_CHECK();
    const unsigned igrid = std::min<unsigned>(ceil_div(ceil_div(V, 32), kNaWarps), (unsigned)num_sms() * 8);
    for (uint32_t it = 0; it < max_iterations; ++it) {
        const int reduce = (epsilon > 0.0 || it + 1 == max_iterations) ? 1 : 0;
        const int check_prev = (it > 0 && epsilon > 0.0) ? 1 : 0;
        na_iteration_kernel<<<igrid, kNaThreads, 0, s>>>(sc, pull_offsets, pull_src, out_degree, V, it, epsilon,
                                                         check_prev, reduce);
        GBX_LAUNCH_CHECK();
    }
    na_finish_kernel<<<grid, 256, 0, s>>>(sc, max_iterations, epsilon > 0.0 ? 1u : 0u, V, ranks);
    GBX_LAUNCH_CHECK();
    if (result) {
        GBX_CUDA(cudaMemcpyAsync(result, &sc->res, sizeof(gbx_pr_result), cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
    }
    return GBX_OK;
}
