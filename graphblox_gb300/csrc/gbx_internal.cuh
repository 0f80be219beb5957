// Internal helpers shared by the libgbx translation units: status handling,
// device queries, stream-ordered buffers, host/device pointer staging, warp
// and block reductions, and the device-resident graph object.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <cstdio>

#include "gbx.h"

namespace gbx {

constexpr uint32_t kIdMask = 0x3FFFFFFFu;      // EXTRACT_VALUE mask, reorder.h:21-23
constexpr uint32_t kInfLevel = 0xFFFFFFFFu;    // unvisited BFS level
constexpr uint32_t kSsspInf = 0xFFFFFFFFu / 2; // UINT_MAX/2, SSSP.c:66-67

// ---- status --------------------------------------------------------------
void set_error(const char *fmt, ...);
void clear_error();
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define GBX_CUDA(call)                                                        \
    do {                                                                      \
        cudaError_t gbx_e_ = (call);                                          \
        if (gbx_e_ != cudaSuccess) return ::gbx::cuda_fail(gbx_e_, #call, __FILE__, __LINE__); \
    } while (0)
// counts kernel launches (every launch site is followed by this check)
void note_launch();
#define GBX_LAUNCH_CHECK()         \
    do {                           \
        ::gbx::note_launch();      \
        GBX_CUDA(cudaGetLastError()); \
    } while (0)
#define GBX_TRY(expr)                                                         \
    do {                                                                      \
        int gbx_s_ = (expr);                                                  \
        if (gbx_s_ != GBX_OK) return gbx_s_;                                  \
    } while (0)
#define GBX_REQUIRE(cond, code, ...)                                          \
    do {                                                                      \
        if (!(cond)) {                                                        \
            ::gbx::set_error(__VA_ARGS__);                                    \
            return (code);                                                    \
        }                                                                     \
    } while (0)

// per-step tables on stderr when the environment sets GBX_TRACE (the GPU
// counterpart of the reference's per-iteration printf tables)
bool trace_enabled();

// ---- device ----------------------------------------------------------------
// Make sure a device is usable; caches per-device properties.
int ensure_device();
int num_sms();             // SMs of the current device
size_t l2_bytes();         // L2 size of the current device

// true when p is device (or managed) memory that kernels can read directly
bool is_device_ptr(const void *p);

inline unsigned ceil_div(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }

// ---- stream-ordered device buffer -----------------------------------------
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    int alloc(size_t count, cudaStream_t stream) {
        release();
        s = stream;
        n = count;
        if (count == 0) return GBX_OK;
        cudaError_t e = cudaMallocAsync((void **)&p, count * sizeof(T), stream);
        if (e != cudaSuccess) {
            p = nullptr;
            n = 0;
            (void)cudaGetLastError();
            set_error("device allocation of %zu bytes failed: %s", count * sizeof(T),
                      cudaGetErrorString(e));
            return GBX_ERR_NOMEM;
        }
        return GBX_OK;
    }
    void release() {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        n = 0;
    }
    T *get() const { return p; }
};

// Input array view: device pointer as is, or a staged device copy of host data.
template <typename T>
struct InArray {
    const T *d = nullptr;
    DevBuf<T> owned;
    int bind(const T *src, size_t count, cudaStream_t s) {
        if (src == nullptr || count == 0) {
            d = nullptr;
            return GBX_OK;
        }
        if (is_device_ptr(src)) {
            d = src;
            return GBX_OK;
        }
        GBX_TRY(owned.alloc(count, s));
        GBX_CUDA(cudaMemcpyAsync(owned.p, src, count * sizeof(T), cudaMemcpyHostToDevice, s));
        d = owned.p;
        return GBX_OK;
    }
};

// Output array view: write directly into device memory, or into a device
// buffer copied back to host memory by finish().
template <typename T>
struct OutArray {
    T *d = nullptr;
    T *host = nullptr;
    size_t n = 0;
    DevBuf<T> owned;
    // staging (optional): device memory of count elements to use for a host
    // destination instead of a new allocation; on_device (optional): the
    // caller's classification of dst, to skip a pointer-attribute query
    int bind(T *dst, size_t count, cudaStream_t s, T *staging = nullptr, int on_device = -1) {
        n = count;
        host = nullptr;
        if (dst == nullptr) {
            d = nullptr;
            return GBX_OK;
        }
        if (on_device == 1 || (on_device < 0 && is_device_ptr(dst))) {
            d = dst;
            return GBX_OK;
        }
        host = dst;
        if (staging) {
            d = staging;
            return GBX_OK;
        }
        GBX_TRY(owned.alloc(count ? count : 1, s));
        d = owned.p;
        return GBX_OK;
    }
    int finish(cudaStream_t s) {
        if (host && n) GBX_CUDA(cudaMemcpyAsync(host, d, n * sizeof(T), cudaMemcpyDeviceToHost, s));
        return GBX_OK;
    }
    bool to_host() const { return host != nullptr; }
};

// ---- warp / block reductions -----------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}

// Sum over the block; result valid in thread 0. `sh` holds >= 32 T.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < (unsigned)nw) ? sh[threadIdx.x] : T(0);
    if (wid == 0) v = warp_sum(v);
    return v;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

}  // namespace gbx

// ---- device-resident graph ---------------------------------------------------
struct gbx_gather_plan;  // row classes for the pull engine (gbx_gather.cuh)

struct gbx_graph {
    int device = 0;
    uint32_t V = 0;
    uint32_t E = 0;
    // forward CSR
    uint32_t *offsets = nullptr;     // V+1
    uint32_t *dest = nullptr;        // E
    float *weight = nullptr;         // E or null
    uint32_t *out_degree = nullptr;  // V
    // inverse CSR (in-edges) or null
    uint32_t *in_offsets = nullptr;  // V+1
    uint32_t *in_src = nullptr;      // E
    float *in_weight = nullptr;      // E or null
    uint32_t *in_degree = nullptr;   // V
    // lazily built pull plans (forward / inverse)
    gbx_gather_plan *plan_fwd = nullptr;
    gbx_gather_plan *plan_inv = nullptr;
    uint32_t max_out_degree = 0;
    uint32_t max_in_degree = 0;
    // forward rows hold no repeated neighbour: -1 unknown, 0 no, 1 yes
    int simple_rows = -1;
    // per vertex: number of neighbours with id <= its own (built by TC on demand)
    uint32_t *low_count = nullptr;
    // every edge has its reverse: -1 unknown, 0 no, 1 yes
    int symmetric = -1;
    // every pull-CSR neighbour has out-degree > 0 (true for an inverse CSR of
    // the same edges, and for symmetric graphs): -1 unknown, 0 no, 1 yes
    int pull_sources_live = -1;
    // BFS: bit v set when v has pull in-edges (built on first use, gbx_bfs.cu)
    uint32_t *bu_live = nullptr;
    // tuning (gbx_graph_set_tuning / gbx_autotune): BFS direction switch and
    // SSSP bucket width (0 = default for the graph's weights)
    uint32_t bfs_alpha = 15, bfs_beta = 18;
    uint32_t sssp_delta = 0;
    // pull engine (PR, SpMV): in-degree above which a row is cut into
    // CTA-sized chunks; rows between 32 and it get a warp each
    uint32_t pull_heavy_min = 4096;
    // triangle-count work decomposition (gbx_tc.cu)
    struct gbx_tc_plan *tc_plan = nullptr;
    // personalised PageRank: in-edge order and chunk tables (gbx_ppr.cu)
    struct gbx_ppr_cache *ppr = nullptr;
    // multi-source BFS: heavy pull-row chunks (gbx_msbfs.cu)
    struct gbx_ms_plan *ms_plan = nullptr;
    // PageRank working memory and captured iteration loop (gbx_pagerank.cu)
    struct gbx_pr_cache *pr_cache = nullptr;
    // betweenness centrality: successor CSR with ascending rows (gbx_bc.cu)
    struct gbx_bc_cache *bc_cache = nullptr;
    // device scratch lent to one synchronous call at a time (gbx::Scratch)
    char *arena = nullptr;
    size_t arena_bytes = 0;
    int arena_busy = 0;

    bool has_inverse() const { return in_offsets != nullptr; }
    // CSR used by pull-direction kernels (reference: inverse when DIRECTED)
    const uint32_t *pull_offsets() const { return in_offsets ? in_offsets : offsets; }
    const uint32_t *pull_src() const { return in_offsets ? in_src : dest; }
    const float *pull_weight() const { return in_offsets ? in_weight : weight; }
    const uint32_t *pull_degree() const { return in_offsets ? in_degree : out_degree; }
};

void gbx_free_tc_plan(struct gbx_tc_plan *p);
void gbx_free_ppr_cache(struct gbx_ppr_cache *c);
void gbx_free_ms_plan(struct gbx_ms_plan *p);
void gbx_free_pr_cache(struct gbx_pr_cache *c);
void gbx_free_bc_cache(struct gbx_bc_cache *c);

namespace gbx {
// Long-lived device arrays (a graph's arrays, scratch arena and plans) come
// from the device's stream-ordered pool, which keeps the memory of a freed
// graph for the next one instead of handing it back to the CUDA driver (a
// cudaMalloc/cudaFree of gigabytes costs milliseconds). dev_alloc orders the
// allocation on stream s; dev_free is for memory no stream uses any more
// (its callers synchronized first) and accepts nullptr.
int dev_alloc(void **p, size_t bytes, cudaStream_t s);
void dev_free(void *p);

// Device scratch for one synchronous call: carved from the graph's arena
// (grown on demand, kept between calls), or from a single stream-ordered
// allocation when another call holds the arena. The holder's stream is
// synchronized before the arena is handed back.
struct Scratch {
    char *base = nullptr;
    size_t used = 0, cap = 0;
    gbx_graph *held = nullptr;
    cudaStream_t stream = nullptr;
    DevBuf<char> own;
    Scratch() = default;
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;
    static size_t round_up(size_t b) { return (b + 255) & ~size_t(255); }
    int take(gbx_graph *g, size_t bytes, cudaStream_t s) {
        stream = s;
        cap = bytes;
        if (__atomic_exchange_n(&g->arena_busy, 1, __ATOMIC_ACQ_REL) == 0) {
            held = g;
            if (g->arena_bytes < bytes) {
                dev_free(g->arena);  // idle: every holder synchronized before release
                g->arena = nullptr;
                g->arena_bytes = 0;
                void *p = nullptr;
                if (dev_alloc(&p, bytes, s) != GBX_OK) {
                    __atomic_store_n(&g->arena_busy, 0, __ATOMIC_RELEASE);
                    held = nullptr;
                    return GBX_ERR_NOMEM;
                }
                g->arena = static_cast<char *>(p);
                g->arena_bytes = bytes;
            }
            base = g->arena;
            return GBX_OK;
        }
        GBX_TRY(own.alloc(bytes, s));
        base = own.p;
        return GBX_OK;
    }
    // next count elements of T (256-byte aligned); the caller sized take()
    // with round_up() of every carve
    template <typename T>
    T *carve(size_t count) {
        T *p = reinterpret_cast<T *>(base + used);
        used += round_up(count * sizeof(T));
        return used <= cap ? p : nullptr;
    }
    ~Scratch() {
        if (held) {
            cudaStreamSynchronize(stream);
            __atomic_store_n(&held->arena_busy, 0, __ATOMIC_RELEASE);
        }
    }
};

// plan for the pull CSR of g (built on first use, cached on the graph)
int get_pull_plan(gbx_graph *g, cudaStream_t s, gbx_gather_plan **plan);
void free_plan(gbx_gather_plan *p);
// device-wide exclusive scans (gbx_scan.cu); temp storage is internal
int exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, cudaStream_t s,
                       uint32_t *total_dev /* may be null */);
int exclusive_scan_u64(const uint32_t *in, uint64_t *out, uint32_t n, cudaStream_t s);
// stable LSD radix sort of (key, value) pairs on `bits` low key bits (gbx_sort.cu)
int radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t n, int bits, cudaStream_t s);
}  // namespace gbx
