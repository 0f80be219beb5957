// Library core: status strings and thread-local error messages, device
// queries, pointer classification, and the device-resident graph object
// (the device copy of the reference's struct GraphCSR, graphCSR.h:14-31).
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstring>
#include <mutex>

#include "gbx_internal.cuh"
#include "gbx_gather.cuh"

namespace gbx {

static thread_local char g_err[512] = {0};
static std::atomic<unsigned long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

bool trace_enabled() {
    static const bool on = [] {
        const char *e = getenv("GBX_TRACE");
        return e && *e && strcmp(e, "0") != 0;
    }();
    return on;
}

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

void clear_error() { g_err[0] = 0; }

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    const char *base = strrchr(file, '/');
    set_error("%s:%d: %s failed: %s", base ? base + 1 : file, line, what, cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) {
        (void)cudaGetLastError();
        return GBX_ERR_NOMEM;
    }
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GBX_ERR_NO_DEVICE;
    return GBX_ERR_CUDA;
}

struct DevProps {
    int sms = 0;
    size_t l2 = 0;
};
static DevProps g_props[64];
static std::once_flag g_props_once[64];

int ensure_device() {
    // a device this thread has already checked stays usable for the process
    static thread_local int checked = -1;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess && dev == checked) return GBX_OK;
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        set_error("no usable CUDA device: %s", cudaGetErrorString(e));
        return GBX_ERR_NO_DEVICE;
    }
    int count = 0;
    e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        (void)cudaGetLastError();
        set_error("no usable CUDA device: %s", cudaGetErrorString(e));
        return GBX_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= 64) return GBX_ERR_NO_DEVICE;
    std::call_once(g_props_once[dev], [dev]() {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, dev) == cudaSuccess) {
            g_props[dev].sms = p.multiProcessorCount;
            g_props[dev].l2 = (size_t)p.l2CacheSize;
            // Working buffers come from the device's default stream-ordered
            // pool. With its default release threshold (0) every stream
            // synchronize hands freed blocks back to the CUDA driver, and the next
            // call maps them again (hundreds of MB per BFS on large graphs);
            // keep up to a quarter of device memory (at most 64 GB) cached in
            // this process instead.
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
                uint64_t keep = std::min<uint64_t>((uint64_t)p.totalGlobalMem / 4, 64ull << 30);
                (void)cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            }
            (void)cudaGetLastError();
        } else {
            g_props[dev].sms = 132;
            g_props[dev].l2 = 50u << 20;
        }
    });
    checked = dev;
    return GBX_OK;
}

int num_sms() {
    int dev = 0;
    cudaGetDevice(&dev);
    return g_props[dev].sms > 0 ? g_props[dev].sms : 148;
}

size_t l2_bytes() {
    int dev = 0;
    cudaGetDevice(&dev);
    return g_props[dev].l2;
}

bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// ---- graph construction kernels ----------------------------------------------

__global__ void mask_ids_kernel(uint32_t *ids, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        ids[i] &= kIdMask;
}

// degree[v] = offsets[v+1] - offsets[v]
__global__ void degree_from_offsets_kernel(const uint32_t *off, uint32_t *deg, uint32_t V) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        deg[v] = off[v + 1] - off[v];
}

// The reference layout is edges_idx + out_degree: the edges of v are the run
// ids[edges_idx[v] .. +deg[v]). bad[0] counts vertices whose run does not
// start at the prefix-sum offset (runs out of vertex order, as in the
// inverse CSR the reference sorts on masked ids), bad[2] runs that end past
// the E edges.
__global__ void check_layout_kernel(const uint32_t *edges_idx, const uint32_t *deg,
                                    const uint32_t *off, uint32_t V, uint32_t E, unsigned *bad) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        if (!deg[v]) continue;
        if (edges_idx[v] != off[v]) atomicAdd(bad, 1u);
        if ((uint64_t)edges_idx[v] + deg[v] > E) atomicAdd(bad + 2, 1u);
    }
}

// Moves every run to its prefix-sum position, keeping the order inside the
// run (one warp per vertex; runs checked in bounds by check_layout_kernel).
__global__ void repack_runs_kernel(const uint32_t *edges_idx, const uint32_t *deg,
                                   const uint32_t *off, uint32_t V, const uint32_t *ids,
                                   const float *w, uint32_t *ids_out, float *w_out) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < V; v += warps) {
        const uint32_t n = deg[v], from = edges_idx[v], to = off[v];
        for (uint32_t k = lane; k < n; k += 32) {
            ids_out[to + k] = ids[from + k];
            if (w) w_out[to + k] = w[from + k];
        }
    }
}

__global__ void check_offsets_kernel(const uint32_t *off, uint32_t V, uint32_t E, unsigned *bad) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        if (off[v] > off[v + 1]) atomicAdd(bad, 1u);
    if (blockIdx.x == 0 && threadIdx.x == 0 && (off[0] != 0 || off[V] != E)) atomicAdd(bad, 1u);
}

__global__ void max_u32_kernel(const uint32_t *a, uint32_t n, uint32_t *out) {
    uint32_t m = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        m = max(m, a[i]);
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

static int grid_for(uint64_t n, int threads = 256) {
    uint64_t b = (n + threads - 1) / threads;
    uint64_t cap = (uint64_t)num_sms() * 8;
    if (b > cap) b = cap;
    return (int)(b ? b : 1);
}

static int copy_in(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    if (!bytes) return GBX_OK;
    cudaMemcpyKind k = is_device_ptr(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    GBX_CUDA(cudaMemcpyAsync(dst, src, bytes, k, s));
    return GBX_OK;
}

int dev_alloc(void **p, size_t bytes, cudaStream_t s) {
    *p = nullptr;
    cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 4, s);
    if (e == cudaErrorMemoryAllocation) {
        // memory the pool keeps from freed graphs goes back to the CUDA driver
        // first, then the allocation is tried once more
        (void)cudaGetLastError();
        int dev = 0;
        cudaMemPool_t pool;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            cudaDeviceSynchronize();
            cudaMemPoolTrimTo(pool, 0);
        }
        e = cudaMallocAsync(p, bytes ? bytes : 4, s);
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        *p = nullptr;
        set_error("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return GBX_ERR_NOMEM;
    }
    return GBX_OK;
}

void dev_free(void *p) {
    if (p) cudaFreeAsync(p, 0);
}

// One direction of a graph (forward or inverse), filled from either layout
// in two passes. fill_stage allocates the arrays and enqueues every copy of
// the caller's arrays; fill_check then runs the validation kernels and their
// host round trips and gathers runs that are out of vertex order. A graph
// stages both directions before it checks either, so its copies follow one
// another over the host link instead of each waiting for a check kernel,
// which may itself wait for SMs that another stream's kernels hold.
struct DirFill {
    uint32_t V = 0, E = 0;
    const uint32_t *edges_idx = nullptr, *degree = nullptr, *offsets = nullptr, *ids = nullptr;
    const float *w = nullptr;
    uint32_t **d_off = nullptr, **d_ids = nullptr, **d_deg = nullptr;
    float **d_w = nullptr;
    uint32_t *max_deg = nullptr;
    InArray<uint32_t> eidx;
    DevBuf<unsigned> bad;  // [0] layout / offset faults, [1] maximum degree, [2] runs past E
    DevBuf<uint32_t> tot;
};

static int fill_stage(DirFill &f, cudaStream_t s) {
    const uint32_t V = f.V, E = f.E;
    GBX_TRY(dev_alloc((void **)f.d_off, (size_t)(V + 1) * 4, s));
    GBX_TRY(dev_alloc((void **)f.d_deg, (size_t)V * 4, s));
    // four ids of zeroed padding: kernels read rows as aligned 16-byte quads
    GBX_TRY(dev_alloc((void **)f.d_ids, ((size_t)E + 4) * 4, s));
    GBX_CUDA(cudaMemsetAsync(*f.d_ids + E, 0, 16, s));
    if (f.w) GBX_TRY(dev_alloc((void **)f.d_w, (size_t)E * 4, s));
    GBX_TRY(f.bad.alloc(3, s));
    GBX_CUDA(cudaMemsetAsync(f.bad.p, 0, 12, s));
    if (f.offsets) {
        GBX_TRY(copy_in(*f.d_off, f.offsets, (size_t)(V + 1) * 4, s));
    } else {
        GBX_TRY(copy_in(*f.d_deg, f.degree, (size_t)V * 4, s));
        GBX_TRY(f.eidx.bind(f.edges_idx, V, s));
    }
    // the edge arrays as given; fill_check gathers them into offset order
    // when the runs turn out not to be in vertex order
    GBX_TRY(copy_in(*f.d_ids, f.ids, (size_t)E * 4, s));
    if (f.w) GBX_TRY(copy_in(*f.d_w, f.w, (size_t)E * 4, s));
    return GBX_OK;
}

static int fill_check(DirFill &f, cudaStream_t s) {
    const uint32_t V = f.V, E = f.E;
    bool repack = false;
    if (f.offsets) {
        check_offsets_kernel<<<grid_for(V), 256, 0, s>>>(*f.d_off, V, E, f.bad.p);
        GBX_LAUNCH_CHECK();
        degree_from_offsets_kernel<<<grid_for(V), 256, 0, s>>>(*f.d_off, *f.d_deg, V);
        GBX_LAUNCH_CHECK();
    } else {
        GBX_TRY(f.tot.alloc(1, s));
        GBX_TRY(exclusive_scan_u32(*f.d_deg, *f.d_off, V, s, f.tot.p));
        GBX_CUDA(cudaMemcpyAsync(*f.d_off + V, f.tot.p, 4, cudaMemcpyDeviceToDevice, s));
        check_layout_kernel<<<grid_for(V), 256, 0, s>>>(f.eidx.d, *f.d_deg, *f.d_off, V, E, f.bad.p);
        GBX_LAUNCH_CHECK();
        uint32_t hv = 0;
        unsigned hl[3] = {0, 0, 0};
        GBX_CUDA(cudaMemcpyAsync(&hv, f.tot.p, 4, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaMemcpyAsync(hl, f.bad.p, 12, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        GBX_REQUIRE(hv == E, GBX_ERR_INVALID, "sum of degrees (%u) != num_edges (%u)", hv, E);
        GBX_REQUIRE(hl[2] == 0, GBX_ERR_INVALID,
                    "%u vertices whose edges_idx + out_degree exceeds num_edges (%u)", hl[2], E);
        repack = hl[0] != 0;
        GBX_CUDA(cudaMemsetAsync(f.bad.p, 0, 4, s));
    }
    if (repack) {
        // runs out of vertex order: gather the copies just made into offset
        // order in new arrays, which then replace them
        uint32_t *ids2 = nullptr;
        float *w2 = nullptr;
        GBX_TRY(dev_alloc((void **)&ids2, ((size_t)E + 4) * 4, s));
        if (f.w && dev_alloc((void **)&w2, (size_t)E * 4, s) != GBX_OK) {
            cudaStreamSynchronize(s);
            dev_free(ids2);
            return GBX_ERR_NOMEM;
        }
        cudaError_t le = cudaMemsetAsync(ids2 + E, 0, 16, s);
        if (le == cudaSuccess) {
            repack_runs_kernel<<<grid_for((uint64_t)V * 32), 256, 0, s>>>(
                f.eidx.d, *f.d_deg, *f.d_off, V, *f.d_ids, f.w ? *f.d_w : nullptr, ids2, w2);
            le = cudaGetLastError();
        }
        cudaStreamSynchronize(s);
        if (le != cudaSuccess) {
            dev_free(ids2);
            dev_free(w2);
            return cuda_fail(le, "repack_runs_kernel", __FILE__, __LINE__);
        }
        note_launch();
        dev_free(*f.d_ids);
        *f.d_ids = ids2;
        if (f.w) {
            dev_free(*f.d_w);
            *f.d_w = w2;
        }
    }
    if (E) {
        mask_ids_kernel<<<grid_for(E), 256, 0, s>>>(*f.d_ids, E);
        GBX_LAUNCH_CHECK();
    }
    max_u32_kernel<<<grid_for(V), 256, 0, s>>>(*f.d_deg, V, f.bad.p + 1);
    GBX_LAUNCH_CHECK();
    unsigned hb[2] = {0, 0};
    GBX_CUDA(cudaMemcpyAsync(hb, f.bad.p, 8, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    GBX_REQUIRE(hb[0] == 0, GBX_ERR_INVALID, "offsets are not non-decreasing from 0 to num_edges");
    *f.max_deg = hb[1];
    return GBX_OK;
}

static int create_common(gbx_graph **out, uint32_t V, uint32_t E, const uint32_t *edges_idx,
                         const uint32_t *deg, const uint32_t *off, const uint32_t *dest,
                         const float *w, const uint32_t *in_idx, const uint32_t *in_deg,
                         const uint32_t *in_off, const uint32_t *in_src, const float *in_w,
                         void *stream) {
    clear_error();
    GBX_REQUIRE(out != nullptr, GBX_ERR_INVALID, "out is NULL");
    *out = nullptr;
    GBX_REQUIRE(V > 0, GBX_ERR_INVALID, "num_vertices must be > 0");
    GBX_REQUIRE(V <= kIdMask + 1u, GBX_ERR_INVALID, "num_vertices exceeds 2^30");
    GBX_REQUIRE((off != nullptr) || (edges_idx != nullptr && deg != nullptr), GBX_ERR_INVALID,
                "forward CSR arrays missing");
    GBX_REQUIRE(E == 0 || dest != nullptr, GBX_ERR_INVALID, "dest is NULL");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    gbx_graph *g = new gbx_graph();
    cudaGetDevice(&g->device);
    g->V = V;
    g->E = E;
    const bool want_inv = (in_off != nullptr) || (in_idx != nullptr && in_deg != nullptr);
    if (want_inv && E && !in_src) {
        delete g;
        set_error("in_src is NULL");
        return GBX_ERR_INVALID;
    }
    DirFill fwd, inv;
    fwd.V = inv.V = V;
    fwd.E = inv.E = E;
    fwd.edges_idx = edges_idx, fwd.degree = deg, fwd.offsets = off, fwd.ids = dest, fwd.w = w;
    fwd.d_off = &g->offsets, fwd.d_ids = &g->dest, fwd.d_w = &g->weight, fwd.d_deg = &g->out_degree;
    fwd.max_deg = &g->max_out_degree;
    inv.edges_idx = in_idx, inv.degree = in_deg, inv.offsets = in_off, inv.ids = in_src, inv.w = in_w;
    inv.d_off = &g->in_offsets, inv.d_ids = &g->in_src, inv.d_w = &g->in_weight, inv.d_deg = &g->in_degree;
    inv.max_deg = &g->max_in_degree;
    int st = fill_stage(fwd, s);
    if (st == GBX_OK && want_inv) st = fill_stage(inv, s);
    if (st == GBX_OK) st = fill_check(fwd, s);
    if (st == GBX_OK && want_inv) st = fill_check(inv, s);
    if (st != GBX_OK) {
        cudaStreamSynchronize(s);  // the stages' copies may still be in flight
        gbx_graph_destroy(g);
        return st;
    }
    *out = g;
    return GBX_OK;
}

}  // namespace gbx

using namespace gbx;

extern "C" {

const char *gbx_status_string(int status) {
    switch (status) {
    case GBX_OK: return "ok";
    case GBX_ERR_INVALID: return "invalid argument";
    case GBX_ERR_CUDA: return "CUDA error";
    case GBX_ERR_NOMEM: return "out of device memory";
    case GBX_ERR_ITER_CAP: return "iteration cap reached";
    case GBX_ERR_NO_DEVICE: return "no usable CUDA device";
    case GBX_ERR_UNSUPPORTED: return "unsupported graph layout";
    case GBX_ERR_DEVICE_TIMEOUT: return "bounded device wait expired";
    default: return "unknown status";
    }
}

const char *gbx_last_error(void) { return g_err; }

const char *gbx_version(void) { return "0.1.0"; }

uint64_t gbx_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int gbx_set_device(int device) {
    clear_error();
    GBX_CUDA(cudaSetDevice(device));
    return ensure_device();
}

int gbx_graph_create_csr(gbx_graph **out, uint32_t num_vertices, uint32_t num_edges,
                         const uint32_t *edges_idx, const uint32_t *out_degree,
                         const uint32_t *dest, const float *weight,
                         const uint32_t *in_edges_idx, const uint32_t *in_degree,
                         const uint32_t *in_src, const float *in_weight, void *stream) {
    GBX_REQUIRE(edges_idx && out_degree, GBX_ERR_INVALID, "edges_idx/out_degree is NULL");
    return create_common(out, num_vertices, num_edges, edges_idx, out_degree, nullptr, dest, weight,
                         in_edges_idx, in_degree, nullptr, in_src, in_weight, stream);
}

int gbx_graph_create_offsets(gbx_graph **out, uint32_t num_vertices, uint32_t num_edges,
                             const uint32_t *offsets, const uint32_t *dest, const float *weight,
                             const uint32_t *in_offsets, const uint32_t *in_src,
                             const float *in_weight, void *stream) {
    GBX_REQUIRE(offsets, GBX_ERR_INVALID, "offsets is NULL");
    return create_common(out, num_vertices, num_edges, nullptr, nullptr, offsets, dest, weight,
                         nullptr, nullptr, in_offsets, in_src, in_weight, stream);
}

int gbx_graph_destroy(gbx_graph *g) {
    if (!g) return GBX_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    cudaDeviceSynchronize();
    dev_free(g->offsets);
    dev_free(g->dest);
    dev_free(g->weight);
    dev_free(g->out_degree);
    dev_free(g->in_offsets);
    dev_free(g->in_src);
    dev_free(g->in_weight);
    dev_free(g->in_degree);
    dev_free(g->low_count);
    dev_free(g->bu_live);
    gbx_free_tc_plan(g->tc_plan);
    gbx_free_ppr_cache(g->ppr);
    gbx_free_ms_plan(g->ms_plan);
    gbx_free_pr_cache(g->pr_cache);
    gbx_free_bc_cache(g->bc_cache);
    dev_free(g->arena);
    free_plan(g->plan_fwd);
    free_plan(g->plan_inv);
    cudaSetDevice(prev);
    delete g;
    return GBX_OK;
}

int gbx_graph_info(const gbx_graph *g, uint32_t *num_vertices, uint32_t *num_edges,
                   int *has_inverse, int *has_weights) {
    GBX_REQUIRE(g, GBX_ERR_INVALID, "graph is NULL");
    if (num_vertices) *num_vertices = g->V;
    if (num_edges) *num_edges = g->E;
    if (has_inverse) *has_inverse = g->has_inverse() ? 1 : 0;
    if (has_weights) *has_weights = g->weight ? 1 : 0;
    return GBX_OK;
}

int gbx_graph_device_arrays(const gbx_graph *g, const uint32_t **offsets, const uint32_t **dest,
                            const float **weight, const uint32_t **in_offsets,
                            const uint32_t **in_src, const float **in_weight) {
    GBX_REQUIRE(g, GBX_ERR_INVALID, "graph is NULL");
    if (offsets) *offsets = g->offsets;
    if (dest) *dest = g->dest;
    if (weight) *weight = g->weight;
    if (in_offsets) *in_offsets = g->in_offsets;
    if (in_src) *in_src = g->in_src;
    if (in_weight) *in_weight = g->in_weight;
    return GBX_OK;
}

}  // extern "C"
