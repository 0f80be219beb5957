// Direction-optimising BFS (the reference's
// breadthFirstSearchDirectionOptimizedGraphCSR, BFS.c:335-485, with the
// top-down step :498-546 and the bottom-up step :562-613).
//
// State in HBM: level[V] (0xFFFFFFFF = unvisited), parent[V], a visited
// bitmap and two frontier bitmaps (V/8 bytes each: 512 KiB at 4M vertices,
// resident in L2), and two vertex queues.
//
//  top-down  : the frontier queue's degrees are prefix-summed; a persistent
//              grid walks the flattened edge list in tiles of 1024 edges
//              (consecutive threads on consecutive edges, so dest[] loads are
//              coalesced), finds each edge's frontier vertex by a binary
//              search bounded to the tile's range, claims unvisited
//              neighbours with atomicOr on the visited bitmap, and appends
//              them to the next queue with one atomic per warp (ballot +
//              popc ranks).
//  bottom-up : one warp per 32 consecutive vertices = one bitmap word; each
//              unvisited lane scans its pull neighbours until one is in the
//              current frontier bitmap; the warp ballot is the next-frontier
//              word and is or-ed into the visited word by a single writer.
//
// The direction heuristic is the reference's (alpha 15, beta 18, mu/mf/nf
// bookkeeping in uint32 arithmetic), evaluated on the host after each step
// from a 24-byte counter block, so processed_nodes and iteration match the
// reference's stats.
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {

struct BfsCounters {
    uint32_t qlen;  // vertices appended to the next queue (degree > 0)
    uint32_t nf;    // vertices claimed in this step
    uint32_t mf;    // sum over claimed of max(out_degree, 1) (BFS.c:537)
    uint32_t pad;
    unsigned long long edges;  // sum of out_degree over claimed
};

constexpr int kTdThreads = 256;
constexpr int kTdItems = 4;
constexpr uint32_t kTdTile = kTdThreads * kTdItems;

__global__ void bfs_init_kernel(uint32_t *level, int32_t *parent, uint32_t *visited, uint32_t V,
                                uint32_t words, uint32_t source) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        level[v] = v == source ? 0u : kInfLevel;
        parent[v] = v == source ? (int32_t)source : -1;
    }
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += gridDim.x * blockDim.x)
        visited[w] = (w == (source >> 5)) ? (1u << (source & 31)) : 0u;
}

__global__ void gather_degrees_kernel(const uint32_t *q, uint32_t qlen, const uint32_t *deg,
                                      uint32_t *out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < qlen; i += gridDim.x * blockDim.x)
        out[i] = deg[q[i]];
}

// largest f in [lo, hi] with pre[f] <= i
__device__ __forceinline__ uint32_t frontier_search(const uint32_t *pre, uint32_t lo, uint32_t hi,
                                                    uint32_t i) {
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(pre + mid) <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(kTdThreads)
    bfs_top_down_kernel(const uint32_t *__restrict__ q, const uint32_t *__restrict__ pre, uint32_t qlen,
                        const uint32_t *__restrict__ total_edges, const uint32_t *__restrict__ off,
                        const uint32_t *__restrict__ dest, const uint32_t *__restrict__ outdeg,
                        uint32_t *visited, uint32_t *level, int32_t *parent, uint32_t lnext,
                        uint32_t *qnext, BfsCounters *cnt) {
    __shared__ uint32_t s_range[2];
    const uint32_t M = *total_edges;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t nf = 0, mf = 0;
    unsigned long long edges = 0;
    for (uint64_t base = (uint64_t)blockIdx.x * kTdTile; base < M; base += (uint64_t)gridDim.x * kTdTile) {
        uint64_t tile_end = base + kTdTile < M ? base + kTdTile : (uint64_t)M;
        uint32_t last = (uint32_t)tile_end - 1;
        if (threadIdx.x < 2) {
            uint32_t target = threadIdx.x == 0 ? (uint32_t)base : last;
            s_range[threadIdx.x] = frontier_search(pre, 0, qlen - 1, target);
        }
        __syncthreads();
        const uint32_t flo = s_range[0], fhi = s_range[1];
#pragma unroll
        for (int k = 0; k < kTdItems; ++k) {
            uint64_t i = base + (uint64_t)k * kTdThreads + threadIdx.x;
            bool claimed = false;
            uint32_t u = 0, du = 0;
            if (i < M) {
                uint32_t f = frontier_search(pre, flo, fhi, (uint32_t)i);
                uint32_t v = __ldg(q + f);
                uint32_t e = __ldg(off + v) + ((uint32_t)i - __ldg(pre + f));
                u = __ldg(dest + e);
                uint32_t bit = 1u << (u & 31);
                uint32_t *word = visited + (u >> 5);
                if (!(__ldcg(word) & bit)) {
                    uint32_t old = atomicOr(word, bit);
                    if (!(old & bit)) {
                        claimed = true;
                        level[u] = lnext;
                        parent[u] = (int32_t)v;
                        du = __ldg(outdeg + u);
                        nf += 1;
                        mf += du ? du : 1u;
                        edges += du;
                    }
                }
            }
            bool push = claimed && du > 0;
            unsigned m = __ballot_sync(0xffffffffu, push);
            if (m) {
                uint32_t leader = __ffs(m) - 1;
                uint32_t basepos = 0;
                if (lane == leader) basepos = atomicAdd(&cnt->qlen, (uint32_t)__popc(m));
                basepos = __shfl_sync(0xffffffffu, basepos, leader);
                if (push) qnext[basepos + __popc(m & ((1u << lane) - 1u))] = u;
            }
        }
        __syncthreads();
    }
    // per-warp counter flush
    nf = warp_sum(nf);
    mf = warp_sum(mf);
    edges = warp_sum(edges);
    if (lane == 0 && nf) {
        atomicAdd(&cnt->nf, nf);
        atomicAdd(&cnt->mf, mf);
        atomicAdd(&cnt->edges, edges);
    }
}

// frontier bitmap of the vertices at level `l` (entering bottom-up)
__global__ void level_to_bitmap_kernel(const uint32_t *level, uint32_t V, uint32_t l, uint32_t *bm,
                                       uint32_t words) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = gw; w < words; w += nw) {
        uint32_t v = w * 32 + lane;
        unsigned m = __ballot_sync(0xffffffffu, v < V && level[v] == l);
        if (lane == 0) bm[w] = m;
    }
}

__global__ void __launch_bounds__(256)
    bfs_bottom_up_kernel(const uint32_t *__restrict__ poff, const uint32_t *__restrict__ psrc,
                         const uint32_t *__restrict__ cur, uint32_t *__restrict__ next,
                         uint32_t *visited, uint32_t *level, int32_t *parent,
                         const uint32_t *__restrict__ outdeg, uint32_t V, uint32_t words,
                         uint32_t lnext, BfsCounters *cnt) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    uint32_t nf = 0;
    unsigned long long edges = 0;
    for (uint32_t w = gw; w < words; w += nw) {
        uint32_t vis = visited[w];
        if (vis == 0xFFFFFFFFu) {
            if (lane == 0) next[w] = 0;
            continue;
        }
        uint32_t v = w * 32 + lane;
        bool found = false;
        if (v < V && !((vis >> lane) & 1u)) {
            uint32_t b = __ldg(poff + v), e = __ldg(poff + v + 1);
            for (uint32_t j = b; j < e; ++j) {
                uint32_t u = __ldg(psrc + j);
                if ((__ldg(cur + (u >> 5)) >> (u & 31)) & 1u) {
                    level[v] = lnext;
                    parent[v] = (int32_t)u;
                    found = true;
                    break;
                }
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, found);
        if (found) edges += __ldg(outdeg + v);
        if (lane == 0) {
            next[w] = m;
            if (m) visited[w] = vis | m;
            nf += __popc(m);
        }
    }
    edges = warp_sum(edges);
    if (lane == 0) {
        if (nf) atomicAdd(&cnt->nf, nf);
        if (edges) atomicAdd(&cnt->edges, edges);
    }
}

// bitmapToArrayQueue (arrayQueue.c:310-337): frontier bitmap -> queue of its
// vertices with out-degree > 0 (degree-0 vertices have nothing to expand)
__global__ void bitmap_to_queue_kernel(const uint32_t *bm, uint32_t words, uint32_t V,
                                       const uint32_t *outdeg, uint32_t *q, BfsCounters *cnt) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = gw; w < words; w += nw) {
        uint32_t word = bm[w];
        if (!word) continue;
        uint32_t v = w * 32 + lane;
        bool push = ((word >> lane) & 1u) && v < V && outdeg[v] > 0;
        unsigned m = __ballot_sync(0xffffffffu, push);
        if (!m) continue;
        uint32_t basepos = 0;
        if (lane == 0) basepos = atomicAdd(&cnt->qlen, (uint32_t)__popc(m));
        basepos = __shfl_sync(0xffffffffu, basepos, 0);
        if (push) q[basepos + __popc(m & ((1u << lane) - 1u))] = v;
    }
}

__global__ void bfs_finish_kernel(const uint32_t *level, const int32_t *parent,
                                  const uint32_t *outdeg, uint32_t V, uint32_t *dist,
                                  int32_t *par_out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        uint32_t l = level[v];
        if (dist) dist[v] = l == kInfLevel ? 0u : l;
        if (par_out) {
            uint32_t d = outdeg[v];
            par_out[v] = l == kInfLevel ? (d ? -(int32_t)d : -1) : parent[v];
        }
    }
}

struct BfsWork {
    DevBuf<uint32_t> level, visited, bm0, bm1, q0, q1, degs, pre, total;
    DevBuf<int32_t> parent;
    DevBuf<BfsCounters> cnt;
    int alloc(uint32_t V, cudaStream_t s) {
        uint32_t words = (V + 31) / 32;
        GBX_TRY(level.alloc(V, s));
        GBX_TRY(parent.alloc(V, s));
        GBX_TRY(visited.alloc(words, s));
        GBX_TRY(bm0.alloc(words, s));
        GBX_TRY(bm1.alloc(words, s));
        GBX_TRY(q0.alloc(V, s));
        GBX_TRY(q1.alloc(V, s));
        GBX_TRY(degs.alloc(V, s));
        GBX_TRY(pre.alloc(V, s));
        GBX_TRY(total.alloc(1, s));
        GBX_TRY(cnt.alloc(1, s));
        return GBX_OK;
    }
};

static int grid_for(uint64_t n, int threads = 256, int per_sm = 8) {
    uint64_t b = (n + threads - 1) / threads;
    uint64_t cap = (uint64_t)num_sms() * per_sm;
    return (int)std::max<uint64_t>(1, std::min(b, cap));
}

static int read_counters(BfsCounters *h, BfsCounters *d, cudaStream_t s) {
    GBX_CUDA(cudaMemcpyAsync(h, d, sizeof(BfsCounters), cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}

// One top-down step from queue q (qlen entries). Returns counters in *h.
static int top_down_step(gbx_graph *g, BfsWork &w, const uint32_t *q, uint32_t qlen, uint32_t *qnext,
                         uint32_t lnext, BfsCounters *h, cudaStream_t s) {
    GBX_CUDA(cudaMemsetAsync(w.cnt.p, 0, sizeof(BfsCounters), s));
    if (qlen > 0) {
        gather_degrees_kernel<<<grid_for(qlen), 256, 0, s>>>(q, qlen, g->out_degree, w.degs.p);
        GBX_LAUNCH_CHECK();
        GBX_TRY(exclusive_scan_u32(w.degs.p, w.pre.p, qlen, s, w.total.p));
        bfs_top_down_kernel<<<num_sms() * 8, kTdThreads, 0, s>>>(
            q, w.pre.p, qlen, w.total.p, g->offsets, g->dest, g->out_degree, w.visited.p,
            w.level.p, w.parent.p, lnext, qnext, w.cnt.p);
        GBX_LAUNCH_CHECK();
    }
    return read_counters(h, w.cnt.p, s);
}

static int bottom_up_step(gbx_graph *g, BfsWork &w, const uint32_t *cur, uint32_t *next,
                          uint32_t lnext, BfsCounters *h, cudaStream_t s) {
    uint32_t words = (g->V + 31) / 32;
    GBX_CUDA(cudaMemsetAsync(w.cnt.p, 0, sizeof(BfsCounters), s));
    bfs_bottom_up_kernel<<<grid_for((uint64_t)words * 32), 256, 0, s>>>(
        g->pull_offsets(), g->pull_src(), cur, next, w.visited.p, w.level.p, w.parent.p,
        g->out_degree, g->V, words, lnext, w.cnt.p);
    GBX_LAUNCH_CHECK();
    return read_counters(h, w.cnt.p, s);
}

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_bfs(gbx_graph *g, uint32_t source, int mode, uint32_t *distances,
                       int32_t *parents, gbx_bfs_result *result, void *stream) {
    clear_error();
    GBX_REQUIRE(g, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(source < g->V, GBX_ERR_INVALID, "source %u out of range [0, %u)", source, g->V);
    GBX_REQUIRE(mode >= 0 && mode <= 2, GBX_ERR_INVALID, "mode must be 0, 1 or 2");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V, words = (V + 31) / 32;
    BfsWork w;
    GBX_TRY(w.alloc(V, s));
    OutArray<uint32_t> dist;
    OutArray<int32_t> par;
    GBX_TRY(dist.bind(distances, V, s));
    GBX_TRY(par.bind(parents, V, s));

    bfs_init_kernel<<<grid_for(V), 256, 0, s>>>(w.level.p, w.parent.p, w.visited.p, V, words, source);
    GBX_LAUNCH_CHECK();
    uint32_t hdeg = 0;
    GBX_CUDA(cudaMemcpyAsync(&hdeg, g->out_degree + source, 4, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaMemcpyAsync(w.q0.p, &source, 4, cudaMemcpyHostToDevice, s));
    GBX_CUDA(cudaStreamSynchronize(s));

    gbx_bfs_result r = {};
    r.processed_nodes = 1;
    r.iteration = 1;
    r.edges_traversed = hdeg;
    uint32_t *q = w.q0.p, *qn = w.q1.p;
    uint32_t *bcur = w.bm0.p, *bnext = w.bm1.p;
    uint32_t qlen = hdeg ? 1u : 0u;  // queue of vertices to expand (degree > 0)
    uint32_t qsize = 1;              // the reference's queue size (all claimed)
    uint32_t L = 0;
    const uint32_t alpha = 15, beta = 18;
    uint32_t mu = g->E, mf = hdeg;
    BfsCounters h;

    auto do_bottom_up_phase = [&](uint32_t nf_start, bool until_empty) -> int {
        level_to_bitmap_kernel<<<grid_for((uint64_t)words * 32), 256, 0, s>>>(w.level.p, V, L, bcur, words);
        GBX_LAUNCH_CHECK();
        uint32_t nf = nf_start, nf_prev;
        do {
            nf_prev = nf;
            GBX_TRY(bottom_up_step(g, w, bcur, bnext, L + 1, &h, s));
            nf = h.nf;
            std::swap(bcur, bnext);
            r.processed_nodes += nf;
            r.iteration++;
            r.bottom_up_steps++;
            r.edges_traversed += h.edges;
            if (nf) L++;
            if (until_empty && nf == 0) break;
        } while (until_empty ? true : (nf > nf_prev || nf > V / beta));
        qsize = nf;
        // bitmapToArrayQueue: the last step's new vertices become the queue
        GBX_CUDA(cudaMemsetAsync(w.cnt.p, 0, sizeof(BfsCounters), s));
        if (nf) {
            bitmap_to_queue_kernel<<<grid_for((uint64_t)words * 32), 256, 0, s>>>(
                bcur, words, V, g->out_degree, q, w.cnt.p);
            GBX_LAUNCH_CHECK();
        }
        GBX_TRY(read_counters(&h, w.cnt.p, s));
        qlen = h.qlen;
        return GBX_OK;
    };

    if (mode == 0) {
        // pull-only BFS (BFS.c:140-213): bottom-up steps until no vertex is added
        GBX_TRY(do_bottom_up_phase(1, true));
    } else {
        while (qsize) {
            if (mode == 2 && mf > mu / alpha) {
                GBX_TRY(do_bottom_up_phase(qsize, false));
                mf = 1;
            } else {
                mu -= mf;
                GBX_TRY(top_down_step(g, w, q, qlen, qn, L + 1, &h, s));
                mf = h.mf;
                qsize = h.nf;
                qlen = h.qlen;
                std::swap(q, qn);
                r.processed_nodes += qsize;
                r.iteration++;
                r.top_down_steps++;
                r.edges_traversed += h.edges;
                if (qsize) L++;
            }
        }
    }
    r.depth = L;
    bfs_finish_kernel<<<grid_for(V), 256, 0, s>>>(w.level.p, w.parent.p, g->out_degree, V, dist.d,
                                                  par.d);
    GBX_LAUNCH_CHECK();
    GBX_TRY(dist.finish(s));
    GBX_TRY(par.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    if (result) *result = r;
    return GBX_OK;
}
