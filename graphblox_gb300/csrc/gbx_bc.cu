// Betweenness centrality (Brandes), Bellman-Ford and the stack DFS of the
// reference host (betweennessCentrality.c, bellmanFord.c, DFS.c).
//
// Brandes needs, from a vertex v, the vertices w whose pull row holds v
// (its successors in the shortest-path DAG), in ascending id order: the
// reference folds the dependency contributions into v from the top of its
// stack down, i.e. in descending (level, id) order of w, and float addition
// is not associative. That successor CSR is the forward CSR when the graph
// has an inverse and its rows are sorted, otherwise the transpose of the
// pull CSR built here once per graph by a stable sort on the neighbour id.
#include "gbx_internal.cuh"

#include <atomic>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

struct gbx_bc_cache {
    uint32_t *succ_off = nullptr;  // V+1, owned when built here
    uint32_t *succ_ids = nullptr;  // E
    bool owned = false;
};

void gbx_free_bc_cache(struct gbx_bc_cache *c) {
    if (!c) return;
    if (c->owned) {
        cudaFree(c->succ_off);
        cudaFree(c->succ_ids);
    }
    delete c;
}

namespace gbx {

static unsigned grid_sm(uint64_t n, int threads = 256) {
    const uint64_t b = (n + threads - 1) / threads;
    const uint64_t cap = (uint64_t)num_sms() * 8;
    return (unsigned)(b == 0 ? 1 : (b > cap ? cap : b));
}

// flag[0] = 1 when some row of (off, ids) is not ascending
__global__ void rows_sorted_kernel(const uint32_t *off, const uint32_t *ids, uint32_t V, unsigned *flag) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < V; v += warps) {
        const uint32_t b = off[v], e = off[v + 1];
        bool bad = false;
        for (uint32_t j = b + 1 + lane; j < e; j += 32)
            bad |= (ids[j - 1] & kIdMask) > (ids[j] & kIdMask);
        if (__any_sync(0xffffffffu, bad)) {
            if (lane == 0) atomicOr(flag, 1u);
        }
    }
}

// keys[j] = neighbour id of entry j, vals[j] = the vertex whose row holds j
// (rows are in vertex order, so a stable sort on keys keeps vals ascending)
__global__ void transpose_pairs_kernel(const uint32_t *off, const uint32_t *ids, uint32_t V, uint32_t E,
                                       uint32_t *keys, uint32_t *vals) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < E; j += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = V;  // last v with off[v] <= j
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (off[mid] <= j) lo = mid; else hi = mid;
        }
        keys[j] = ids[j] & kIdMask;
        vals[j] = lo;
    }
}

// run starts of a sorted key array -> per-key counts (deg[k] = run length)
__global__ void run_lengths_kernel(const uint32_t *keys, uint32_t E, uint32_t *deg) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        if (i + 1 == E || keys[i + 1] != k) {
            // the run of k ends here; find its start by the previous key's end
            uint32_t lo = 0, hi = i;  // first index with keys[idx] == k
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (keys[mid] < k) lo = mid + 1; else hi = mid;
            }
            deg[k] = i + 1 - lo;
        }
    }
}

// transpose of the pull CSR into toff (V+1) / tids (E + 4 zeroed ids)
static int build_transpose(const gbx_graph *g, uint32_t *toff, uint32_t *tids, cudaStream_t s) {
    const uint32_t V = g->V, E = g->E;
    DevBuf<uint32_t> keys, deg, tot;
    GBX_TRY(keys.alloc(E ? E : 1, s));
    GBX_TRY(deg.alloc(V, s));
    GBX_TRY(tot.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(deg.p, 0, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(tids + E, 0, 16, s));
    if (E) {
        transpose_pairs_kernel<<<grid_sm(E), 256, 0, s>>>(g->pull_offsets(), g->pull_src(), V, E, keys.p, tids);
        GBX_LAUNCH_CHECK();
        int bits = 0;
        while (bits < 32 && ((V - 1) >> bits)) ++bits;
        GBX_TRY(radix_sort_pairs(keys.p, tids, E, bits, s));
        run_lengths_kernel<<<grid_sm(E), 256, 0, s>>>(keys.p, E, deg.p);
        GBX_LAUNCH_CHECK();
    }
    GBX_TRY(exclusive_scan_u32(deg.p, toff, V, s, tot.p));
    GBX_CUDA(cudaMemcpyAsync(toff + V, tot.p, 4, cudaMemcpyDeviceToDevice, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}

static int bc_successors(gbx_graph *g, cudaStream_t s, const uint32_t **off, const uint32_t **ids) {
    if (!g->bc_cache) {
        const uint32_t V = g->V, E = g->E;
        bool use_forward = false;
        if (g->has_inverse()) {
            DevBuf<unsigned> flag;
            GBX_TRY(flag.alloc(1, s));
            GBX_CUDA(cudaMemsetAsync(flag.p, 0, 4, s));
            rows_sorted_kernel<<<grid_sm((uint64_t)V * 32), 256, 0, s>>>(g->offsets, g->dest, V, flag.p);
            GBX_LAUNCH_CHECK();
            unsigned h = 0;
            GBX_CUDA(cudaMemcpyAsync(&h, flag.p, 4, cudaMemcpyDeviceToHost, s));
            GBX_CUDA(cudaStreamSynchronize(s));
            use_forward = h == 0;
        }
        gbx_bc_cache *c = new gbx_bc_cache();
        if (use_forward) {
            c->succ_off = g->offsets;
            c->succ_ids = g->dest;
        } else {
            uint32_t *toff = nullptr, *tids = nullptr;
            int st = GBX_OK;
            if (cudaMalloc(&toff, ((size_t)V + 1) * 4) != cudaSuccess ||
                cudaMalloc(&tids, ((size_t)E + 4) * 4) != cudaSuccess) {
                (void)cudaGetLastError();
                set_error("device allocation of the successor CSR failed");
                st = GBX_ERR_NOMEM;
            }
            if (st == GBX_OK) st = build_transpose(g, toff, tids, s);
            if (st != GBX_OK) {
                cudaStreamSynchronize(s);
                cudaFree(toff);
                cudaFree(tids);
                delete c;
                return st;
            }
            c->succ_off = toff;
            c->succ_ids = tids;
            c->owned = true;
        }
        g->bc_cache = c;
    }
    *off = g->bc_cache->succ_off;
    *ids = g->bc_cache->succ_ids;
    return GBX_OK;
}

}  // namespace gbx

// ---- betweenness centrality --------------------------------------------------
namespace gbx {

// Vertices whose successor row is longer than this are "heavy": their rows
// are cut across the whole grid (forward pushes and backward terms), while
// a warp handles each lighter row. The packed per-level counter gives every
// heavy vertex its list slot (high half) and its term-buffer base (low
// half) in one atomic, so the list is ordered by base.
constexpr uint32_t kBcHeavy = 1024;

struct BcCounters {
    unsigned long long next;   // vertices claimed for the next level
    unsigned long long dag;    // predecessor entries (DAG edges) of this root
    unsigned long long heavy;  // next level's heavy vertices << 32 | their row total
    unsigned long long pad;
};

__device__ __forceinline__ void bc_note_heavy(const uint32_t *off, uint32_t v, BcCounters *c, uint2 *heavy) {
    const uint32_t d = off[v + 1] - off[v];
    if (d > kBcHeavy) {
        const unsigned long long old = atomicAdd(&c->heavy, (1ull << 32) | d);
        heavy[old >> 32] = make_uint2(v, (uint32_t)old);
    }
}

__global__ void bc_root_kernel(const uint32_t *off, uint32_t root, uint32_t *dist, int32_t *sigma,
                               uint32_t *stack, BcCounters *c, uint2 *heavy) {
    dist[root] = 0;
    sigma[root] = 1;
    stack[0] = root;
    bc_note_heavy(off, root, c, heavy);
}

// claim v for level L+1 from a level-L vertex with sigma su; returns true
// when v is a successor (claimed now or earlier in this level)
__device__ __forceinline__ bool bc_claim(uint32_t v, uint32_t L, unsigned su, uint32_t *dist, int32_t *sigma,
                                         bool &fresh) {
    const uint32_t old = atomicCAS(dist + v, kInfLevel, L + 1);
    fresh = old == kInfLevel;
    const bool hit = fresh || old == L + 1;
    if (hit) atomicAdd(reinterpret_cast<unsigned *>(sigma) + v, su);
    return hit;
}

// warp-aggregated append of the lanes' fresh vertices to the next level
__device__ __forceinline__ void bc_append(bool fresh, uint32_t v, const uint32_t *off, uint32_t *next,
                                          BcCounters *c, uint2 *heavy_next) {
    const uint32_t lane = threadIdx.x & 31;
    const unsigned fm = __ballot_sync(0xffffffffu, fresh);
    if (!fm) return;
    uint32_t pos = 0;
    if (lane == 0) pos = (uint32_t)atomicAdd(&c->next, (unsigned long long)__popc(fm));
    pos = __shfl_sync(0xffffffffu, pos, 0);
    if (fresh) {
        next[pos + __popc(fm & ((1u << lane) - 1u))] = v;
        bc_note_heavy(off, v, c, heavy_next);
    }
}

// One forward level for the light vertices of level[0..n), a warp per
// vertex, pushed over the successor CSR: a successor v not reached yet is
// claimed for level L+1 and appended to next[], and every successor at
// level L+1 adds sigma[u] -- the reference's sigma[v] += sigma[u] over the
// frontier entries of v's pull row (betweennessCentrality.c:322-336); int
// addition wraps and is associative, so the order does not matter.
__global__ void bc_forward_kernel(const uint32_t *off, const uint32_t *ids, const uint32_t *level, uint32_t n,
                                  uint32_t L, uint32_t *dist, int32_t *sigma, uint32_t *next, BcCounters *c,
                                  uint2 *heavy_next) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    unsigned entries = 0;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const uint32_t u = level[i];
        const uint32_t b = off[u], e = off[u + 1];
        if (e - b > kBcHeavy) continue;  // bc_forward_heavy_kernel
        const unsigned su = (unsigned)sigma[u];
        for (uint32_t base = b; base < e; base += 32) {
            const uint32_t j = base + lane;
            bool fresh = false, hit = false;
            uint32_t v = 0;
            if (j < e) {
                v = ids[j] & kIdMask;
                hit = bc_claim(v, L, su, dist, sigma, fresh);
            }
            entries += (unsigned)__popc(__ballot_sync(0xffffffffu, hit));
            bc_append(fresh, v, off, next, c, heavy_next);
        }
    }
    if (lane == 0 && entries) atomicAdd(&c->dag, (unsigned long long)entries);
}

// last i in [0, n) with heavy[i].y <= e (the bases ascend with i)
__device__ __forceinline__ uint32_t bc_heavy_owner(const uint2 *heavy, uint32_t n, uint32_t e) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (heavy[mid].y <= e) lo = mid; else hi = mid;
    }
    return lo;
}

// The heavy vertices' rows of one forward level, one entry per thread over
// the concatenated rows [0, total).
__global__ void bc_forward_heavy_kernel(const uint32_t *off, const uint32_t *ids, const uint2 *heavy, uint32_t nh,
                                        uint32_t total, uint32_t L, uint32_t *dist, int32_t *sigma,
                                        uint32_t *next, BcCounters *c, uint2 *heavy_next) {
    const uint32_t lane = threadIdx.x & 31;
    unsigned entries = 0;
    const uint32_t stride = gridDim.x * blockDim.x;  // a multiple of 32
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < total; base += stride) {
        const uint32_t e = base + lane;
        bool fresh = false, hit = false;
        uint32_t v = 0;
        if (e < total) {
            const uint2 h = heavy[bc_heavy_owner(heavy, nh, e)];
            v = ids[off[h.x] + (e - h.y)] & kIdMask;
            hit = bc_claim(v, L, (unsigned)sigma[h.x], dist, sigma, fresh);
        }
        entries += (unsigned)__popc(__ballot_sync(0xffffffffu, hit));
        bc_append(fresh, v, off, next, c, heavy_next);
    }
    if (lane == 0 && entries) atomicAdd(&c->dag, (unsigned long long)entries);
}

// term of successor w of v (sv = sigma[v]), 0 when w is not a successor:
// (sigma[v] * 1.0 / sigma[w]) * double(1.0f + dep[w]), each step rounded on
// its own (betweennessCentrality.c:445-449)
__device__ __forceinline__ double bc_term(double sv, uint32_t w, uint32_t L, const uint32_t *dist,
                                          const int32_t *sigma, const float *dep) {
    if (dist[w] != L + 1) return 0.0;
    const int32_t sw = sigma[w];
    if (sw == 0) return 0.0;
    return __dmul_rn(__ddiv_rn(sv, (double)sw), (double)__fadd_rn(1.0f, dep[w]));
}

// acc <- float(double(acc) + t) for the lanes' nonzero terms, lane 0 first.
// A zero term is the identity of this step (acc is never -0), so skipping
// non-successors keeps the reference's result.
__device__ __forceinline__ float bc_fold(float acc, double term) {
    unsigned m = __ballot_sync(0xffffffffu, term != 0.0);
    while (m) {
        const int k = __ffs(m) - 1;
        const double t = __shfl_sync(0xffffffffu, term, k);
        acc = __double2float_rn(__dadd_rn((double)acc, t));
        m &= m - 1u;
    }
    return acc;
}

// bc[v] += dep[v] / 2 for every v but the root, one root after another in
// the caller's order (the reference adds each root's dependencies as its
// stack unwinds; unreached vertices and the deepest level add +0, which
// leaves bc unchanged)
__global__ void bc_accumulate_kernel(float *bc, const float *dep, uint32_t V, uint32_t root) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        if (v != root) bc[v] = __fadd_rn(bc[v], __fdiv_rn(dep[v], 2.0f));
}

// One backward level for the light vertices of level[0..n). Each folds its
// successors at level L+1 in descending id order, as the reference's walk
// down its stack reaches them (betweennessCentrality.c:432-455), then
// dep[v] is the result (bc_accumulate_kernel adds it). A warp loads 32
// entries at a time from the end of v's ascending row.
__global__ void bc_backward_kernel(const uint32_t *off, const uint32_t *ids, const uint32_t *level, uint32_t n,
                                   uint32_t L, const uint32_t *dist, const int32_t *sigma, float *dep) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const uint32_t v = level[i];
        const uint32_t b = off[v], e = off[v + 1];
        if (e - b > kBcHeavy) continue;  // bc_terms_kernel + bc_fold_heavy_kernel
        const double sv = (double)sigma[v];
        float acc = 0.0f;
        for (uint32_t top = e; top > b;) {
            const uint32_t avail = top - b;
            const double term = lane < avail ? bc_term(sv, ids[top - 1 - lane] & kIdMask, L, dist, sigma, dep) : 0.0;
            acc = bc_fold(acc, term);
            top = avail > 32u ? top - 32u : b;
        }
        if (lane == 0) dep[v] = acc;
    }
}

// The heavy vertices' rows of one backward level, one entry per thread over
// the concatenated rows [0, total): flag[e] = 1 when the entry is a
// successor with sigma != 0 (the only entries whose terms can be nonzero)...
__global__ void bc_flags_kernel(const uint32_t *off, const uint32_t *ids, const uint2 *heavy, uint32_t nh,
                                uint32_t total, uint32_t L, const uint32_t *dist, const int32_t *sigma,
                                uint32_t *flag) {
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const uint2 h = heavy[bc_heavy_owner(heavy, nh, e)];
        const uint32_t w = ids[off[h.x] + (e - h.y)] & kIdMask;
        flag[e] = (dist[w] == L + 1 && sigma[w] != 0) ? 1u : 0u;
    }
}

// ... then their terms, compacted in row order at pos[e] (exclusive scan of flag)
__global__ void bc_terms_kernel(const uint32_t *off, const uint32_t *ids, const uint2 *heavy, uint32_t nh,
                                uint32_t total, uint32_t L, const uint32_t *dist, const int32_t *sigma,
                                const float *dep, const uint32_t *flag, const uint32_t *pos, double *terms) {
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        if (!flag[e]) continue;
        const uint2 h = heavy[bc_heavy_owner(heavy, nh, e)];
        terms[pos[e]] = bc_term((double)sigma[h.x], ids[off[h.x] + (e - h.y)] & kIdMask, L, dist, sigma, dep);
    }
}

// ... and their folds: a warp per heavy vertex over its compacted terms
// [pos[base], pos[base + row length]), from the end
__global__ void bc_fold_heavy_kernel(const uint32_t *off, const uint2 *heavy, uint32_t nh, const uint32_t *pos,
                                     const double *terms, float *dep) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nh; i += warps) {
        const uint2 h = heavy[i];
        const uint32_t b = pos[h.y], e = pos[h.y + (off[h.x + 1] - off[h.x])];
        float acc = 0.0f;
        uint32_t top = e;
        double cur = (top > b && lane < top - b) ? terms[top - 1 - lane] : 0.0;
        while (top > b) {
            const uint32_t avail = top - b;
            const uint32_t nxt = avail > 32u ? top - 32u : b;
            // load the next chunk before folding this one
            const double ahead = (nxt > b && lane < nxt - b) ? terms[nxt - 1 - lane] : 0.0;
            acc = bc_fold(acc, cur);
            cur = ahead;
            top = nxt;
        }
        if (lane == 0) dep[h.x] = acc;
    }
}

static unsigned warp_grid(uint64_t items) { return grid_sm(items * 32); }

// Per-root working memory of one worker.
struct BcRoot {
    DevBuf<uint32_t> dist, stack, flag, pos;
    DevBuf<int32_t> sigma;
    DevBuf<float> dep;
    DevBuf<uint2> heavy;
    DevBuf<BcCounters> ctr;
    DevBuf<double> terms;
    uint32_t levels = 0;
    unsigned long long dag = 0;
    void release() {
        dist.release();
        stack.release();
        flag.release();
        pos.release();
        sigma.release();
        dep.release();
        heavy.release();
        ctr.release();
        terms.release();
    }
    int alloc(uint32_t V, cudaStream_t s) {
        GBX_TRY(dist.alloc(V, s));
        GBX_TRY(stack.alloc(V, s));
        GBX_TRY(sigma.alloc(V, s));
        GBX_TRY(dep.alloc(V, s));
        GBX_TRY(heavy.alloc(V, s));
        GBX_TRY(ctr.alloc(1, s));
        return GBX_OK;
    }
};

// Brandes for one root on stream s: dist, sigma and dep of every vertex
// (dep is what bc_accumulate_kernel adds); one host sync per forward level.
static int bc_one_root(const uint32_t *soff, const uint32_t *sids, uint32_t V, uint32_t root, BcRoot &w,
                       cudaStream_t s) {
    uint32_t *dist = w.dist.p, *stack = w.stack.p;
    int32_t *sigma = w.sigma.p;
    float *dep = w.dep.p;
    uint2 *heavy = w.heavy.p;
    BcCounters *ctr = w.ctr.p;
    GBX_CUDA(cudaMemsetAsync(dist, 0xFF, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(sigma, 0, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(dep, 0, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(ctr, 0, sizeof(BcCounters), s));
    bc_root_kernel<<<1, 1, 0, s>>>(soff, root, dist, sigma, stack, ctr, heavy);
    GBX_LAUNCH_CHECK();
    BcCounters hc{};
    GBX_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    std::vector<uint32_t> start{0u, 1u}, hstart{0u, (uint32_t)(hc.heavy >> 32)}, htotal{(uint32_t)hc.heavy};
    size_t max_total = htotal[0];
    for (uint32_t L = 0;; ++L) {
        const uint32_t n = start[L + 1] - start[L];
        const uint32_t nh = hstart[L + 1] - hstart[L];
        GBX_CUDA(cudaMemsetAsync(&ctr->next, 0, 8, s));
        GBX_CUDA(cudaMemsetAsync(&ctr->heavy, 0, 8, s));
        uint32_t *next = stack + start[L + 1];
        uint2 *heavy_next = heavy + hstart[L + 1];
        bc_forward_kernel<<<warp_grid(n), 256, 0, s>>>(soff, sids, stack + start[L], n, L, dist, sigma, next, ctr,
                                                       heavy_next);
        GBX_LAUNCH_CHECK();
        if (nh) {
            bc_forward_heavy_kernel<<<grid_sm(htotal[L]), 256, 0, s>>>(soff, sids, heavy + hstart[L], nh, htotal[L],
                                                                       L, dist, sigma, next, ctr, heavy_next);
            GBX_LAUNCH_CHECK();
        }
        GBX_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        if (hc.next == 0) break;
        start.push_back(start[L + 1] + (uint32_t)hc.next);
        hstart.push_back(hstart[L + 1] + (uint32_t)(hc.heavy >> 32));
        htotal.push_back((uint32_t)hc.heavy);
        if (htotal.back() > max_total) max_total = htotal.back();
    }
    w.dag = hc.dag;
    w.levels = (uint32_t)start.size() - 1;  // levels 0 .. levels-1 are non-empty
    if (max_total > w.flag.n) {
        GBX_TRY(w.flag.alloc(max_total, s));
        GBX_TRY(w.pos.alloc(max_total + 1, s));
    }
    for (int L = (int)w.levels - 2; L >= 0; --L) {
        const uint32_t n = start[L + 1] - start[L];
        const uint32_t nh = hstart[L + 1] - hstart[L];
        bc_backward_kernel<<<warp_grid(n), 256, 0, s>>>(soff, sids, stack + start[L], n, (uint32_t)L, dist, sigma,
                                                        dep);
        GBX_LAUNCH_CHECK();
        if (!nh) continue;
        const uint32_t tot = htotal[L];
        uint2 *hl = heavy + hstart[L];
        bc_flags_kernel<<<grid_sm(tot), 256, 0, s>>>(soff, sids, hl, nh, tot, (uint32_t)L, dist, sigma, w.flag.p);
        GBX_LAUNCH_CHECK();
        GBX_TRY(exclusive_scan_u32(w.flag.p, w.pos.p, tot, s, w.pos.p + tot));
        uint32_t nvalid = 0;
        GBX_CUDA(cudaMemcpyAsync(&nvalid, w.pos.p + tot, 4, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        if (nvalid > w.terms.n) GBX_TRY(w.terms.alloc(nvalid, s));
        if (nvalid) {
            bc_terms_kernel<<<grid_sm(tot), 256, 0, s>>>(soff, sids, hl, nh, tot, (uint32_t)L, dist, sigma, dep,
                                                         w.flag.p, w.pos.p, w.terms.p);
            GBX_LAUNCH_CHECK();
        }
        bc_fold_heavy_kernel<<<warp_grid(nh), 256, 0, s>>>(soff, hl, nh, w.pos.p, w.terms.p, dep);
        GBX_LAUNCH_CHECK();
    }
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}

// Roots in flight at once: each root's longest dependency fold is serial
// (one hub's successors in order), so independent roots overlap their folds
// with one another's level sweeps.
constexpr uint32_t kBcConcurrentRoots = 8;

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_betweenness(gbx_graph *g, uint32_t num_roots, const uint32_t *roots, float *centrality,
                               uint32_t *distances, int32_t *sigma_out, float *dependency,
                               gbx_bc_result *result, void *stream) {
    clear_error();
    GBX_REQUIRE(g != nullptr, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(centrality != nullptr, GBX_ERR_INVALID, "centrality is NULL");
    GBX_REQUIRE(num_roots == 0 || roots != nullptr, GBX_ERR_INVALID, "roots is NULL");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    std::vector<uint32_t> hroots(num_roots);
    if (num_roots) {
        if (is_device_ptr(roots)) {
            GBX_CUDA(cudaMemcpyAsync(hroots.data(), roots, (size_t)num_roots * 4, cudaMemcpyDeviceToHost, s));
            GBX_CUDA(cudaStreamSynchronize(s));
        } else {
            std::memcpy(hroots.data(), roots, (size_t)num_roots * 4);
        }
    }
    for (uint32_t r = 0; r < num_roots; ++r)
        GBX_REQUIRE(hroots[r] < V, GBX_ERR_INVALID, "root %u (%u) out of range [0, %u)", r, hroots[r], V);
    const uint32_t *soff = nullptr, *sids = nullptr;
    GBX_TRY(bc_successors(g, s, &soff, &sids));
    OutArray<float> obc;
    GBX_TRY(obc.bind(centrality, V, s));
    if (obc.to_host()) GBX_CUDA(cudaMemcpyAsync(obc.d, centrality, (size_t)V * 4, cudaMemcpyHostToDevice, s));
    const uint32_t K = num_roots < kBcConcurrentRoots ? num_roots : kBcConcurrentRoots;
    std::vector<cudaStream_t> ws(K, nullptr);
    std::vector<BcRoot> work(K);
    int st = GBX_OK;
    for (uint32_t k = 0; k < K && st == GBX_OK; ++k) {
        if (cudaStreamCreateWithFlags(&ws[k], cudaStreamNonBlocking) != cudaSuccess) {
            (void)cudaGetLastError();
            set_error("stream creation failed");
            st = GBX_ERR_CUDA;
        }
        if (st == GBX_OK) st = work[k].alloc(V, ws[k]);
    }
    // the caller's pending work on s (the centrality upload) before the workers
    if (st == GBX_OK && cudaStreamSynchronize(s) != cudaSuccess) st = GBX_ERR_CUDA;
    // Workers take roots in order as they free up; each root's dependencies
    // are added to bc in root order: a worker waits for the previous root's
    // turn (host token) and makes its add wait for the previous add (event).
    const int device = g->device;
    std::vector<cudaEvent_t> ev(K, nullptr);
    for (uint32_t k = 0; k < K && st == GBX_OK; ++k)
        if (cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming) != cudaSuccess) {
            (void)cudaGetLastError();
            set_error("event creation failed");
            st = GBX_ERR_CUDA;
        }
    std::mutex mu;
    std::condition_variable turn;
    uint32_t next_add = 0;               // root whose add goes next
    cudaEvent_t prev_add = nullptr;      // event after the previous root's add
    std::atomic<uint32_t> next_root{0};
    std::atomic<bool> failed{st != GBX_OK};
    // the first failure (in time) is the one reported; workers that give up
    // their roots after it record nothing
    int first_rc = GBX_OK;
    std::string first_msg;
    constexpr int kSkipped = 1;
    auto record_failure = [&](int rc) {  // caller holds mu
        if (first_rc == GBX_OK) {
            first_rc = rc;
            first_msg = gbx_last_error();  // the message is per thread
        }
        failed.store(true);
    };
    std::vector<uint32_t> last_of(K, UINT32_MAX);
    std::vector<std::thread> th;
    for (uint32_t k = 0; k < K && st == GBX_OK; ++k)
        th.emplace_back([&, k] {
            cudaSetDevice(device);
            for (;;) {
                const uint32_t r = next_root.fetch_add(1);
                if (r >= num_roots) break;
                int rc = failed.load() ? kSkipped : bc_one_root(soff, sids, V, hroots[r], work[k], ws[k]);
                std::unique_lock<std::mutex> lk(mu);
                if (rc != GBX_OK && rc != kSkipped) record_failure(rc);
                turn.wait(lk, [&] { return next_add == r; });
                if (rc == GBX_OK && !failed.load()) {
                    if (prev_add) cudaStreamWaitEvent(ws[k], prev_add, 0);
                    bc_accumulate_kernel<<<grid_sm(V), 256, 0, ws[k]>>>(obc.d, work[k].dep.p, V, hroots[r]);
                    note_launch();
                    if (cudaGetLastError() != cudaSuccess || cudaEventRecord(ev[k], ws[k]) != cudaSuccess) {
                        set_error("betweenness accumulation launch failed");
                        rc = GBX_ERR_CUDA;
                        record_failure(rc);
                    }
                    prev_add = ev[k];
                }
                last_of[k] = r;
                next_add = r + 1;
                lk.unlock();
                turn.notify_all();
                if (rc != GBX_OK) break;
            }
        });
    for (auto &t : th) t.join();
    if (first_rc != GBX_OK && st == GBX_OK) {
        st = first_rc;
        set_error("betweenness: %s", first_msg.c_str());
    }
    for (uint32_t k = 0; k < K; ++k)
        if (ws[k] && cudaStreamSynchronize(ws[k]) != cudaSuccess && st == GBX_OK) {
            st = GBX_ERR_CUDA;
            set_error("betweenness: a worker stream failed");
        }
    for (uint32_t k = 0; k < K; ++k)
        if (ev[k]) cudaEventDestroy(ev[k]);
    uint32_t last = 0;  // the worker that ran the last root holds its state
    for (uint32_t k = 0; k < K; ++k)
        if (num_roots && last_of[k] == num_roots - 1) last = k;
    if (st == GBX_OK) st = obc.finish(s);
    if (st == GBX_OK && num_roots) {
        BcRoot &w = work[last];
        if (distances) {
            OutArray<uint32_t> o;
            if ((st = o.bind(distances, V, s)) == GBX_OK) {
                cudaMemcpyAsync(o.d, w.dist.p, (size_t)V * 4, cudaMemcpyDeviceToDevice, s);
                st = o.finish(s);
                cudaStreamSynchronize(s);
            }
        }
        if (st == GBX_OK && sigma_out) {
            OutArray<int32_t> o;
            if ((st = o.bind(sigma_out, V, s)) == GBX_OK) {
                cudaMemcpyAsync(o.d, w.sigma.p, (size_t)V * 4, cudaMemcpyDeviceToDevice, s);
                st = o.finish(s);
                cudaStreamSynchronize(s);
            }
        }
        if (st == GBX_OK && dependency) {
            OutArray<float> o;
            if ((st = o.bind(dependency, V, s)) == GBX_OK) {
                cudaMemcpyAsync(o.d, w.dep.p, (size_t)V * 4, cudaMemcpyDeviceToDevice, s);
                st = o.finish(s);
                cudaStreamSynchronize(s);
            }
        }
    }
    if (cudaStreamSynchronize(s) != cudaSuccess && st == GBX_OK) st = GBX_ERR_CUDA;
    if (st == GBX_OK && result) {
        result->iteration = num_roots;
        result->processed_nodes = num_roots ? (uint32_t)work[last].dag : 0;
        result->levels = num_roots ? work[last].levels : 0;
    }
    for (uint32_t k = 0; k < K; ++k) {
        if (ws[k]) cudaStreamSynchronize(ws[k]);
        work[k].release();  // frees on ws[k], before the stream goes
    }
    for (uint32_t k = 0; k < K; ++k)
        if (ws[k]) cudaStreamDestroy(ws[k]);
    return st;
}

// ---- Bellman-Ford and DFS -----------------------------------------------------
namespace gbx {

// Parents of the shortest-path tree: the smallest u with an edge u->v and
// (uint32)((float)dist[u] + w) == dist[v]. The reference keeps whichever
// relaxation wrote last (bellmanFord.c:134-227), so its parents depend on
// the schedule; every such u is a valid parent and the smallest is the
// deterministic choice. par[] starts at UINT32_MAX (unreached). Each thread
// takes kBfEdges consecutive edges (hub rows spread over many threads):
// one binary search for the first edge's source, then a walk forward.
constexpr uint32_t kBfEdges = 16;

__global__ void bf_parents_kernel(const uint32_t *off, const uint32_t *dest, const float *w, uint32_t V,
                                  uint32_t E, const uint32_t *dist, uint32_t source, uint32_t *par) {
    const uint32_t chunks = (E + kBfEdges - 1) / kBfEdges;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < chunks; c += gridDim.x * blockDim.x) {
        const uint32_t e0 = c * kBfEdges, e1 = e0 + kBfEdges < E ? e0 + kBfEdges : E;
        uint32_t lo = 0, hi = V;  // last u with off[u] <= e0
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (off[mid] <= e0) lo = mid; else hi = mid;
        }
        uint32_t u = lo, uend = off[u + 1];
        for (uint32_t j = e0; j < e1; ++j) {
            while (j >= uend) uend = off[++u + 1];
            const uint32_t du = dist[u];
            if (du == kSsspInf) continue;
            const uint32_t v = dest[j] & kIdMask;
            const float wt = w ? w[j] : 1.0f;
            if (v != source && __float2uint_rz(__fadd_rn(__uint2float_rn(du), wt)) == dist[v]) atomicMin(par + v, u);
        }
    }
}

__global__ void set_u32_kernel(uint32_t *a, uint32_t i, uint32_t value) { a[i] = value; }

// The reference's stack DFS (DFS.c:156-205) run by one warp, since each pop
// depends on every earlier one: pop v, scan its row in CSR order 32 entries
// at a time; a neighbour not visited yet is taken by the first lane holding
// it (a repeated neighbour in the same chunk resolves to its first copy, as
// in the sequential loop), gets parent v and distance dist[v] + 1 and is
// pushed in row order. A vertex is pushed at most once, so the stacks never
// hold more than V entries and the loop ends after at most V pops.
// Each pop is a chain of dependent loads, so the kernel keeps that chain
// short: the visited set is a shared-memory bitmap when V fits (else the
// parents array is read), distances travel on the stack beside the ids, and
// the entry on top after a push is kept in registers.
constexpr uint32_t kDfsSmemBits = 1536u * 1024u;  // 192 KB of bitmap

__global__ void dfs_warp_kernel(const uint32_t *off, const uint32_t *dest, uint32_t V, uint32_t source,
                                uint32_t *dist, int32_t *par, uint32_t *stack, uint32_t *stack_dist,
                                uint32_t *processed) {
    extern __shared__ uint32_t seen[];
    const uint32_t lane = threadIdx.x & 31;
    const bool in_smem = V <= kDfsSmemBits;
    if (in_smem) {
        for (uint32_t i = lane; i < (V + 31) / 32; i += 32) seen[i] = 0;
        __syncwarp();
        if (lane == 0) seen[source >> 5] |= 1u << (source & 31);
    }
    if (lane == 0) par[source] = (int32_t)source;
    __syncwarp();
    uint32_t top = 1, pops = 0;
    uint32_t cv = source, cd = 0;  // the top entry, valid when cached
    bool cached = true;
    while (top > 0) {
        uint32_t v, d;
        if (cached) {
            v = cv;
            d = cd;
        } else {
            v = stack[top - 1];
            d = stack_dist[top - 1];
        }
        --top;
        cached = false;
        ++pops;
        const uint32_t e = off[v + 1];
        for (uint32_t base = off[v]; base < e; base += 32) {
            const uint32_t j = base + lane;
            const uint32_t u = j < e ? (dest[j] & kIdMask) : 0xFFFFFFFFu;
            bool take = false;
            if (j < e) take = in_smem ? !((seen[u >> 5] >> (u & 31)) & 1u) : par[u] < 0;
            const unsigned peers = __match_any_sync(0xffffffffu, u);
            take = take && lane == (uint32_t)(__ffs(peers) - 1);
            const unsigned m = __ballot_sync(0xffffffffu, take);
            if (take) {
                if (in_smem) atomicOr(&seen[u >> 5], 1u << (u & 31));
                par[u] = (int32_t)v;
                dist[u] = d + 1u;
                const uint32_t at = top + __popc(m & ((1u << lane) - 1u));
                stack[at] = u;
                stack_dist[at] = d + 1u;
            }
            if (m) {
                // the last pushed entry (highest lane) is the new top
                const int hi = 31 - __clz(m);
                cv = __shfl_sync(0xffffffffu, u, hi);
                cd = d + 1u;
                cached = true;
            }
            top += (uint32_t)__popc(m);
            __syncwarp();
        }
    }
    if (lane == 0) *processed = pops;
}

}  // namespace gbx

extern "C" int gbx_bellman_ford(gbx_graph *g, uint32_t source, uint32_t *distances, uint32_t *parents,
                                gbx_sssp_result *result, void *stream) {
    clear_error();
    GBX_REQUIRE(g != nullptr, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(distances != nullptr, GBX_ERR_INVALID, "distances is NULL");
    GBX_REQUIRE(source < g->V, GBX_ERR_INVALID, "source %u out of range [0, %u)", source, g->V);
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    OutArray<uint32_t> od;
    GBX_TRY(od.bind(distances, V, s));
    gbx_sssp_result r{};
    GBX_TRY(gbx_sssp(g, source, 0, od.d, &r, stream));
    if (parents) {
        OutArray<uint32_t> op;
        GBX_TRY(op.bind(parents, V, s));
        GBX_CUDA(cudaMemsetAsync(op.d, 0xFF, (size_t)V * 4, s));
        bf_parents_kernel<<<grid_sm(((uint64_t)g->E + kBfEdges - 1) / kBfEdges), 256, 0, s>>>(
            g->offsets, g->dest, g->weight, V, g->E, od.d, source, op.d);
        GBX_LAUNCH_CHECK();
        set_u32_kernel<<<1, 1, 0, s>>>(op.d, source, source);
        GBX_LAUNCH_CHECK();
        GBX_TRY(op.finish(s));
        GBX_CUDA(cudaStreamSynchronize(s));
    }
    GBX_TRY(od.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    if (result) *result = r;
    return GBX_OK;
}

extern "C" int gbx_dfs(gbx_graph *g, uint32_t source, uint32_t *distances, int32_t *parents,
                       uint32_t *processed_nodes, void *stream) {
    clear_error();
    GBX_REQUIRE(g != nullptr, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(distances != nullptr && parents != nullptr, GBX_ERR_INVALID, "distances/parents is NULL");
    GBX_REQUIRE(source < g->V, GBX_ERR_INVALID, "source %u out of range [0, %u)", source, g->V);
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    OutArray<uint32_t> od;
    OutArray<int32_t> op;
    GBX_TRY(od.bind(distances, V, s));
    GBX_TRY(op.bind(parents, V, s));
    DevBuf<uint32_t> stack, stack_dist, pops;
    GBX_TRY(stack.alloc((size_t)V + 1, s));
    GBX_TRY(stack_dist.alloc((size_t)V + 1, s));
    GBX_TRY(pops.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(od.d, 0, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(op.d, 0xFF, (size_t)V * 4, s));
    const size_t smem = V <= kDfsSmemBits ? (size_t)((V + 31) / 32) * 4 : 0;
    if (smem > 48 * 1024)
        GBX_CUDA(cudaFuncSetAttribute(dfs_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dfs_warp_kernel<<<1, 32, smem, s>>>(g->offsets, g->dest, V, source, od.d, op.d, stack.p, stack_dist.p, pops.p);
    GBX_LAUNCH_CHECK();
    uint32_t hp = 0;
    GBX_CUDA(cudaMemcpyAsync(&hp, pops.p, 4, cudaMemcpyDeviceToHost, s));
    GBX_TRY(od.finish(s));
    GBX_TRY(op.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    if (processed_nodes) *processed_nodes = hp;
    return GBX_OK;
}

// ---- the reference's random roots ------------------------------------------------
// Host code: the Mersenne Twister MT19937 (Matsumoto and Nishimura, 1998)
// with the seeding of its first release (Knuth's LCG x <- 69069 x + 1, the
// upper 16 bits of two draws per state word), as the reference's
// mt19937.c seeds it (graphConfig.c:84 uses 27491095), and the rejection
// loop of generateRandomRootBetweennessCentrality (betweennessCentrality.c:
// 172-189): draw until the value is a vertex whose out-degree exceeds E/V.
namespace {

// The generator state in the reference's layout (624 unsigned long words and
// the index, mt19937.h:58-62), stepped by gbx_mt19937_next.
struct Mt19937 {
    unsigned long mt[624];
    int mti = 624;
    explicit Mt19937(uint32_t seed) {
        for (int i = 0; i < 624; ++i) {
            mt[i] = seed & 0xffff0000u;
            seed = 69069u * seed + 1u;
            mt[i] |= (seed & 0xffff0000u) >> 16;
            seed = 69069u * seed + 1u;
        }
    }
    uint32_t next() { return gbx_mt19937_next(mt, &mti); }
};

}  // namespace

// One draw: regenerate the 624 words when they are used up (the twist), then
// temper the next one. The words hold 32-bit values in 64-bit slots, as the
// reference's do.
extern "C" uint32_t gbx_mt19937_next(unsigned long *mt, int *mti) {
    if (*mti >= 624) {
        for (int k = 0; k < 624; ++k) {
            const unsigned long y = (mt[k] & 0x80000000UL) | (mt[(k + 1) % 624] & 0x7fffffffUL);
            mt[k] = mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1UL) ? 0x9908b0dfUL : 0UL);
        }
        *mti = 0;
    }
    unsigned long y = mt[(*mti)++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680UL;
    y ^= (y << 15) & 0xefc60000UL;
    y ^= y >> 18;
    return (uint32_t)y;
}

extern "C" int gbx_reference_roots(gbx_graph *g, uint32_t seed, uint32_t n, uint32_t *roots) {
    clear_error();
    GBX_REQUIRE(g != nullptr, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(n == 0 || roots != nullptr, GBX_ERR_INVALID, "roots is NULL");
    GBX_TRY(ensure_device());
    const uint32_t V = g->V, avg = g->E / g->V;
    std::vector<uint32_t> deg(V);
    GBX_CUDA(cudaMemcpy(deg.data(), g->out_degree, (size_t)V * 4, cudaMemcpyDeviceToHost));
    uint32_t maxdeg = 0;
    for (uint32_t d : deg) maxdeg = d > maxdeg ? d : maxdeg;
    GBX_REQUIRE(n == 0 || maxdeg > avg, GBX_ERR_INVALID,
                "no vertex has an out-degree above the average (%u): the draw would not end", avg);
    Mt19937 m(seed);
    for (uint32_t i = 0; i < n; ++i) {
        for (;;) {
            const uint32_t r = m.next();
            if (r < V && deg[r] > avg) {
                roots[i] = r;
                break;
            }
        }
    }
    return GBX_OK;
}
