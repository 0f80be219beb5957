// Batched BFS and PageRank over many graphs in one persistent launch.
// No reference counterpart as a batch: each graph gets exactly the per-graph
// results of the reference's breadthFirstSearchGraphCSR (BFS.c:103-127, the
// direction-optimising loop :335-485) and pageRankPullGraphCSR
// (pageRank.c:245-368), the same as gbx_bfs / gbx_pagerank_pull.
//
// Layout (gbx_batch): the graphs' CSRs packed back to back. Packed vertex
// vertex_base[g] + v is graph g's vertex v; offsets[] (total V + 1) hold
// global edge positions; dest / in_src hold graph-local ids. A device work
// queue deals whole graphs to CTAs, largest edge count first.
//
// One CTA owns one graph at a time, so a level or an iteration ends with
// __syncthreads instead of a grid barrier, and the per-graph working set
// lives in shared memory:
//   BFS: visited / frontier / next bitmaps (3 x V/8 bytes); neighbour tests
//        are shared-memory bit probes. Top-down flattens the out-edges of 32
//        frontier vertices per warp; bottom-up gives each warp 32 unvisited
//        vertices, one lane each, scanning in-edges until a frontier parent.
//   PR:  contributions (4V bytes) in shared memory; the gather streams the
//        graph's in-edge ids from global memory and reads contributions from
//        shared memory. Rows above 32 in-edges are summed by the whole warp
//        with per-lane Kahan compensation.
// Graphs too large for the shared-memory capacity use the same code on a
// per-CTA global scratch slot.
#include <algorithm>
#include <numeric>
#include <vector>

#include "gbx_internal.cuh"

struct gbx_batch {
    int device = 0;
    uint32_t G = 0, V = 0, E = 0;
    uint32_t max_v = 0;
    uint32_t *vbase = nullptr;       // G+1
    uint32_t *offsets = nullptr;     // V+1, global edge positions
    uint32_t *dest = nullptr;        // E, graph-local ids
    uint32_t *in_offsets = nullptr;  // V+1 or null (pull = forward CSR)
    uint32_t *in_src = nullptr;      // E or null
    uint32_t *order = nullptr;       // G, graph ids by descending edge count
    std::vector<uint32_t> h_vbase;   // host copy of vbase
    const uint32_t *poff() const { return in_offsets ? in_offsets : offsets; }
    const uint32_t *psrc() const { return in_offsets ? in_src : dest; }
};

namespace gbx {

constexpr int kBbThreads = 512;
constexpr int kBbWarps = kBbThreads / 32;
constexpr uint32_t kBbWordsCap = 4096;  // bitmap words in shared memory: V <= 131072
constexpr int kBpThreads = 1024;
constexpr int kBpWarps = kBpThreads / 32;
constexpr uint32_t kBpSmemV = 49152;  // contributions in shared memory: V <= 49152 (192 KiB)

__device__ __forceinline__ uint32_t bb_next_graph(uint32_t *cursor, uint32_t G, const uint32_t *order,
                                                  uint32_t *s_slot) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t i = atomicAdd(cursor, 1u);
        *s_slot = i < G ? order[i] : 0xFFFFFFFFu;
    }
    __syncthreads();
    return *s_slot;
}

struct BbArgs {
    uint32_t G;
    const uint32_t *vbase, *off, *dest, *poff, *psrc, *order, *sources;
    uint32_t *dist;
    int32_t *parent;
    gbx_bfs_result *res;
    uint32_t *cursor;
    uint32_t *scratch;  // per CTA: 3 * scratch_words
    uint32_t scratch_words;
    uint32_t alpha, beta;
};

// ---- BFS -----------------------------------------------------------------------
__global__ void __launch_bounds__(kBbThreads, 2) bfs_batched_kernel(BbArgs a) {
    extern __shared__ uint32_t s_bits[];  // 3 * kBbWordsCap
    __shared__ uint32_t s_pre[kBbWarps][33];
    __shared__ uint32_t s_slot, s_nf;
    __shared__ unsigned long long s_mf;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (;;) {
        const uint32_t g = bb_next_graph(a.cursor, a.G, a.order, &s_slot);
        if (g == 0xFFFFFFFFu) break;
        const uint32_t vb = a.vbase[g], Vg = a.vbase[g + 1] - vb;
        const uint32_t words = (Vg + 31) / 32;
        uint32_t *S, *F, *N;
        if (words <= kBbWordsCap) {
            S = s_bits;
            F = s_bits + kBbWordsCap;
            N = s_bits + 2 * kBbWordsCap;
        } else {
            uint32_t *base = a.scratch + (size_t)blockIdx.x * 3 * a.scratch_words;
            S = base;
            F = base + a.scratch_words;
            N = base + 2 * a.scratch_words;
        }
        const uint32_t *off = a.off + vb;  // off[v], v local; values are global edge positions
        const uint32_t *poff = a.poff + vb;
        const uint32_t src = a.sources[g];
        const uint32_t Eg = off[Vg] - off[0];
        for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) {
            S[w] = 0;
            F[w] = 0;
            N[w] = 0;
        }
        for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x) a.dist[vb + v] = 0;
        if (threadIdx.x == 0) {
            s_nf = 0;
            s_mf = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            S[src >> 5] = 1u << (src & 31);
            F[src >> 5] = 1u << (src & 31);
            if (a.parent) a.parent[vb + src] = (int32_t)src;
        }
        __syncthreads();
        const uint32_t deg_src = off[src + 1] - off[src];
        unsigned long long mf = deg_src, edges_total = deg_src;
        uint32_t processed = 1, iteration = 1, L = 0, td = 0, bu = 0, nf_prev = 0;
        bool in_bu = false;
        for (uint32_t step = 0; step <= Vg; ++step) {
            const unsigned long long mu = (unsigned long long)Eg - edges_total;
            bool use_bu;
            if (in_bu)
                use_bu = true;
            else
                use_bu = mf > mu / a.alpha;
            uint32_t my_nf = 0;
            unsigned long long my_mf = 0;
            if (use_bu) {
                // each warp owns whole words of S and N: no atomics on them
                for (uint32_t w = warp; w < words; w += kBbWarps) {
                    const uint32_t valid = (w + 1) * 32 <= Vg ? 0xFFFFFFFFu : ((1u << (Vg & 31)) - 1u);
                    const uint32_t unv = ~S[w] & valid;
                    if (!unv) continue;
                    const uint32_t v = w * 32 + lane;
                    uint32_t found = 0xFFFFFFFFu;
                    if ((unv >> lane) & 1u) {
                        const uint32_t b = poff[v], e = poff[v + 1];
                        for (uint32_t j = b; j < e; ++j) {
                            const uint32_t u = __ldg(a.psrc + j);
                            if ((F[u >> 5] >> (u & 31)) & 1u) {
                                found = u;
                                break;
                            }
                        }
                    }
                    const uint32_t hit = __ballot_sync(0xFFFFFFFFu, found != 0xFFFFFFFFu);
                    if (found != 0xFFFFFFFFu) {
                        a.dist[vb + v] = L + 1;
                        if (a.parent) a.parent[vb + v] = (int32_t)found;
                        my_mf += off[v + 1] - off[v];
                    }
                    if (lane == 0 && hit) {
                        S[w] |= hit;
                        N[w] = hit;
                        my_nf += __popc(hit);
                    }
                }
                bu++;
            } else {
                for (uint32_t w = warp; w < words; w += kBbWarps) {
                    const uint32_t fw = F[w];
                    if (!fw) continue;
                    const uint32_t u = w * 32 + lane;
                    const bool mine = (fw >> lane) & 1u;
                    const uint32_t eb = mine ? off[u] : 0;
                    const uint32_t deg = mine ? off[u + 1] - eb : 0;
                    // exclusive prefix of the 32 degrees
                    uint32_t incl = deg;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                        if (lane >= (uint32_t)o) incl += t;
                    }
                    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
                    s_pre[warp][lane] = incl - deg;
                    if (lane == 31) s_pre[warp][32] = total;
                    __syncwarp();
                    for (uint32_t j = lane; j < total; j += 32) {
                        // owner: last k with s_pre[k] <= j (degree-0 lanes share a prefix; take the last)
                        uint32_t lo = 0, hi = 31;
                        while (lo < hi) {
                            const uint32_t mid = (lo + hi + 1) >> 1;
                            if (s_pre[warp][mid] <= j) lo = mid; else hi = mid - 1;
                        }
                        const uint32_t k = lo;
                        const uint32_t uu = w * 32 + k;
                        const uint32_t e = off[uu] + (j - s_pre[warp][k]);
                        const uint32_t v = __ldg(a.dest + e);
                        const uint32_t bit = 1u << (v & 31);
                        if (S[v >> 5] & bit) continue;
                        const uint32_t old = atomicOr(&S[v >> 5], bit);
                        if (old & bit) continue;
                        atomicOr(&N[v >> 5], bit);
                        a.dist[vb + v] = L + 1;
                        if (a.parent) a.parent[vb + v] = (int32_t)uu;
                        my_nf++;
                        my_mf += off[v + 1] - off[v];
                    }
                    __syncwarp();
                }
                td++;
            }
            my_nf = warp_sum(my_nf);
            my_mf = warp_sum(my_mf);
            if (lane == 0 && (my_nf || my_mf)) {
                atomicAdd(&s_nf, my_nf);
                atomicAdd(&s_mf, my_mf);
            }
            __syncthreads();
            const uint32_t nf = s_nf;
            const unsigned long long nmf = s_mf;
            __syncthreads();
            if (threadIdx.x == 0) {
                s_nf = 0;
                s_mf = 0;
            }
            // the old frontier becomes the next output bitmap
            for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) F[w] = 0;
            uint32_t *t = F;
            F = N;
            N = t;
            __syncthreads();
            processed += nf;
            iteration++;
            edges_total += nmf;
            if (nf == 0) break;
            L++;
            if (use_bu) {
                // the reference stays bottom-up while the frontier grows or is large
                in_bu = nf > nf_prev || nf > Vg / a.beta;
                nf_prev = nf;
            } else {
                nf_prev = nf;
            }
            mf = nmf;
        }
        // unreached vertices: parent = -out_degree, or -1 without out-edges
        if (a.parent) {
            for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x) {
                if (!((S[v >> 5] >> (v & 31)) & 1u)) {
                    const uint32_t d = off[v + 1] - off[v];
                    a.parent[vb + v] = d ? -(int32_t)d : -1;
                }
            }
        }
        if (threadIdx.x == 0 && a.res) {
            gbx_bfs_result r;
            r.processed_nodes = processed;
            r.iteration = iteration;
            r.depth = L;
            r.top_down_steps = td;
            r.bottom_up_steps = bu;
            r.reserved = 0;
            r.edges_traversed = edges_total;
            a.res[g] = r;
        }
    }
}

// ---- PageRank --------------------------------------------------------------------
struct BpArgs {
    uint32_t G;
    const uint32_t *vbase, *off, *poff, *psrc, *order;
    float *ranks;    // output, also one rank buffer
    float *rother;   // second rank buffer (V)
    float *scratch;  // per CTA contributions for graphs above kBpSmemV
    uint32_t scratch_v;
    uint32_t *cursor;
    uint32_t max_it;
    double epsilon;
    gbx_pr_result *res;
};

// Shared memory of one PageRank CTA (dynamic): contributions, then the
// partial sums of heavy-row pieces, then the heavy-row table.
constexpr uint32_t kBpHeavyMax = 1024;                // heavy rows per graph
constexpr uint32_t kBpSlots = 4096 + kBpHeavyMax;     // piece partials
constexpr uint32_t kBpHeavyMin = 512;                 // in-degree above which a row is split
constexpr size_t kBpSmemBytes = (size_t)kBpSmemV * 4 + (size_t)kBpSlots * 4 + (size_t)(2 * kBpHeavyMax + 1) * 4;

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float x) {
    const float y = __fsub_rn(x, comp);
    const float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

// Exclusive scan of one value per thread over the block (blockDim.x = kBpThreads);
// returns the thread's prefix, *total the sum. Uses s_tmp[32].
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t *s_tmp, uint32_t *total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    __syncthreads();
    if (lane == 31) s_tmp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kBpWarps ? s_tmp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= (uint32_t)o) w += t;
        }
        s_tmp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    const uint32_t before = warp ? s_tmp[warp - 1] : 0u;
    *total = s_tmp[kBpWarps - 1];
    return before + incl - x;
}

// Rows of one graph, per iteration, as tasks dealt to warps by a
// shared-memory counter (so a slow task does not hold a fixed share):
//   pieces  kBpHeavyMin..-edge slices of the heavy rows (in-degree > T); a
//           warp sums one with per-lane Kahan and a warp reduction, and the
//           partial goes to its slot;
//   units   32 consecutive rows: light rows (<= 32 in-edges) one lane each,
//           four index loads in flight, medium rows by the whole warp with
//           per-lane Kahan; heavy rows are skipped here.
// After the barrier one thread per heavy row adds its pieces' partials in
// piece order. Every sum has a fixed order, so ranks are deterministic.
__global__ void __launch_bounds__(kBpThreads, 1) pr_batched_kernel(BpArgs a) {
    extern __shared__ float s_mem[];
    float *s_contrib = s_mem;
    float *s_part = s_mem + kBpSmemV;
    uint32_t *s_hrow = reinterpret_cast<uint32_t *>(s_part + kBpSlots);
    uint32_t *s_hfirst = s_hrow + kBpHeavyMax;
    __shared__ uint32_t s_slot, s_active, s_task, s_cnt, s_tmp[32];
    __shared__ unsigned long long s_hedges;
    __shared__ double s_err;
    const uint32_t lane = threadIdx.x & 31;
    const float damp = 0.85f;
    const float base = 1.0f - 0.85f;
    const bool can_stop = a.epsilon > 0.0;
    for (;;) {
        const uint32_t g = bb_next_graph(a.cursor, a.G, a.order, &s_slot);
        if (g == 0xFFFFFFFFu) break;
        const uint32_t vb = a.vbase[g], Vg = a.vbase[g + 1] - vb;
        float *contrib = Vg <= kBpSmemV ? s_contrib : a.scratch + (size_t)blockIdx.x * a.scratch_v;
        const uint32_t *off = a.off + vb;
        const uint32_t *poff = a.poff + vb;
        float *rc = a.ranks + vb, *rn = a.rother + vb;
        const double inv_n = 1.0 / (double)Vg;
        // heavy rows: the smallest threshold T >= kBpHeavyMin with at most
        // kBpHeavyMax rows above it
        uint32_t T = kBpHeavyMin;
        for (;;) {
            if (threadIdx.x == 0) {
                s_cnt = 0;
                s_hedges = 0;
            }
            __syncthreads();
            uint32_t c = 0;
            unsigned long long he = 0;
            for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x) {
                const uint32_t d = poff[v + 1] - poff[v];
                if (d > T) {
                    ++c;
                    he += d;
                }
            }
            c = warp_sum(c);
            he = warp_sum(he);
            if (lane == 0 && c) {
                atomicAdd(&s_cnt, c);
                atomicAdd(&s_hedges, he);
            }
            __syncthreads();
            if (s_cnt <= kBpHeavyMax) break;
            T *= 2;
            __syncthreads();
        }
        const uint32_t nh = s_cnt;
        // piece length: a multiple of 32 that keeps the pieces within the slots
        const unsigned long long want = (s_hedges + (kBpSlots - kBpHeavyMax) - 1) / (kBpSlots - kBpHeavyMax);
        const uint32_t P = (uint32_t)max(512ull, (want + 31) / 32 * 32);
        __syncthreads();
        if (threadIdx.x == 0) s_cnt = 0;
        __syncthreads();
        for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x)
            if (poff[v + 1] - poff[v] > T) s_hrow[atomicAdd(&s_cnt, 1u)] = v;
        __syncthreads();
        uint32_t np = 0;
        if (threadIdx.x < nh) {
            const uint32_t h = s_hrow[threadIdx.x];
            np = (poff[h + 1] - poff[h] + P - 1) / P;
        }
        uint32_t n_pieces = 0;
        const uint32_t first = block_exclusive_scan(np, s_tmp, &n_pieces);
        if (threadIdx.x < nh) s_hfirst[threadIdx.x] = first;
        if (threadIdx.x == 0) s_hfirst[nh] = n_pieces;
        for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x) {
            rc[v] = base;
            const uint32_t d = off[v + 1] - off[v];
            contrib[v] = d ? __fdiv_rn(base, (float)d) : 0.0f;
        }
        if (threadIdx.x == 0) {
            s_active = 0;
            s_err = 0.0;
            s_task = 0;
        }
        __syncthreads();
        const uint32_t units = (Vg + 31) / 32;
        const uint32_t n_tasks = n_pieces + units;
        uint32_t k = a.max_it, executed = 0, active_last = 0;
        double err_last = 0.0;
        for (uint32_t it = 0; it < a.max_it; ++it) {
            const bool reduce = can_stop || it + 1 == a.max_it;
            double err = 0.0;
            uint32_t active = 0;
            for (;;) {
                uint32_t t = 0;
                if (lane == 0) t = atomicAdd(&s_task, 1u);
                t = __shfl_sync(0xFFFFFFFFu, t, 0);
                if (t >= n_tasks) break;
                if (t < n_pieces) {
                    uint32_t lo = 0, hi = nh - 1;  // last heavy row with first piece <= t
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi + 1) >> 1;
                        if (s_hfirst[mid] <= t) lo = mid; else hi = mid - 1;
                    }
                    const uint32_t h = s_hrow[lo];
                    const uint32_t pb = poff[h] + (t - s_hfirst[lo]) * P;
                    const uint32_t pe = min(pb + P, poff[h + 1]);
                    float s = 0.f, c = 0.f;
                    for (uint32_t j = pb + lane; j < pe; j += 32) kahan_add(s, c, contrib[__ldg(a.psrc + j)]);
                    s = warp_sum(s);
                    if (lane == 0) s_part[t] = s;
                    continue;
                }
                const uint32_t v = (t - n_pieces) * 32 + lane;
                const bool ok = v < Vg;
                const uint32_t b = ok ? poff[v] : 0, e = ok ? poff[v + 1] : 0;
                const uint32_t d = e - b;
                float sum = 0.f;
                if (d <= 32) {
                    uint32_t j = b;
                    for (; j + 4 <= e; j += 4) {
                        const uint32_t u0 = __ldg(a.psrc + j), u1 = __ldg(a.psrc + j + 1);
                        const uint32_t u2 = __ldg(a.psrc + j + 2), u3 = __ldg(a.psrc + j + 3);
                        const float x0 = contrib[u0], x1 = contrib[u1], x2 = contrib[u2], x3 = contrib[u3];
                        sum = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(sum, x0), x1), x2), x3);
                    }
                    for (; j < e; ++j) sum = __fadd_rn(sum, contrib[__ldg(a.psrc + j)]);
                }
                uint32_t mv = __ballot_sync(0xFFFFFFFFu, d > 32 && d <= T);
                while (mv) {
                    const uint32_t kk = __ffs(mv) - 1;
                    mv &= mv - 1;
                    const uint32_t hb = __shfl_sync(0xFFFFFFFFu, b, kk), hd = __shfl_sync(0xFFFFFFFFu, e, kk);
                    float s = 0.f, c = 0.f;
                    for (uint32_t j = hb + lane; j < hd; j += 32) kahan_add(s, c, contrib[__ldg(a.psrc + j)]);
                    s = warp_sum(s);
                    if (lane == kk) sum = s;
                }
                if (ok && d <= T) {
                    const float next = __fadd_rn(base, __fmul_rn(damp, sum));
                    const float prev = rc[v];
                    rn[v] = next;
                    if (reduce) {
                        const double dd = (double)fabsf(__fsub_rn(next, prev));
                        err += dd * inv_n;
                        active += dd >= a.epsilon ? 1u : 0u;
                    }
                }
            }
            __syncthreads();
            // heavy rows: pieces in order
            if (threadIdx.x < nh) {
                const uint32_t h = s_hrow[threadIdx.x];
                float s = 0.f, c = 0.f;
                for (uint32_t p = s_hfirst[threadIdx.x]; p < s_hfirst[threadIdx.x + 1]; ++p) kahan_add(s, c, s_part[p]);
                const float next = __fadd_rn(base, __fmul_rn(damp, s));
                const float prev = rc[h];
                rn[h] = next;
                if (reduce) {
                    const double dd = (double)fabsf(__fsub_rn(next, prev));
                    err += dd * inv_n;
                    active += dd >= a.epsilon ? 1u : 0u;
                }
            }
            if (reduce) {
                err = warp_sum(err);
                active = warp_sum(active);
                if (lane == 0) {
                    atomicAdd(&s_err, err);
                    atomicAdd(&s_active, active);
                }
            }
            __syncthreads();
            // next contributions from the new ranks (shared memory is rewritten only now)
            for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x) {
                const uint32_t d = off[v + 1] - off[v];
                contrib[v] = d ? __fdiv_rn(rn[v], (float)d) : 0.0f;
            }
            const uint32_t act = s_active;
            const double er = s_err;
            if (threadIdx.x == 0) s_task = 0;
            __syncthreads();
            if (threadIdx.x == 0) {
                s_active = 0;
                s_err = 0.0;
            }
            float *t = rc;
            rc = rn;
            rn = t;
            executed = it + 1;
            active_last = can_stop ? act : Vg;
            err_last = er;
            if (can_stop && act == 0) {
                k = it;
                break;
            }
        }
        // final ranks / N into the output buffer
        float *out = a.ranks + vb;
        const float nf = (float)Vg;
        for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x) out[v] = __fdiv_rn(rc[v], nf);
        if (threadIdx.x == 0 && a.res) {
            gbx_pr_result r;
            r.iterations = k;
            r.active_last = executed ? active_last : 0;
            r.error_total = executed ? err_last : 0.0;
            a.res[g] = r;
        }
    }
}

// ---- validation ------------------------------------------------------------------
// One block per graph: offsets non-decreasing inside [off[vb], off[vb+Vg]],
// neighbour ids below Vg. Sets *bad on any violation.
__global__ void batch_check_kernel(const uint32_t *vbase, uint32_t G, const uint32_t *off, const uint32_t *ids,
                                   uint32_t E, uint32_t *bad) {
    for (uint32_t g = blockIdx.x; g < G; g += gridDim.x) {
        const uint32_t vb = vbase[g], Vg = vbase[g + 1] - vb;
        for (uint32_t v = threadIdx.x; v < Vg; v += blockDim.x) {
            const uint32_t b = off[vb + v], e = off[vb + v + 1];
            if (e < b || e > E) {
                atomicOr(bad, 1u);
                continue;
            }
            for (uint32_t j = b; j < e; ++j)
                if (ids[j] >= Vg) {
                    atomicOr(bad, 2u);
                    break;
                }
        }
    }
}

}  // namespace gbx

using namespace gbx;

namespace {

template <typename T>
int upload(T **dst, const T *src, size_t n, cudaStream_t s) {
    GBX_CUDA(cudaMalloc(dst, std::max<size_t>(n, 1) * sizeof(T)));
    if (n) GBX_CUDA(cudaMemcpyAsync(*dst, src, n * sizeof(T), cudaMemcpyDefault, s));
    return GBX_OK;
}

template <typename T>
int to_host(std::vector<T> &out, const T *src, size_t n, cudaStream_t s) {
    out.resize(n);
    if (n) GBX_CUDA(cudaMemcpyAsync(out.data(), src, n * sizeof(T), cudaMemcpyDefault, s));
    return GBX_OK;
}

int batch_create(gbx_batch *b, uint32_t G, const uint32_t *vertex_base, const uint32_t *offsets,
                 const uint32_t *dest, const uint32_t *in_offsets, const uint32_t *in_src, cudaStream_t s) {
    std::vector<uint32_t> vb;
    GBX_TRY(to_host(vb, vertex_base, (size_t)G + 1, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    GBX_REQUIRE(vb[0] == 0, GBX_ERR_INVALID, "vertex_base[0] must be 0");
    for (uint32_t g = 0; g < G; ++g)
        GBX_REQUIRE(vb[g + 1] > vb[g], GBX_ERR_INVALID, "graph %u has no vertices", g);
    const uint32_t V = vb[G];
    std::vector<uint32_t> off;
    GBX_TRY(to_host(off, offsets, (size_t)V + 1, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    GBX_REQUIRE(off[0] == 0, GBX_ERR_INVALID, "offsets[0] must be 0");
    const uint32_t E = off[V];
    b->G = G;
    b->V = V;
    b->E = E;
    std::vector<uint32_t> order(G);
    std::vector<uint64_t> eg(G);
    for (uint32_t g = 0; g < G; ++g) {
        eg[g] = (uint64_t)off[vb[g + 1]] - off[vb[g]] + (vb[g + 1] - vb[g]);
        b->max_v = std::max(b->max_v, vb[g + 1] - vb[g]);
    }
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return eg[x] > eg[y]; });
    GBX_REQUIRE(dest || E == 0, GBX_ERR_INVALID, "dest is NULL");
    GBX_TRY(upload(&b->vbase, vb.data(), vb.size(), s));
    GBX_TRY(upload(&b->offsets, off.data(), off.size(), s));
    GBX_TRY(upload(&b->dest, dest, E, s));
    GBX_TRY(upload(&b->order, order.data(), order.size(), s));
    if (in_offsets) {
        GBX_REQUIRE(in_src || E == 0, GBX_ERR_INVALID, "in_offsets without in_src");
        GBX_TRY(upload(&b->in_offsets, in_offsets, (size_t)V + 1, s));
        GBX_TRY(upload(&b->in_src, in_src, E, s));
    }
    DevBuf<uint32_t> bad;
    GBX_TRY(bad.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
    const unsigned grid = std::max(1u, std::min<unsigned>(G, (unsigned)num_sms() * 16));
    batch_check_kernel<<<grid, 256, 0, s>>>(b->vbase, G, b->offsets, b->dest, E, bad.p);
    GBX_LAUNCH_CHECK();
    if (b->in_offsets) {
        batch_check_kernel<<<grid, 256, 0, s>>>(b->vbase, G, b->in_offsets, b->in_src, E, bad.p);
        GBX_LAUNCH_CHECK();
    }
    uint32_t hbad = 0;
    GBX_CUDA(cudaMemcpyAsync(&hbad, bad.p, 4, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    b->h_vbase = std::move(vb);
    GBX_REQUIRE(hbad == 0, GBX_ERR_INVALID, "packed CSR rejected: %s",
                (hbad & 1) ? "offsets decrease or exceed the edge count" : "a neighbour id is not below its graph's vertex count");
    return GBX_OK;
}

void batch_free(gbx_batch *b) {
    cudaFree(b->vbase);
    cudaFree(b->offsets);
    cudaFree(b->dest);
    cudaFree(b->in_offsets);
    cudaFree(b->in_src);
    cudaFree(b->order);
    delete b;
}

}  // namespace

extern "C" int gbx_batch_create(gbx_batch **out, uint32_t num_graphs, const uint32_t *vertex_base,
                                const uint32_t *offsets, const uint32_t *dest, const uint32_t *in_offsets,
                                const uint32_t *in_src, void *stream) {
    clear_error();
    GBX_REQUIRE(out, GBX_ERR_INVALID, "out is NULL");
    *out = nullptr;
    GBX_REQUIRE(num_graphs > 0 && vertex_base && offsets, GBX_ERR_INVALID, "empty batch or NULL tables");
    GBX_TRY(ensure_device());
    gbx_batch *b = new gbx_batch();
    cudaGetDevice(&b->device);
    const int st = batch_create(b, num_graphs, vertex_base, offsets, dest, in_offsets, in_src, (cudaStream_t)stream);
    if (st != GBX_OK) {
        cudaStreamSynchronize((cudaStream_t)stream);
        batch_free(b);
        return st;
    }
    *out = b;
    return GBX_OK;
}

extern "C" int gbx_batch_destroy(gbx_batch *b) {
    clear_error();
    if (!b) return GBX_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    cudaDeviceSynchronize();
    batch_free(b);
    cudaSetDevice(prev);
    return GBX_OK;
}

extern "C" int gbx_batch_info(const gbx_batch *b, uint32_t *num_graphs, uint32_t *num_vertices,
                              uint32_t *num_edges) {
    clear_error();
    GBX_REQUIRE(b, GBX_ERR_INVALID, "batch is NULL");
    if (num_graphs) *num_graphs = b->G;
    if (num_vertices) *num_vertices = b->V;
    if (num_edges) *num_edges = b->E;
    return GBX_OK;
}

extern "C" int gbx_bfs_batched(gbx_batch *b, const uint32_t *sources, uint32_t *distances, int32_t *parents,
                               gbx_bfs_result *results, void *stream) {
    clear_error();
    GBX_REQUIRE(b && sources && distances, GBX_ERR_INVALID, "batch, sources or distances is NULL");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<uint32_t> hs;
    GBX_TRY(to_host(hs, sources, b->G, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    const std::vector<uint32_t> &vb = b->h_vbase;
    for (uint32_t g = 0; g < b->G; ++g)
        GBX_REQUIRE(hs[g] < vb[g + 1] - vb[g], GBX_ERR_INVALID, "source %u of graph %u is not below its %u vertices",
                    hs[g], g, vb[g + 1] - vb[g]);
    InArray<uint32_t> src_d;
    GBX_TRY(src_d.bind(sources, b->G, s));
    OutArray<uint32_t> dist;
    OutArray<int32_t> par;
    OutArray<gbx_bfs_result> res;
    GBX_TRY(dist.bind(distances, b->V, s));
    GBX_TRY(par.bind(parents, b->V, s));
    GBX_TRY(res.bind(results, b->G, s));
    DevBuf<uint32_t> cursor, scratch;
    GBX_TRY(cursor.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(cursor.p, 0, 4, s));
    const size_t smem = (size_t)3 * kBbWordsCap * sizeof(uint32_t);
    GBX_CUDA(cudaFuncSetAttribute(bfs_batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    GBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bfs_batched_kernel, kBbThreads, smem));
    const unsigned grid = std::max(1u, std::min<unsigned>((unsigned)num_sms() * std::max(occ, 1), b->G));
    const uint32_t words_max = (b->max_v + 31) / 32;
    BbArgs a;
    a.scratch_words = 0;
    a.scratch = nullptr;
    if (words_max > kBbWordsCap) {
        a.scratch_words = words_max;
        GBX_TRY(scratch.alloc((size_t)grid * 3 * words_max, s));
        a.scratch = scratch.p;
    }
    a.G = b->G;
    a.vbase = b->vbase;
    a.off = b->offsets;
    a.dest = b->dest;
    a.poff = b->poff();
    a.psrc = b->psrc();
    a.order = b->order;
    a.sources = src_d.d;
    a.dist = dist.d;
    a.parent = par.d;
    a.res = res.d;
    a.cursor = cursor.p;
    a.alpha = 15;
    a.beta = 18;
    bfs_batched_kernel<<<grid, kBbThreads, smem, s>>>(a);
    GBX_LAUNCH_CHECK();
    GBX_TRY(dist.finish(s));
    GBX_TRY(par.finish(s));
    GBX_TRY(res.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}

extern "C" int gbx_pr_batched(gbx_batch *b, uint32_t max_iterations, double epsilon, float *ranks,
                              gbx_pr_result *results, void *stream) {
    clear_error();
    GBX_REQUIRE(b && ranks, GBX_ERR_INVALID, "batch or ranks is NULL");
    GBX_REQUIRE(epsilon >= 0.0, GBX_ERR_INVALID, "epsilon must be >= 0");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    OutArray<float> out;
    OutArray<gbx_pr_result> res;
    GBX_TRY(out.bind(ranks, b->V, s));
    GBX_TRY(res.bind(results, b->G, s));
    DevBuf<float> other, scratch;
    DevBuf<uint32_t> cursor;
    GBX_TRY(other.alloc(b->V, s));
    GBX_TRY(cursor.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(cursor.p, 0, 4, s));
    const size_t smem = kBpSmemBytes;
    GBX_CUDA(cudaFuncSetAttribute(pr_batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    GBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pr_batched_kernel, kBpThreads, smem));
    const unsigned grid = std::max(1u, std::min<unsigned>((unsigned)num_sms() * std::max(occ, 1), b->G));
    BpArgs a;
    a.scratch = nullptr;
    a.scratch_v = 0;
    if (b->max_v > kBpSmemV) {
        a.scratch_v = b->max_v;
        GBX_TRY(scratch.alloc((size_t)grid * b->max_v, s));
        a.scratch = scratch.p;
    }
    a.G = b->G;
    a.vbase = b->vbase;
    a.off = b->offsets;
    a.poff = b->poff();
    a.psrc = b->psrc();
    a.order = b->order;
    a.ranks = out.d;
    a.rother = other.p;
    a.cursor = cursor.p;
    a.max_it = max_iterations;
    a.epsilon = epsilon;
    a.res = res.d;
    pr_batched_kernel<<<grid, kBpThreads, smem, s>>>(a);
    GBX_LAUNCH_CHECK();
    GBX_TRY(out.finish(s));
    GBX_TRY(res.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}
