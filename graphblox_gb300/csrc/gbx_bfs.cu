// Direction-optimising BFS (the reference's
// breadthFirstSearchDirectionOptimizedGraphCSR, BFS.c:335-485, with the
// top-down step :498-546 and the bottom-up step :562-613), as ONE persistent
// cooperative kernel: the whole traversal, including the direction
// decisions, runs on the device with one grid barrier per step.
//
// State in HBM: level[V] and parent[V] (the output arrays themselves, in the
// reference's format from the start: unreached vertices keep level 0 and
// parent -out_degree or -1, so no conversion pass follows), a visited
// bitmap and two frontier bitmaps (V/8 bytes each, L2-resident), and two
// generations of frontier lists: a queue of vertices with out-degree in
// (0, kHubDeg] and a hub list for larger ones.
//
//  top-down  : warps take work units from an atomic cursor. A unit is either
//              kHubChunk edges of one hub (hubs are cut so no warp serialises
//              a hub's row) or 32 queued vertices whose edges the warp
//              flattens (warp scan of degrees, consecutive lanes on
//              consecutive edges, 4 loads in flight per lane). Unvisited
//              neighbours are claimed with atomicOr on the visited bitmap and
//              appended with one atomic per warp (ballot + popc ranks); a hub
//              is appended with a single 64-bit atomic that returns both its
//              list slot and the first of its edge chunks, so the hub list is
//              born sorted by chunk.
//  bottom-up : one warp per bitmap word (32 vertices); each unvisited lane
//              scans its pull neighbours until one is in the current frontier
//              bitmap (4, then 16 probes in flight; the warp finishes rows
//              longer than kBuProbe together); the ballot is the
//              next-frontier word. Found vertices are also appended to the
//              next generation's queue / hub list, so leaving bottom-up needs
//              no bitmap-to-list pass.
//
// The direction heuristic is the reference's (alpha 15, beta 18, mu/mf/nf in
// uint32 arithmetic). Every CTA evaluates it redundantly from the previous
// step's counters (triple-buffered, so CTA 0 can clear the next slot while
// others still read the last one), which is what lets one barrier per step
// suffice. processed_nodes and iteration therefore match the reference.
#include <algorithm>
#include <cstddef>
#include <vector>

#include "gbx_coop.cuh"

namespace gbx {

constexpr uint32_t kHubDeg = 1024;    // out-degree above which a vertex is a hub
constexpr uint32_t kHubChunk = 1024;  // edges per hub work unit
constexpr uint32_t kBuProbe = 64;     // bottom-up: in-edges a lane probes alone before the warp helps
constexpr uint32_t kTdMaxSplit = 64;  // top-down: most warps sharing one 32-vertex group's edges
constexpr uint32_t kBuWords = 8;      // bottom-up: frontier-bitmap words (32 vertices each) per work unit
constexpr int kBfsThreads = 768;
constexpr int kBfsWarps = kBfsThreads / 32;

struct BfsStep {
    unsigned cursor;          // work-unit cursor
    unsigned nf;              // vertices claimed
    unsigned mf;              // sum over claimed of max(out_degree, 1) (BFS.c:537)
    unsigned qlen;            // next queue length
    unsigned long long hub;   // next hub list: (count << 32) | chunks
    unsigned long long edges; // sum of out_degree over claimed
    unsigned long long busy_sum, busy_max;  // warps' time in the step's phase (traced runs only)
};

// Step trace (printed when GBX_TRACE is set): kind, frontier size, time.
constexpr unsigned kTraceMax = 96;
enum : unsigned { kTrStart = 0, kTrTopDown = 1, kTrBottomUp = 2, kTrToBitmap = 3, kTrToLists = 4 };
struct TraceRec {
    unsigned kind, value;
    unsigned long long ns, busy_sum, busy_max;
};

// One traversal's results where the host collects them after a run of
// traversals (gbx_bfs_trials): the final counters and the error words.
struct BfsSlot {
    unsigned processed, iteration, td_steps, bu_steps, depth, status, timeout, pad;
    unsigned long long edges_total;
};

struct BfsState {
    GridSync gs;
    BfsStep step[3];
    BfsStep conv;  // lists rebuilt from a bitmap when leaving bottom-up
    unsigned processed, iteration, td_steps, bu_steps, depth, status;
    unsigned long long edges_total;
    unsigned ntrace, pad2;
    TraceRec trace[kTraceMax];
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void trace_step(BfsState *st, unsigned kind, unsigned value,
                                           const BfsStep *step = nullptr) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && st->ntrace < kTraceMax) {
        TraceRec &r = st->trace[st->ntrace++];
        r.kind = kind;
        r.value = value;
        r.ns = global_ns();
        r.busy_sum = step ? __ldcg(&step->busy_sum) : 0;
        r.busy_max = step ? __ldcg(&step->busy_max) : 0;
    }
}

// Traced runs: each warp's time inside a step's phase, summed and maxed over
// warps, tells a load-imbalanced step (max close to the step) from a
// throughput-bound one (mean close to the step).
struct BusyClock {
    bool on;
    unsigned long long t0;
    __device__ __forceinline__ explicit BusyClock(bool trace) : on(trace), t0(trace ? global_ns() : 0) {}
    __device__ __forceinline__ void stop(BfsStep *cnt) {
        if (!on || (threadIdx.x & 31) != 0) return;
        const unsigned long long d = global_ns() - t0;
        atomicAdd(&cnt->busy_sum, d);
        atomicMax(&cnt->busy_max, d);
    }
};

struct BfsArgs {
    const uint32_t *off, *dest, *poff, *psrc, *outdeg;
    uint32_t V, words, E, mode, source;
    uint32_t alpha, beta;  // direction switch: bottom-up when mf > mu/alpha, stay while nf > V/beta
    uint32_t pull_live;    // every pull neighbour has out-degree > 0
    uint32_t trace;        // record per-step warp busy times
    const uint32_t *live;  // bit v: v has pull in-edges (only such vertices can be found bottom-up)
    uint32_t *level;
    int32_t *parent;
    uint32_t *visited;
    uint32_t *bm[2];
    uint32_t *q[2];
    uint32_t *hv[2];
    uint32_t *hc[2];
    BfsState *st;
    BfsSlot *slot;  // NULL, or where this traversal's results are copied at its end
};

__device__ __forceinline__ uint32_t hub_chunks(uint32_t d) { return (d + kHubChunk - 1) / kHubChunk; }

// Claim u (reached from v) at level lnext; all lanes call together.
struct Claimer {
    const BfsArgs &a;
    uint32_t lnext;
    uint32_t *qout, *hvout, *hcout;
    uint32_t *fbm;  // frontier bitmap of level lnext to fill, or null
    BfsStep *cnt;
    WarpQueue wq;
    unsigned nf = 0, mf = 0;
    unsigned long long edges = 0;
    __device__ __forceinline__ Claimer(const BfsArgs &a_, uint32_t l, uint32_t *q, uint32_t *hv, uint32_t *hc,
                                       uint32_t *f, BfsStep *c, uint32_t *wbuf)
        : a(a_), lnext(l), qout(q), hvout(hv), hcout(hc), fbm(f), cnt(c), wq(wbuf) {}
    // Four candidate edges per lane: the visited-word loads and the
    // targets' out-degrees (needed only by the winners, but loading them
    // here takes them off the claim's dependent chain), then the atomicOr
    // claims, are issued back to back so their latencies overlap.
    __device__ __forceinline__ void claim4(const uint32_t (&v)[4], const uint32_t (&u)[4], const bool (&act)[4]) {
        uint32_t pre[4], old[4], du[4], dpre[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            pre[q] = act[q] ? __ldcg(a.visited + (u[q] >> 5)) : 0xFFFFFFFFu;
            dpre[q] = act[q] ? __ldg(a.outdeg + u[q]) : 0u;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t bit = 1u << (u[q] & 31);
            old[q] = (act[q] && !(pre[q] & bit)) ? atomicOr(a.visited + (u[q] >> 5), bit) : 0xFFFFFFFFu;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const bool won = !(old[q] & (1u << (u[q] & 31)));
            du[q] = won ? dpre[q] : 0u;
            if (won) {
                a.level[u[q]] = lnext;
                a.parent[u[q]] = (int32_t)v[q];
                if (fbm) atomicOr(fbm + (u[q] >> 5), 1u << (u[q] & 31));
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const bool won = !(old[q] & (1u << (u[q] & 31)));
            bool push = false;
            if (won) {
                nf += 1;
                mf += du[q] ? du[q] : 1u;
                edges += du[q];
                if (du[q] > kHubDeg) {
                    unsigned long long h = atomicAdd(&cnt->hub, (1ull << 32) | hub_chunks(du[q]));
                    uint32_t slot = (uint32_t)(h >> 32);
                    hvout[slot] = u[q];
                    hcout[slot] = (uint32_t)h;
                } else {
                    push = du[q] > 0;
                }
            }
            wq.push(u[q], push, qout, &cnt->qlen);
        }
    }
    __device__ __forceinline__ void flush() {
        wq.flush(qout, &cnt->qlen);
        unsigned n = warp_sum(nf), f = warp_sum(mf);
        unsigned long long e = warp_sum(edges);
        if ((threadIdx.x & 31) == 0 && n) {
            atomicAdd(&cnt->nf, n);
            atomicAdd(&cnt->mf, f);
            atomicAdd(&cnt->edges, e);
        }
    }
};

// Position of the r-th set bit (from 0) of m; m has more than r set bits.
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t r) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t w = 16; w >= 1; w >>= 1) {
        const uint32_t low = __popc((m >> pos) & ((1u << w) - 1u));
        if (r >= low) {
            r -= low;
            pos += w;
        }
    }
    return pos;
}

__device__ void top_down_phase(const BfsArgs &a, const uint32_t *qin, uint32_t qn, const uint32_t *hvin,
                               const uint32_t *hcin, uint32_t nh, uint32_t nc, BfsStep *cur, uint32_t *qout,
                               uint32_t *hvout, uint32_t *hcout, uint32_t lnext, uint32_t *fbm, uint32_t *clear_bm,
                               uint32_t *s_pre, uint32_t *s_base, uint32_t *s_v, uint32_t *s_wq) {
    const uint32_t lane = threadIdx.x & 31;
    BusyClock clock(a.trace != 0);
    if (clear_bm) {
        // the bitmap the next top-down step fills (not read during this one)
        for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < a.words; w += gridDim.x * blockDim.x)
            clear_bm[w] = 0u;
    }
    Claimer claim(a, lnext, qout, hvout, hcout, fbm, cur, s_wq);
    // a frontier with fewer 32-vertex groups than warps cuts each group's
    // edges into `split` interleaved parts of 128-edge batches
    // Work units: a frontier with few units per warp cuts each 32-vertex
    // group's edges into `split` interleaved parts of 128-edge batches and
    // each hub chunk's batches into `hsplit` parts (a small step's work is
    // then not one warp's serial chain); the group parts are dealt first,
    // the hub chunks after them.
    const uint32_t groups = (qn + 31) / 32;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t split = groups ? max(1u, min(kTdMaxSplit, nwarps / groups)) : 1u;
    const uint32_t hsplit = nc ? max(1u, min(kHubChunk / 128, nwarps / nc)) : 1u;
    const uint32_t gunits = groups * split;
    const uint32_t units = gunits + nc * hsplit;
    UnitDealer dealer(&cur->cursor);
    for (;;) {
        const uint32_t unit = dealer.take(units);
        if (unit >= units) break;
        if (unit >= gunits) {
            // kHubChunk edges of one hub (every hsplit-th batch of them)
            const uint32_t chunk = (unit - gunits) / hsplit, hpart = (unit - gunits) % hsplit;
            const uint32_t h = warp_chunk_owner(hcin, nh, chunk);
            const uint32_t v = __ldcg(hvin + h);
            const uint32_t rb = __ldg(a.off + v), re = __ldg(a.off + v + 1);
            const uint32_t cb = rb + (chunk - __ldcg(hcin + h)) * kHubChunk;
            const uint32_t ce = min(cb + kHubChunk, re);
            // the next batch's ids are loaded before this batch is claimed
            const uint32_t stride = hsplit * 128;
            uint32_t un[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t j = cb + hpart * 128 + q * 32 + lane;
                un[q] = j < ce ? __ldg(a.dest + j) : 0u;
            }
            for (uint32_t j0 = cb + hpart * 128; j0 < ce; j0 += stride) {
                uint32_t u[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    u[q] = un[q];
                    const uint32_t j = j0 + stride + q * 32 + lane;
                    un[q] = j < ce ? __ldg(a.dest + j) : 0u;
                }
                const uint32_t vv[4] = {v, v, v, v};
                const bool act[4] = {j0 + lane < ce, j0 + 32 + lane < ce, j0 + 64 + lane < ce, j0 + 96 + lane < ce};
                claim.claim4(vv, u, act);
            }
        } else {
            // 32 queued vertices, edges flattened over the warp (one part)
            const uint32_t group = unit / split, part = unit % split;
            const uint32_t qi = group * 32 + lane;
            uint32_t v = 0, b = 0, d = 0;
            if (qi < qn) {
                v = __ldcg(qin + qi);
                b = __ldg(a.off + v);
                d = __ldg(a.off + v + 1) - b;
            }
            uint32_t incl = d;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += t;
            }
            s_pre[lane] = incl - d;
            s_base[lane] = b;
            s_v[lane] = v;
            if (lane == 31) s_pre[32] = incl;
            __syncwarp();
            const uint32_t tot = s_pre[32];
            // each batch's ids are loaded one batch ahead (k: owner lane of
            // the loading stream, advanced monotonically)
            uint32_t k = 0;
            uint32_t un[4], sn[4];
            auto load = [&](uint32_t i0, uint32_t (&uu)[4], uint32_t (&ss)[4]) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint32_t i = i0 + q * 32 + lane;
                    uu[q] = 0;
                    ss[q] = 0;
                    if (i < tot) {
                        while (s_pre[k + 1] <= i) ++k;
                        ss[q] = s_v[k];
                        uu[q] = __ldg(a.dest + s_base[k] + (i - s_pre[k]));
                    }
                }
            };
            load(part * 128, un, sn);
            for (uint32_t i0 = part * 128; i0 < tot; i0 += split * 128) {
                uint32_t u[4], src[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    u[q] = un[q];
                    src[q] = sn[q];
                }
                load(i0 + split * 128, un, sn);
                const bool act[4] = {i0 + lane < tot, i0 + 32 + lane < tot, i0 + 64 + lane < tot, i0 + 96 + lane < tot};
                claim.claim4(src, u, act);
            }
            __syncwarp();
        }
    }
    claim.flush();
    clock.stop(cur);
}

// Probe in-edges [j, el) of one vertex, N at a time: the ids, then their
// frontier words, are loaded back to back; returns the first frontier member
// or 0xFFFFFFFF. The frontier bitmap is read through L1: it was written in
// the previous step, and the grid barrier's acquire orders those writes
// before these loads.
template <int N>
__device__ __forceinline__ uint32_t bu_probe(const BfsArgs &a, const uint32_t *cur_bm, uint32_t j, uint32_t el) {
    uint32_t u[N], fw[N];
#pragma unroll
    for (int q = 0; q < N; ++q) u[q] = (j + q < el) ? __ldg(a.psrc + j + q) : 0u;
#pragma unroll
    for (int q = 0; q < N; ++q) fw[q] = (j + q < el) ? cur_bm[u[q] >> 5] : 0u;
    uint32_t pick = 0xFFFFFFFFu;
#pragma unroll
    for (int q = N - 1; q >= 0; --q)
        if ((fw[q] >> (u[q] & 31)) & 1u) pick = u[q];
    return pick;
}

// One bottom-up step. A work unit is kBuWords frontier-bitmap words; its
// candidates -- vertices not yet visited that have pull in-edges (the live
// bitmap), the only ones a bottom-up step can find -- are numbered word by
// word and dealt to the lanes 32 at a time, so a lane never idles on a
// visited or edgeless vertex. Each lane probes its candidate's in-edges
// until one is in the current frontier bitmap (4, then 16 in flight; the
// warp finishes rows longer than kBuProbe together). The found bits of the
// unit's words are gathered in shared memory and written once, with the
// next-frontier word of every word of the unit (zero when nothing was
// found). Found vertices are also appended to the next generation's queue /
// hub list, so leaving bottom-up needs no bitmap-to-list pass.
__device__ void bottom_up_phase(const BfsArgs &a, const uint32_t *cur_bm, uint32_t *next_bm, uint32_t lnext,
                                BfsStep *cnt, uint32_t *qout, uint32_t *hvout, uint32_t *hcout, uint32_t *s_wq,
                                uint32_t *s_found) {
    const uint32_t lane = threadIdx.x & 31;
    BusyClock clock(a.trace != 0);
    unsigned nf = 0;
    unsigned long long edges = 0;
    WarpQueue wq(s_wq);
    const uint32_t units = (a.words + kBuWords - 1) / kBuWords;
    UnitDealer dealer(&cnt->cursor);
    for (uint32_t unit = dealer.take(units); unit < units; unit = dealer.take(units)) {
        const uint32_t w0 = unit * kBuWords;
        const uint32_t nw = min(a.words - w0, kBuWords);
        // lane k < nw holds word w0 + k (only this warp writes these words in the step)
        const uint32_t vis = lane < nw ? __ldcg(a.visited + w0 + lane) : 0xFFFFFFFFu;
        const uint32_t cand = lane < nw ? (~vis & __ldg(a.live + w0 + lane)) : 0u;
        const uint32_t c = __popc(cand);
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += t;
        }
        const uint32_t excl = incl - c, total = __shfl_sync(0xffffffffu, incl, 31);
        if (lane < kBuWords) s_found[lane] = 0u;
        __syncwarp();
        // candidate i -> (its word k, its vertex, that vertex's row bounds and
        // out-degree); the next round's rows are loaded while this round probes
        auto candidate = [&](uint32_t i, uint32_t &k, uint32_t &v, uint32_t &b, uint32_t &e, uint32_t &dv) {
            k = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xffffffffu, excl, k + step) <= i) k += step;
            const uint32_t mk = __shfl_sync(0xffffffffu, cand, k);
            const uint32_t ek = __shfl_sync(0xffffffffu, excl, k);
            v = b = e = dv = 0;
            if (i < total) {
                v = (w0 + k) * 32 + nth_set_bit(mk, i - ek);
                b = __ldg(a.poff + v);
                e = __ldg(a.poff + v + 1);
                dv = __ldg(a.outdeg + v);
            }
        };
        uint32_t nk, nv_, nb, ne, nd;
        candidate(lane, nk, nv_, nb, ne, nd);
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t i = base + lane;
            const bool act = i < total;
            const uint32_t k = nk, v = nv_, b = nb, e = ne, dv = nd;
            if (base + 32 < total) candidate(base + 32 + lane, nk, nv_, nb, ne, nd);
            bool found = false;
            uint32_t tb = 0, te = 0;  // in-edges still to probe after the lane's own first kBuProbe
            if (act) {
                const uint32_t el = min(e, b + kBuProbe);
                // a short first round (most vertices that have a frontier
                // in-neighbour meet it among their first few), then wide rounds
                uint32_t pu = bu_probe<4>(a, cur_bm, b, el);
                for (uint32_t j = b + 4; pu == 0xFFFFFFFFu && j < el; j += 16) pu = bu_probe<16>(a, cur_bm, j, el);
                if (pu != 0xFFFFFFFFu) {
                    a.level[v] = lnext;
                    a.parent[v] = (int32_t)pu;
                    found = true;
                } else if (el < e) {
                    tb = el;
                    te = e;
                }
            }
            // rows longer than kBuProbe that found nothing in their first part:
            // the whole warp scans the rest, 128 in-edges per step, one row at a time
            for (unsigned tv = __ballot_sync(0xffffffffu, tb < te); tv; tv &= tv - 1) {
                const uint32_t owner = __ffs(tv) - 1;
                const uint32_t hb = __shfl_sync(0xffffffffu, tb, owner), he = __shfl_sync(0xffffffffu, te, owner);
                for (uint32_t j0 = hb; j0 < he; j0 += 128) {
                    uint32_t u[4], fw[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint32_t j = j0 + q * 32 + lane;
                        u[q] = j < he ? __ldg(a.psrc + j) : 0u;
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) fw[q] = j0 + q * 32 + lane < he ? cur_bm[u[q] >> 5] : 0u;
                    uint32_t pick = 0xFFFFFFFFu;
#pragma unroll
                    for (int q = 3; q >= 0; --q)
                        if ((fw[q] >> (u[q] & 31)) & 1u) pick = u[q];
                    const unsigned hm = __ballot_sync(0xffffffffu, pick != 0xFFFFFFFFu);
                    if (hm) {
                        const uint32_t pu = __shfl_sync(0xffffffffu, pick, __ffs(hm) - 1);
                        if (lane == owner) {
                            a.level[v] = lnext;
                            a.parent[v] = (int32_t)pu;
                            found = true;
                        }
                        break;
                    }
                }
            }
            if (found) {
                atomicOr(s_found + k, 1u << (v & 31));
                edges += dv;
                if (dv > kHubDeg) {
                    const unsigned long long h = atomicAdd(&cnt->hub, (1ull << 32) | hub_chunks(dv));
                    const uint32_t slot = (uint32_t)(h >> 32);
                    hvout[slot] = v;
                    hcout[slot] = (uint32_t)h;
                }
            }
            // the vertices found also form the next step's lists, in case the
            // traversal returns to top-down after this step (bitmapToArrayQueue)
            wq.push(v, found && dv > 0 && dv <= kHubDeg, qout, &cnt->qlen);
        }
        __syncwarp();
        if (lane < nw) {
            const uint32_t m = s_found[lane];
            next_bm[w0 + lane] = m;
            if (m) a.visited[w0 + lane] = vis | m;
            nf += __popc(m);
        }
        __syncwarp();
    }
    wq.flush(qout, &cnt->qlen);
    nf = warp_sum(nf);
    edges = warp_sum(edges);
    if (lane == 0 && (nf || edges)) {
        atomicAdd(&cnt->nf, nf);
        atomicAdd(&cnt->edges, edges);
    }
    clock.stop(cnt);
}

// arrayQueueToBitmap (arrayQueue.c:284-308) from the lists themselves, into a
// bitmap that is still all zero: the queue and hub lists hold every frontier
// vertex with out-degree > 0, and the caller checks that the others cannot
// matter (no other frontier vertex, or no pull neighbour of out-degree 0).
__device__ void lists_to_bitmap_phase(const uint32_t *qin, uint32_t qn, const uint32_t *hvin, uint32_t nh,
                                      uint32_t *bm) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    for (uint32_t i = tid; i < qn + nh; i += nt) {
        const uint32_t v = i < qn ? __ldcg(qin + i) : __ldcg(hvin + (i - qn));
        atomicOr(bm + (v >> 5), 1u << (v & 31));
    }
}

__device__ void level_to_bitmap_phase(const BfsArgs &a, uint32_t l, uint32_t *bm) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w0 = gw; w0 < a.words; w0 += 4 * nw) {
        uint32_t lv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t v = (w0 + q * nw) * 32 + lane;
            lv[q] = (w0 + q * nw < a.words && v < a.V) ? __ldcg(a.level + v) : kInfLevel;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            // unreached vertices also hold level 0: the visited word keeps
            // them out of level 0's frontier
            const uint32_t vis = w0 + q * nw < a.words ? __ldcg(a.visited + w0 + q * nw) : 0u;
            const unsigned m = __ballot_sync(0xffffffffu, lv[q] == l) & vis;
            if (lane == 0 && w0 + q * nw < a.words) bm[w0 + q * nw] = m;
        }
    }
}

__device__ __forceinline__ void zero_step(BfsStep *s) {
    s->cursor = 0;
    s->nf = 0;
    s->mf = 0;
    s->qlen = 0;
    s->hub = 0;
    s->edges = 0;
    s->busy_sum = 0;
    s->busy_max = 0;
}

__global__ void __launch_bounds__(kBfsThreads, 1) bfs_persistent_kernel(BfsArgs a) {
    __shared__ uint32_t s_pre[kBfsWarps][33];
    __shared__ uint32_t s_base[kBfsWarps][32];
    __shared__ uint32_t s_v[kBfsWarps][32];
    __shared__ uint32_t s_wq[kBfsWarps][kWarpQueueCap];
    __shared__ uint32_t s_found[kBfsWarps][kBuWords];
    __shared__ BfsStep s_cnt;  // the finished step's counters (fetch_counters)
    const uint32_t wid = threadIdx.x >> 5;
    BfsState *st = a.st;
    grid_barrier_init();
    const uint32_t alpha = a.alpha, beta = a.beta;
    // DO bookkeeping, evaluated identically by every CTA
    uint32_t mu = a.E, mf = __ldg(a.outdeg + a.source), qsize = 1, nf_prev = 0, L = 0;
    uint32_t processed = 1, iteration = 1, td = 0, bu = 0;
    unsigned long long edges_total = __ldg(a.outdeg + a.source);
    bool in_bu = false, done = false, failed = false;
    bool bm_clean[2] = {true, true};  // frontier bitmaps still all zero (cleared by bfs_init_kernel)
    // Until the first bottom-up step, top-down steps also set the bits of the
    // vertices they claim in the next frontier bitmap (and clear the other
    // bitmap for the step after), so the switch to bottom-up finds the
    // frontier bitmap ready (bm_ready) and needs no conversion pass.
    bool bm_track = a.mode == 2, bm_ready = false;
    const uint32_t max_steps = 2 * a.V + 16;
    // lists for step 0: prepared by the host in generation 0
    uint32_t qn = __ldcg(&st->conv.qlen);
    unsigned long long hub0 = __ldcg(&st->conv.hub);
    uint32_t nh = (uint32_t)(hub0 >> 32), nc = (uint32_t)hub0;
    trace_step(st, kTrStart, 1);
    for (uint32_t s = 0; !done; ++s) {
        if (s >= max_steps) {
            failed = true;
            break;
        }
        BfsStep *cur = &st->step[s % 3];
        if (blockIdx.x == 0 && threadIdx.x == 0) zero_step(&st->step[(s + 1) % 3]);
        const uint32_t ib = s & 1, ob = ib ^ 1;
        bool use_bu;
        if (a.mode == 0) {
            use_bu = true;
        } else if (a.mode == 1) {
            use_bu = false;
        } else if (in_bu) {
            use_bu = true;  // still inside the reference's do { } while loop
        } else {
            use_bu = mf > mu / alpha;
        }
        if (use_bu) {
            if (!in_bu) {
                if (!bm_ready) {
                    // arrayQueueToBitmap: frontier bitmap of the current level,
                    // scattered from the lists when they hold the whole frontier
                    // and the bitmap is still clear, else from level[]
                    if (bm_clean[ib] && (a.pull_live || qsize == qn + nh))
                        lists_to_bitmap_phase(a.q[ib], qn, a.hv[ib], nh, a.bm[ib]);
                    else
                        level_to_bitmap_phase(a, L, a.bm[ib]);
                    if (!grid_barrier(&st->gs)) { failed = true; break; }
                    trace_step(st, kTrToBitmap, qsize);
                }
                bm_clean[ib] = false;
                bm_track = bm_ready = false;
                nf_prev = qsize;
                in_bu = true;
            }
            bottom_up_phase(a, a.bm[ib], a.bm[ob], L + 1, cur, a.q[ob], a.hv[ob], a.hc[ob], s_wq[wid],
                            s_found[wid]);
            bm_clean[ob] = false;
            if (!grid_barrier(&st->gs)) { failed = true; break; }
            fetch_counters(cur, &s_cnt);
            const uint32_t nf = s_cnt.nf;
            trace_step(st, kTrBottomUp, nf, cur);
            processed += nf;
            iteration++;
            bu++;
            edges_total += s_cnt.edges;
            if (nf) L++;
            bool again = a.mode == 0 ? nf > 0 : (nf > nf_prev || nf > a.V / beta);
            nf_prev = nf;
            if (!again) {
                in_bu = false;
                qsize = nf;
                if (nf == 0 || a.mode == 0) {
                    done = true;
                } else {
                    // bitmapToArrayQueue: the step itself wrote the lists of
                    // generation s+1
                    qn = s_cnt.qlen;
                    unsigned long long hb = s_cnt.hub;
                    nh = (uint32_t)(hb >> 32);
                    nc = (uint32_t)hb;
                    mf = 1;
                }
            }
        } else {
            mu -= mf;
            // bm[ob] is clear here while tracking: bfs_init_kernel cleared both
            // bitmaps, and each tracking step clears bm[ib] for the next one
            top_down_phase(a, a.q[ib], qn, a.hv[ib], a.hc[ib], nh, nc, cur, a.q[ob], a.hv[ob], a.hc[ob], L + 1,
                           bm_track ? a.bm[ob] : nullptr, bm_track && s > 0 ? a.bm[ib] : nullptr, s_pre[wid],
                           s_base[wid], s_v[wid], s_wq[wid]);
            if (bm_track) {
                bm_clean[ob] = false;
                bm_clean[ib] = true;
                bm_ready = true;
            }
            if (!grid_barrier(&st->gs)) { failed = true; break; }
            fetch_counters(cur, &s_cnt);
            const uint32_t nf = s_cnt.nf;
            trace_step(st, kTrTopDown, nf, cur);
            mf = s_cnt.mf;
            qsize = nf;
            processed += nf;
            iteration++;
            td++;
            edges_total += s_cnt.edges;
            qn = s_cnt.qlen;
            unsigned long long hb = s_cnt.hub;
            nh = (uint32_t)(hb >> 32);
            nc = (uint32_t)hb;
            if (nf) L++;
            if (qsize == 0) done = true;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->processed = processed;
        st->iteration = iteration;
        st->td_steps = td;
        st->bu_steps = bu;
        st->depth = L;
        st->edges_total = edges_total;
        st->status = failed ? 1u : 0u;
        if (a.slot) {
            BfsSlot &o = *a.slot;
            o.processed = processed;
            o.iteration = iteration;
            o.td_steps = td;
            o.bu_steps = bu;
            o.depth = L;
            o.edges_total = edges_total;
            o.status = failed ? 1u : 0u;
            o.timeout = ld_acquire_u32(&st->gs.error);
        }
    }
}

// Per traversal: levels, parents, visited and both frontier bitmaps, the
// traversal state (zeroed as 32-bit words by the grid), and the generation-0
// lists: the source alone, as a hub when its degree is large. The state
// words that hold those lists are written only by thread 0, after its own
// share of the zeroing.
__global__ void bfs_init_kernel(uint32_t *level, int32_t *parent, uint32_t *visited, uint32_t *bm0,
                                uint32_t *bm1, uint32_t V, uint32_t words, uint32_t source,
                                const uint32_t *outdeg, uint32_t *q0, uint32_t *hv0, uint32_t *hc0,
                                BfsState *st) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    for (uint32_t v = tid; v < V; v += nt) {
        // the reference's values for unreached vertices (BFS.c:59-74); the
        // traversal overwrites the reached ones
        const uint32_t d = __ldg(outdeg + v);
        level[v] = 0u;
        parent[v] = v == source ? (int32_t)source : (d ? -(int32_t)d : -1);
    }
    for (uint32_t w = tid; w < words; w += nt) {
        visited[w] = (w == (source >> 5)) ? (1u << (source & 31)) : 0u;
        bm0[w] = 0;
        bm1[w] = 0;
    }
    static_assert(sizeof(BfsState) % 4 == 0, "state is zeroed as words");
    constexpr uint32_t kStateWords = sizeof(BfsState) / 4;
    uint32_t *sw = reinterpret_cast<uint32_t *>(st);
    const uint32_t conv_lo = (uint32_t)(offsetof(BfsState, conv) / 4);
    const uint32_t conv_hi = conv_lo + (uint32_t)(sizeof(BfsStep) / 4);
    for (uint32_t i = tid; i < kStateWords; i += nt)
        if (i < conv_lo || i >= conv_hi) sw[i] = 0u;
    if (tid == 0) {
        const uint32_t d = outdeg[source];
        BfsStep c = {};
        if (d > kHubDeg) {
            hv0[0] = source;
            hc0[0] = 0;
            c.hub = (1ull << 32) | hub_chunks(d);
        } else if (d > 0) {
            q0[0] = source;
            c.qlen = 1;
        }
        st->conv = c;
    }
}

// live[w] bit b: vertex 32w + b exists and has pull in-edges
__global__ void live_bits_kernel(const uint32_t *poff, uint32_t V, uint32_t words, uint32_t *live) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += nw) {
        const uint32_t v = w * 32 + lane;
        const bool has = v < V && __ldg(poff + v + 1) > __ldg(poff + v);
        const unsigned m = __ballot_sync(0xffffffffu, has);
        if (lane == 0) live[w] = m;
    }
}

// sets *bad when some pull neighbour has out-degree 0
__global__ void pull_live_kernel(const uint32_t *psrc, uint32_t E, const uint32_t *outdeg, uint32_t *bad) {
    bool dead = false;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < E; j += gridDim.x * blockDim.x)
        dead |= __ldg(outdeg + __ldcs(psrc + j)) == 0;
    if (__any_sync(0xffffffffu, dead) && (threadIdx.x & 31) == 0) *bad = 1;
}

// Working arrays of one traversal, carved from the graph's scratch arena;
// the last two are staging for host-memory outputs.
struct BfsWork {
    uint32_t *level, *visited, *bm0, *bm1, *q0, *q1, *hv0, *hv1, *hc0, *hc1, *dist_stage;
    int32_t *parent, *par_stage;
    BfsState *st;
    static size_t bytes(uint32_t V, bool stage) {
        const size_t words = (V + 31) / 32, r = Scratch::round_up((size_t)V * 4);
        return 8 * r + 3 * Scratch::round_up(words * 4) + (stage ? 2 * r : 0) +
               Scratch::round_up(sizeof(BfsState));
    }
    int carve(Scratch &sc, uint32_t V, bool stage) {
        const size_t words = (V + 31) / 32;
        level = sc.carve<uint32_t>(V);
        parent = sc.carve<int32_t>(V);
        visited = sc.carve<uint32_t>(words);
        bm0 = sc.carve<uint32_t>(words);
        bm1 = sc.carve<uint32_t>(words);
        q0 = sc.carve<uint32_t>(V);
        q1 = sc.carve<uint32_t>(V);
        hv0 = sc.carve<uint32_t>(V);
        hv1 = sc.carve<uint32_t>(V);
        hc0 = sc.carve<uint32_t>(V);
        hc1 = sc.carve<uint32_t>(V);
        dist_stage = stage ? sc.carve<uint32_t>(V) : nullptr;
        par_stage = stage ? sc.carve<int32_t>(V) : nullptr;
        st = sc.carve<BfsState>(1);
        GBX_REQUIRE(st != nullptr, GBX_ERR_CUDA, "BFS scratch carve overflow");
        return GBX_OK;
    }
};

// Graph-level set-up shared by every traversal of the graph: whether every
// pull source has out-edges, and the bitmap of vertices with pull in-edges.
int bfs_graph_setup(gbx_graph *g, cudaStream_t s) {
    const uint32_t V = g->V, words = (V + 31) / 32;
    if (g->pull_sources_live < 0) {
        DevBuf<uint32_t> bad;
        GBX_TRY(bad.alloc(1, s));
        GBX_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
        if (g->E) {
            pull_live_kernel<<<std::min<unsigned>(ceil_div(g->E, 256), (unsigned)num_sms() * 8), 256, 0, s>>>(
                g->pull_src(), g->E, g->out_degree, bad.p);
            GBX_LAUNCH_CHECK();
        }
        uint32_t h = 0;
        GBX_CUDA(cudaMemcpyAsync(&h, bad.p, 4, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        g->pull_sources_live = h ? 0 : 1;
    }
    if (!g->bu_live) {
        // kept with the graph: which vertices a bottom-up step can find
        void *live = nullptr;
        GBX_TRY(dev_alloc(&live, (size_t)words * 4, s));
        g->bu_live = static_cast<uint32_t *>(live);
        live_bits_kernel<<<std::min<unsigned>(ceil_div(words * 32, 256), (unsigned)num_sms() * 8), 256, 0, s>>>(
            g->pull_offsets(), V, words, g->bu_live);
        GBX_LAUNCH_CHECK();
    }
    return GBX_OK;
}

// One traversal from `source` on stream s: the init kernel, then the
// persistent kernel, levels into lev and parents into parp (device arrays
// of V entries).
int bfs_enqueue(gbx_graph *g, const BfsWork &w, uint32_t source, int mode, uint32_t *lev, int32_t *parp,
                BfsSlot *slot, cudaStream_t s) {
    const uint32_t V = g->V, words = (V + 31) / 32;
    const unsigned grid1 = std::min<unsigned>(ceil_div(V, 256), (unsigned)num_sms() * 8);
    bfs_init_kernel<<<grid1, 256, 0, s>>>(lev, parp, w.visited, w.bm0, w.bm1, V, words, source, g->out_degree,
                                          w.q0, w.hv0, w.hc0, w.st);
    GBX_LAUNCH_CHECK();
    BfsArgs a;
    a.off = g->offsets;
    a.dest = g->dest;
    a.poff = g->pull_offsets();
    a.psrc = g->pull_src();
    a.outdeg = g->out_degree;
    a.V = V;
    a.words = words;
    a.E = g->E;
    a.mode = (uint32_t)mode;
    a.source = source;
    a.alpha = g->bfs_alpha;
    a.beta = g->bfs_beta;
    a.pull_live = g->pull_sources_live == 1 ? 1u : 0u;
    a.live = g->bu_live;
    a.trace = trace_enabled() ? 1u : 0u;
    a.level = lev;
    a.parent = parp;
    a.visited = w.visited;
    a.bm[0] = w.bm0;
    a.bm[1] = w.bm1;
    a.q[0] = w.q0;
    a.q[1] = w.q1;
    a.hv[0] = w.hv0;
    a.hv[1] = w.hv1;
    a.hc[0] = w.hc0;
    a.hc[1] = w.hc1;
    a.st = w.st;
    a.slot = slot;
    int grid = 0;
    static int grid_cache[64] = {0};
    GBX_TRY(coop_grid(bfs_persistent_kernel, kBfsThreads, 0, &grid, &grid_cache));
    void *args[] = {&a};
    GBX_CUDA(cudaLaunchCooperativeKernel((const void *)bfs_persistent_kernel, grid, kBfsThreads, args, 0, s));
    GBX_LAUNCH_CHECK();
    return GBX_OK;
}

void bfs_fill_result(gbx_bfs_result *r, unsigned processed, unsigned iteration, unsigned depth, unsigned td,
                     unsigned bu, unsigned long long edges) {
    r->processed_nodes = processed;
    r->iteration = iteration;
    r->depth = depth;
    r->top_down_steps = td;
    r->bottom_up_steps = bu;
    r->reserved = 0;
    r->edges_traversed = edges;
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
    const uint32_t V = g->V;
    const int dist_dev = distances ? (is_device_ptr(distances) ? 1 : 0) : 1;
    const int par_dev = parents ? (is_device_ptr(parents) ? 1 : 0) : 1;
    const bool stage = !dist_dev || !par_dev;
    Scratch sc;
    GBX_TRY(sc.take(g, BfsWork::bytes(V, stage), s));
    BfsWork w;
    GBX_TRY(w.carve(sc, V, stage));
    OutArray<uint32_t> dist;
    OutArray<int32_t> par;
    GBX_TRY(dist.bind(distances, V, s, w.dist_stage, dist_dev));
    GBX_TRY(par.bind(parents, V, s, w.par_stage, par_dev));
    GBX_TRY(bfs_graph_setup(g, s));
    // levels and parents live in the output arrays (device memory, or their
    // device staging) when the caller asked for them
    GBX_TRY(bfs_enqueue(g, w, source, mode, dist.d ? dist.d : w.level, par.d ? par.d : w.parent, nullptr, s));
    GBX_TRY(dist.finish(s));
    GBX_TRY(par.finish(s));
    // the counters (and the step trace only when it is printed)
    BfsState hs;
    GBX_CUDA(cudaMemcpyAsync(&hs, w.st, trace_enabled() ? sizeof(hs) : offsetof(BfsState, trace),
                             cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    GBX_REQUIRE(hs.gs.error == 0, GBX_ERR_DEVICE_TIMEOUT, "BFS grid barrier wait expired");
    GBX_REQUIRE(hs.status == 0, GBX_ERR_ITER_CAP, "BFS step cap reached");
    if (trace_enabled()) {
        static const char *names[] = {"start", "TD", "BU", "->bitmap", "->lists"};
        int grid = 0;
        static int grid_cache[64] = {0};
        GBX_TRY(coop_grid(bfs_persistent_kernel, kBfsThreads, 0, &grid, &grid_cache));
        const unsigned nwarps = (unsigned)grid * (kBfsThreads / 32);
        fprintf(stderr, "| gbx_bfs source %u: %-9s | %-10s | %-10s | %-12s | %-12s |\n", source, "step", "vertices",
                "us", "warp max us", "warp mean us");
        for (unsigned i = 1; i < hs.ntrace && i < kTraceMax; ++i)
            fprintf(stderr, "| %-23s | %-10u | %-10.2f | %-12.2f | %-12.2f |\n", names[hs.trace[i].kind % 5],
                    hs.trace[i].value, (hs.trace[i].ns - hs.trace[i - 1].ns) * 1e-3, hs.trace[i].busy_max * 1e-3,
                    hs.trace[i].busy_sum * 1e-3 / nwarps);
    }
    if (result)
        bfs_fill_result(result, hs.processed, hs.iteration, hs.depth, hs.td_steps, hs.bu_steps, hs.edges_total);
    return GBX_OK;
}

// A second stream and two pairs of events for copies that overlap the next
// trial: done[b] marks a trial's output in staging buffer b as complete,
// copied[b] marks its copy to the host as finished. The destructor waits for
// the copy stream, so staging buffers are never released under a copy.
struct CopyLane {
    cudaStream_t cs = nullptr;
    cudaEvent_t done[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
    int create() {
        GBX_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            GBX_CUDA(cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming));
            GBX_CUDA(cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming));
        }
        return GBX_OK;
    }
    ~CopyLane() {
        if (cs) cudaStreamSynchronize(cs);
        for (int b = 0; b < 2; ++b) {
            if (done[b]) cudaEventDestroy(done[b]);
            if (copied[b]) cudaEventDestroy(copied[b]);
        }
        if (cs) cudaStreamDestroy(cs);
    }
};

extern "C" int gbx_bfs_trials(gbx_graph *g, const uint32_t *sources, uint32_t num_sources, int mode,
                              uint32_t *distances, int32_t *parents, uint64_t out_stride,
                              gbx_bfs_result *results, void *stream) {
    clear_error();
    GBX_REQUIRE(g, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(num_sources == 0 || (sources && results), GBX_ERR_INVALID, "sources or results is NULL");
    GBX_REQUIRE(mode >= 0 && mode <= 2, GBX_ERR_INVALID, "mode must be 0, 1 or 2");
    for (uint32_t i = 0; i < num_sources; ++i)
        GBX_REQUIRE(sources[i] < g->V, GBX_ERR_INVALID, "source %u (trial %u) out of range [0, %u)", sources[i], i,
                    g->V);
    GBX_REQUIRE(out_stride == 0 || out_stride >= g->V, GBX_ERR_INVALID, "out_stride must be 0 or >= %u", g->V);
    if (num_sources == 0) return GBX_OK;
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    const bool dist_host = distances && !is_device_ptr(distances);
    const bool par_host = parents && !is_device_ptr(parents);
    Scratch sc;
    GBX_TRY(sc.take(g, BfsWork::bytes(V, false), s));
    BfsWork w;
    GBX_TRY(w.carve(sc, V, false));
    GBX_TRY(bfs_graph_setup(g, s));
    DevBuf<BfsSlot> slots;
    GBX_TRY(slots.alloc(num_sources, s));
    // host outputs: each array gets two device staging buffers, used by
    // alternate trials; trial i's copy to the host runs on a second stream
    // while trial i+1 traverses, and trial i+2 waits for it before writing
    // into the same buffer
    DevBuf<uint32_t> dstage;
    DevBuf<int32_t> pstage;
    if (dist_host) GBX_TRY(dstage.alloc(2 * (size_t)V, s));
    if (par_host) GBX_TRY(pstage.alloc(2 * (size_t)V, s));
    CopyLane copies;
    if (dist_host || par_host) GBX_TRY(copies.create());
    // every traversal re-initialises the shared work arrays on the stream, so
    // the traversals run back to back without the host in between
    for (uint32_t i = 0; i < num_sources; ++i) {
        const uint32_t b = i & 1;
        const size_t off = (size_t)i * out_stride;
        uint32_t *lev = dist_host ? dstage.p + (size_t)b * V : distances ? distances + off : w.level;
        int32_t *parp = par_host ? pstage.p + (size_t)b * V : parents ? parents + off : w.parent;
        if (copies.cs && i >= 2) GBX_CUDA(cudaStreamWaitEvent(s, copies.copied[b], 0));
        GBX_TRY(bfs_enqueue(g, w, sources[i], mode, lev, parp, slots.p + i, s));
        if (copies.cs) {
            GBX_CUDA(cudaEventRecord(copies.done[b], s));
            GBX_CUDA(cudaStreamWaitEvent(copies.cs, copies.done[b], 0));
            if (dist_host)
                GBX_CUDA(cudaMemcpyAsync(distances + off, lev, (size_t)V * 4, cudaMemcpyDeviceToHost, copies.cs));
            if (par_host)
                GBX_CUDA(cudaMemcpyAsync(parents + off, parp, (size_t)V * 4, cudaMemcpyDeviceToHost, copies.cs));
            GBX_CUDA(cudaEventRecord(copies.copied[b], copies.cs));
        }
    }
    std::vector<BfsSlot> hs(num_sources);
    GBX_CUDA(cudaMemcpyAsync(hs.data(), slots.p, num_sources * sizeof(BfsSlot), cudaMemcpyDeviceToHost, s));
    if (copies.cs) GBX_CUDA(cudaStreamSynchronize(copies.cs));
    GBX_CUDA(cudaStreamSynchronize(s));
    for (uint32_t i = 0; i < num_sources; ++i) {
        GBX_REQUIRE(hs[i].timeout == 0, GBX_ERR_DEVICE_TIMEOUT, "BFS grid barrier wait expired (trial %u)", i);
        GBX_REQUIRE(hs[i].status == 0, GBX_ERR_ITER_CAP, "BFS step cap reached (trial %u)", i);
        bfs_fill_result(results + i, hs[i].processed, hs[i].iteration, hs[i].depth, hs[i].td_steps,
                        hs[i].bu_steps, hs[i].edges_total);
    }
    return GBX_OK;
}
