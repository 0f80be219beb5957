// Single-source shortest paths (the reference's SSSPDataDrivenPushGraphCSR,
// SSSP.c:514-653, with its relaxation SSSPAtomicRelax, :180-254), as one
// persistent cooperative kernel.
//
// Near/far delta-stepping: vertices whose tentative distance is below the
// current threshold form the "near" list and are relaxed round after round
// (atomicMin on dist[]); improvements at or above the threshold go to the
// "far" pile (each vertex at most once, flagged). When near drains, the
// threshold jumps one delta past the smallest pending far distance (empty
// buckets cost nothing, unlike the reference's full-V bucket sweeps), and far
// entries below it move to near. A near vertex is expanded from the
// distance read when its work unit starts, which its first unit records
// (settled[v]); a far entry whose distance still equals that record is
// dropped as already expanded. A near vertex improved again during the
// round (its stamp already holds the round: the improvement queued it for
// the next round) is not expanded in this one, since the next round expands
// it from the better distance; units that started before the improvement
// relax from the older distance, which is harmless, and a vertex's last
// expansion, in a round without an improvement of it, reads one distance in
// all its units. One grid barrier per round, two for a large round: its
// relaxations are reductions that nobody waits for (the lowered distance and
// a touched bit), and a scan of the touched bitmap after the barrier queues
// the lowered vertices (in such a round "improved again" is a touched bit).
// The result is the unique fixed point
//   dist[u] = min over (v->u) of (uint32)((float)dist[v] + w),
// i.e. the reference's distances. Work units and hub splitting are those of
// the persistent BFS (gbx_bfs.cu): 32 near vertices flattened per warp, or
// kHubChunk edges of one high-degree vertex. Edge ids and weights are read
// with evict-first loads: they stream from HBM either way, and dist / stamp /
// in_far (12 bytes per vertex) should keep the L2.
#include <algorithm>
#include <cstddef>

#include "gbx_coop.cuh"

namespace gbx {

constexpr uint32_t kSsspHubDeg = 1024;
constexpr uint32_t kSsspHubChunk = 2048;
constexpr uint32_t kSsspMaxSplit = 64;  // most warps sharing one 32-vertex group's edges
constexpr uint32_t kStaleRow = 0xFFFFFFFFu;  // snapshot marker of a near row skipped this round
constexpr int kSsspThreads = 1024;
constexpr int kSsspWarps = kSsspThreads / 32;

struct SsspRound {
    unsigned cursor;
    unsigned near_len;          // next near queue (degree in (0, hub])
    unsigned far_len;           // far pile length (carried across rounds)
    unsigned far_min;           // smallest distance pushed at or past the threshold
    unsigned long long near_hub;  // next near hubs: (count << 32) | chunks
    unsigned long long relaxed;
    unsigned kept_min;          // smallest distance the far-pile split kept
    unsigned pad;
};

// Round trace (printed when GBX_TRACE is set): kind (0 start, 1 relax round,
// 2 bucket move), near vertices / new threshold, relaxations / far pile, time.
constexpr unsigned kSsspTraceMax = 256;
struct SsspTraceRec {
    unsigned kind, a;
    unsigned long long b, ns;
};

struct SsspState {
    GridSync gs;
    SsspRound r[3];
    unsigned rounds, status;
    unsigned long long relaxed;
    unsigned ntrace, pad;
    SsspTraceRec trace[kSsspTraceMax];
};

__device__ __forceinline__ void sssp_trace(SsspState *st, unsigned kind, unsigned a, unsigned long long b) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && st->ntrace < kSsspTraceMax) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        SsspTraceRec &r = st->trace[st->ntrace++];
        r.kind = kind;
        r.a = a;
        r.b = b;
        r.ns = t;
    }
}

struct SsspArgs {
    const uint32_t *off, *dest, *outdeg;
    const float *w;
    uint32_t V, delta, source;
    uint32_t *dist, *settled, *stamp, *in_far;
    uint32_t *touched;  // bit v: dist[v] lowered in this (scan-mode) round; all zero between rounds
    uint32_t words;     // (V + 31) / 32
    uint32_t scan_min;  // near vertices (+32 per hub chunk) from which a round runs in scan mode
    uint32_t *q[2], *hv[2], *hc[2];
    uint32_t *far[2];
    SsspState *st;
};

__device__ __forceinline__ uint32_t sssp_add(uint32_t d, float w) {
    // SSSP.c:204: uint32 + float evaluated in float, truncated back to uint32
    return __float2uint_rz(__fadd_rn(__uint2float_rn(d), w));
}

__device__ __forceinline__ uint32_t sssp_chunks(uint32_t d) { return (d + kSsspHubChunk - 1) / kSsspHubChunk; }

struct Relaxer {
    const SsspArgs &a;
    uint32_t threshold, round;
    SsspRound *cnt;
    uint32_t *qout, *hvout, *hcout, *far;
    WarpQueue wnear, wfar;
    unsigned long long relaxed = 0;
    uint32_t far_min = 0xFFFFFFFFu;  // smallest improvement at or past the threshold
    __device__ __forceinline__ Relaxer(const SsspArgs &a_, uint32_t t, uint32_t r, SsspRound *c, uint32_t *q,
                                       uint32_t *hv, uint32_t *hc, uint32_t *f, uint32_t *bn, uint32_t *bf)
        : a(a_), threshold(t), round(r), cnt(c), qout(q), hvout(hv), hcout(hc), far(f), wnear(bn), wfar(bf) {}
    // Four relaxations per lane with their loads and atomics issued back to
    // back (independent), then the queue pushes.
    __device__ __forceinline__ void relax4(const uint32_t (&d)[4], const uint32_t (&e)[4], const uint32_t (&u)[4],
                                           const bool (&act)[4]) {
        uint32_t nd[4], cur[4], old[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float wt = (act[q] && a.w) ? __ldcs(a.w + e[q]) : 1.0f;
            nd[q] = sssp_add(d[q], wt);
            cur[q] = act[q] ? __ldcg(a.dist + u[q]) : 0u;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) old[q] = (act[q] && nd[q] < cur[q]) ? atomicMin(a.dist + u[q], nd[q]) : 0u;
        // the improvements' follow-ups -- the next-near claim, the far flag and
        // the out-degree of a next-near candidate -- are independent of each
        // other, so all of them are issued before any reply is used
        bool imp[4], below[4], far_cl[4];
        uint32_t du[4], stamp_old[4], far_old[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            relaxed += act[q] ? 1u : 0u;
            imp[q] = act[q] && nd[q] < cur[q] && nd[q] < old[q];
            below[q] = imp[q] && nd[q] < threshold;
            far_cl[q] = imp[q] && nd[q] >= threshold;
            if (far_cl[q]) far_min = min(far_min, nd[q]);
            du[q] = below[q] ? __ldg(a.outdeg + u[q]) : 1u;
            stamp_old[q] = below[q] ? atomicExch(a.stamp + u[q], round) : round;
            far_old[q] = far_cl[q] ? atomicExch(a.in_far + u[q], 1u) : 1u;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const bool to_near = below[q] && stamp_old[q] != round;
            const bool to_far = far_cl[q] && far_old[q] == 0u;
            bool hub = false;
            if (du[q] == 0) {
                // nothing to expand: its snapshot is simply its distance, so
                // a far entry it left behind is dropped, not re-bucketed
                atomicMin(a.settled + u[q], nd[q]);
                hub = true;
            } else if (to_near && du[q] > kSsspHubDeg) {
                hub = true;
                unsigned long long h = atomicAdd(&cnt->near_hub, (1ull << 32) | sssp_chunks(du[q]));
                uint32_t slot = (uint32_t)(h >> 32);
                hvout[slot] = u[q];
                hcout[slot] = (uint32_t)h;
            }
            wnear.push(u[q], to_near && !hub, qout, &cnt->near_len);
            wfar.push(u[q], to_far, far, &cnt->far_len);
        }
    }
    // Scan-mode relaxations: the lowered distance and its touched bit are
    // reductions nobody waits for; the round's scan pass then queues the
    // touched vertices. A warp's next batch is not held up by the replies,
    // so a large round keeps many more relaxations in flight. The filtering
    // read of the target's distance goes through L1 (the hubs that most
    // edges point at stay there): a stale copy can only be larger than the
    // current distance, so no improvement is missed; at worst a vertex that
    // was not lowered is touched and expanded once more. The grid barrier's
    // acquire starts every round with fresh copies.
    __device__ __forceinline__ void relax4_red(const uint32_t (&d)[4], const uint32_t (&e)[4],
                                               const uint32_t (&u)[4], const bool (&act)[4]) {
        uint32_t nd[4], cur[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float wt = (act[q] && a.w) ? __ldcs(a.w + e[q]) : 1.0f;
            nd[q] = sssp_add(d[q], wt);
            cur[q] = act[q] ? __ldca(a.dist + u[q]) : 0u;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            relaxed += act[q] ? 1u : 0u;
            if (act[q] && nd[q] < cur[q]) {
                atomicMin(a.dist + u[q], nd[q]);
                atomicOr(a.touched + (u[q] >> 5), 1u << (u[q] & 31));
            }
        }
    }
    __device__ __forceinline__ void flush() {
        wnear.flush(qout, &cnt->near_len);
        wfar.flush(far, &cnt->far_len);
        unsigned long long r = warp_sum(relaxed);
        if ((threadIdx.x & 31) == 0 && r) atomicAdd(&cnt->relaxed, r);
        const uint32_t m = warp_min(far_min);
        if ((threadIdx.x & 31) == 0 && m != 0xFFFFFFFFu) atomicMin(&cnt->far_min, m);
    }
};

__device__ __forceinline__ bool touched_bit(const SsspArgs &a, uint32_t v) {
    return (__ldcg(a.touched + (v >> 5)) >> (v & 31)) & 1u;
}

template <bool kScan>
__device__ void relax_phase(const SsspArgs &a, const uint32_t *qin, uint32_t qn, const uint32_t *hvin,
                            const uint32_t *hcin, uint32_t nh, uint32_t nc, Relaxer &rx, SsspRound *cur,
                            uint32_t *s_pre, uint32_t *s_base, uint32_t *s_d) {
    const uint32_t lane = threadIdx.x & 31;
    // a round with fewer 32-vertex groups than warps cuts each group's edges
    // into `split` interleaved parts (128-edge batches i0 = part*128, +split*128,
    // ...) so that its relaxations are not one warp's serial chain
    const uint32_t groups = (qn + 31) / 32;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    // likewise each hub chunk's 128-edge batches are dealt to `hsplit`
    // warps (batch part, part + hsplit, ...); both splits aim at
    // kUnitsPerWarp units per warp so that the dealer can even the warps out,
    // and the group parts (uneven) are dealt before the hub chunks (even)
    constexpr uint32_t kUnitsPerWarp = 4;
    const uint32_t split = groups ? max(1u, min(kSsspMaxSplit, kUnitsPerWarp * nwarps / groups)) : 1u;
    const uint32_t hsplit = nc ? max(1u, min(kSsspHubChunk / 128, kUnitsPerWarp * nwarps / nc)) : 1u;
    const uint32_t gunits = groups * split;
    const uint32_t units = gunits + nc * hsplit;
    UnitDealer dealer(&cur->cursor);
    for (;;) {
        const uint32_t unit = dealer.take(units);
        if (unit >= units) break;
        if (unit >= gunits) {
            const uint32_t chunk = (unit - gunits) / hsplit, hpart = (unit - gunits) % hsplit;
            const uint32_t h = warp_chunk_owner(hcin, nh, chunk);
            const uint32_t v = __ldcg(hvin + h), first = __ldcg(hcin + h);
            const uint32_t sv = __ldcg(a.stamp + v), d = __ldcg(a.dist + v);
            const uint32_t rb = __ldg(a.off + v), re = __ldg(a.off + v + 1);
            const uint32_t cb = rb + (chunk - first) * kSsspHubChunk;
            // a hub improved in this round is in the next near list already
            const bool stale = kScan ? touched_bit(a, v) : sv == rx.round;
            if (!stale && chunk == first && hpart == 0 && lane == 0) a.settled[v] = d;
            const uint32_t ce = stale ? cb : min(cb + kSsspHubChunk, re);
            // the next batch's ids are loaded before this batch is relaxed
            const uint32_t stride = hsplit * 128;
            uint32_t un[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t j = cb + hpart * 128 + q * 32 + lane;
                un[q] = j < ce ? __ldcs(a.dest + j) : 0u;
            }
            for (uint32_t j0 = cb + hpart * 128; j0 < ce; j0 += stride) {
                uint32_t u[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    u[q] = un[q];
                    const uint32_t j = j0 + stride + q * 32 + lane;
                    un[q] = j < ce ? __ldcs(a.dest + j) : 0u;
                }
                const uint32_t dq[4] = {d, d, d, d};
                const uint32_t eq[4] = {j0 + lane, j0 + 32 + lane, j0 + 64 + lane, j0 + 96 + lane};
                const bool act[4] = {eq[0] < ce, eq[1] < ce, eq[2] < ce, eq[3] < ce};
                if (kScan) rx.relax4_red(dq, eq, u, act); else rx.relax4(dq, eq, u, act);
            }
        } else {
            const uint32_t group = unit / split, part = unit % split;
            const uint32_t qi = group * 32 + lane;
            uint32_t b = 0, deg = 0, d = 0;
            if (qi < qn) {
                const uint32_t v = __ldcg(qin + qi);
                b = __ldg(a.off + v);
                deg = __ldg(a.off + v + 1) - b;
                const uint32_t sv = __ldcg(a.stamp + v);
                d = __ldcg(a.dist + v);
                // improved in this round (so in the next near list): its edges
                // are masked, but the row keeps its place, because every part
                // of a split group must flatten the group identically
                if (kScan ? touched_bit(a, v) : sv == rx.round) d = kStaleRow;
                else if (part == 0) a.settled[v] = d;
            }
            uint32_t incl = deg;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += t;
            }
            s_pre[lane] = incl - deg;
            s_base[lane] = b;
            s_d[lane] = d;
            if (lane == 31) s_pre[32] = incl;
            __syncwarp();
            const uint32_t tot = s_pre[32];
            uint32_t k = 0;
            for (uint32_t i0 = part * 128; i0 < tot; i0 += split * 128) {
                uint32_t u[4], e[4], dd[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint32_t i = i0 + q * 32 + lane;
                    u[q] = 0;
                    e[q] = 0;
                    dd[q] = 0;
                    if (i < tot) {
                        while (s_pre[k + 1] <= i) ++k;
                        e[q] = s_base[k] + (i - s_pre[k]);
                        dd[q] = s_d[k];
                        if (dd[q] != kStaleRow) u[q] = __ldcs(a.dest + e[q]);
                    }
                }
                const bool act[4] = {i0 + lane < tot && dd[0] != kStaleRow, i0 + 32 + lane < tot && dd[1] != kStaleRow,
                                     i0 + 64 + lane < tot && dd[2] != kStaleRow,
                                     i0 + 96 + lane < tot && dd[3] != kStaleRow};
                if (kScan) rx.relax4_red(dd, e, u, act); else rx.relax4(dd, e, u, act);
            }
            __syncwarp();
        }
    }
}

// Scan-mode round, second pass: every vertex whose touched bit is set was
// lowered in this round (some relaxation saw a larger distance and reduced
// it), so it is queued exactly as the per-relaxation follow-ups would have:
// below the threshold into the next near list (hubs into the hub list,
// vertices without out-edges settled on the spot), else into the far pile
// once. A warp takes 32 consecutive vertices (one bitmap word) at a time.
__device__ void scan_phase(const SsspArgs &a, uint32_t thr, SsspRound *cnt, uint32_t *qout, uint32_t *hvout,
                           uint32_t *hcout, uint32_t *far, uint32_t *bn, uint32_t *bf) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    WarpQueue wnear(bn), wfar(bf);
    uint32_t far_min = 0xFFFFFFFFu;
    for (uint32_t w = gw; w < a.words; w += nw) {
        // lane 0 reads and clears the word (one thread: the read is ordered
        // before the clear), the warp gets it by a shuffle
        uint32_t m = 0;
        if (lane == 0) {
            m = __ldcg(a.touched + w);
            if (m) a.touched[w] = 0u;
        }
        m = __shfl_sync(0xffffffffu, m, 0);
        if (!m) continue;
        const uint32_t u = w * 32 + lane;
        const bool t = (m >> lane) & 1u;
        uint32_t d = 0, du = 0, inf = 1;
        if (t) {
            d = __ldcg(a.dist + u);
            du = __ldg(a.outdeg + u);
            inf = __ldcg(a.in_far + u);
        }
        const bool below = t && d < thr;
        bool to_near = false, to_far = false;
        if (below) {
            if (du == 0) {
                a.settled[u] = d;  // nothing to expand
            } else if (du > kSsspHubDeg) {
                const unsigned long long h = atomicAdd(&cnt->near_hub, (1ull << 32) | sssp_chunks(du));
                const uint32_t slot = (uint32_t)(h >> 32);
                hvout[slot] = u;
                hcout[slot] = (uint32_t)h;
            } else {
                to_near = true;
            }
        } else if (t) {
            far_min = min(far_min, d);
            if (!inf) {
                a.in_far[u] = 1u;
                to_far = true;
            }
        }
        wnear.push(u, to_near, qout, &cnt->near_len);
        wfar.push(u, to_far, far, &cnt->far_len);
    }
    wnear.flush(qout, &cnt->near_len);
    wfar.flush(far, &cnt->far_len);
    const uint32_t fm = warp_min(far_min);
    if (lane == 0 && fm != 0xFFFFFFFFu) atomicMin(&cnt->far_min, fm);
}

__device__ __forceinline__ void zero_round(SsspRound *r, uint32_t far_len) {
    r->cursor = 0;
    r->near_len = 0;
    r->far_len = far_len;
    r->far_min = 0xFFFFFFFFu;
    r->near_hub = 0;
    r->relaxed = 0;
    r->kept_min = 0xFFFFFFFFu;
}

__global__ void __launch_bounds__(kSsspThreads, 1) sssp_persistent_kernel(SsspArgs a) {
    __shared__ uint32_t s_pre[kSsspWarps][33];
    __shared__ uint32_t s_base[kSsspWarps][32];
    __shared__ uint32_t s_d[kSsspWarps][32];
    __shared__ uint32_t s_wn[kSsspWarps][kWarpQueueCap];
    __shared__ uint32_t s_wf[kSsspWarps][kWarpQueueCap];
    __shared__ SsspRound s_cnt;  // the finished round's counters (fetch_counters)
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    SsspState *st = a.st;
    grid_barrier_init();
    uint32_t qn = 1, nh = 0, nc = 0, far_len = 0;
    {
        const uint32_t d0 = __ldg(a.outdeg + a.source);
        if (d0 > kSsspHubDeg) { qn = 0; nh = 1; nc = sssp_chunks(d0); }
        else if (d0 == 0) { qn = 0; }
    }
    uint64_t threshold = a.delta;
    // lower bound of the far pile's smallest live distance: the smallest
    // improvement pushed at or past the threshold since the pile was last
    // split (whose split computed the kept entries' exact minimum)
    uint32_t far_lb = 0xFFFFFFFFu;
    uint32_t round = 1, rounds = 0, fb = 0, gen = 0;
    unsigned long long relaxed = 0;
    bool failed = false;
    const uint32_t max_rounds = 4 * a.V + 64;
    // round 0's counters were set by sssp_init_kernel: the first round's
    // relaxations start before any grid barrier
    sssp_trace(st, 0, 1, 0);
    for (uint32_t s = 0;; ++s) {
        SsspRound *cur = &st->r[s % 3];
        if (blockIdx.x == 0 && threadIdx.x == 0) zero_round(&st->r[(s + 1) % 3], 0);
        if (qn + nh > 0) {
            if (rounds >= max_rounds) { failed = true; break; }
            const uint32_t ib = gen & 1;
            round++;
            const uint32_t thr = threshold > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)threshold;
            // far pushes of this round append after the pile's far_len entries
            Relaxer rx(a, thr, round, cur, a.q[ib ^ 1], a.hv[ib ^ 1], a.hc[ib ^ 1], a.far[fb] + far_len, s_wn[wid],
                       s_wf[wid]);
            // a large round relaxes with reductions and queues what it
            // lowered in a scan pass after one more barrier; a small one
            // queues each improvement as it happens
            const bool scan = (uint64_t)qn + 32ull * nc >= a.scan_min;
            if (scan) {
                relax_phase<true>(a, a.q[ib], qn, a.hv[ib], a.hc[ib], nh, nc, rx, cur, s_pre[wid], s_base[wid],
                                  s_d[wid]);
                rx.flush();
                if (!grid_barrier(&st->gs)) { failed = true; break; }
                scan_phase(a, thr, cur, a.q[ib ^ 1], a.hv[ib ^ 1], a.hc[ib ^ 1], a.far[fb] + far_len, s_wn[wid],
                           s_wf[wid]);
            } else {
                relax_phase<false>(a, a.q[ib], qn, a.hv[ib], a.hc[ib], nh, nc, rx, cur, s_pre[wid], s_base[wid],
                                   s_d[wid]);
                rx.flush();
            }
            if (!grid_barrier(&st->gs)) { failed = true; break; }
            fetch_counters(cur, &s_cnt);
            relaxed += s_cnt.relaxed;
            sssp_trace(st, 1, qn + nh, s_cnt.relaxed);
            qn = s_cnt.near_len;
            unsigned long long hb = s_cnt.near_hub;
            nh = (uint32_t)(hb >> 32);
            nc = (uint32_t)hb;
            far_len += s_cnt.far_len;
            far_lb = min(far_lb, s_cnt.far_min);
            gen++;
            rounds++;
            continue;
        }
        if (far_len == 0) break;
        // next threshold: one delta past the far pile's smallest live
        // distance, taken from its lower bound. A bound left low by an entry
        // that was expanded since costs at most one empty bucket move, after
        // which the bound is exact again.
        uint32_t fmin = far_lb;
        if (fmin == 0xFFFFFFFFu) {
            // no bound recorded (not expected: every far entry is pushed or
            // kept with its distance); scan the pile
            uint32_t m = 0xFFFFFFFFu;
            for (uint32_t i = gtid; i < far_len; i += nthreads) {
                uint32_t u = __ldcg(a.far[fb] + i);
                uint32_t d = __ldcg(a.dist + u);
                if (__ldcg(a.settled + u) != d) m = min(m, d);
            }
            m = __reduce_min_sync(0xffffffffu, m);
            if (lane == 0 && m != 0xFFFFFFFFu) atomicMin(&cur->far_min, m);
            if (!grid_barrier(&st->gs)) { failed = true; break; }
            fmin = __ldcg(&cur->far_min);
            if (fmin == 0xFFFFFFFFu) break;  // every far entry is already expanded
        }
        threshold = ((uint64_t)fmin / a.delta + 1) * a.delta;
        round++;
        {
            // split the far pile: below the threshold -> near, the rest stays
            const uint32_t ib = gen & 1;
            const uint32_t thr = threshold > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)threshold;
            uint32_t kmin = 0xFFFFFFFFu;
            WarpQueue wnear(s_wn[wid]), wfar(s_wf[wid]);
            // four pile entries per thread in flight: their ids, then their
            // distances and snapshots, then the claims and degrees
            constexpr uint32_t kSplitIlp = 4;
            for (uint32_t base = blockIdx.x * blockDim.x; base < far_len; base += kSplitIlp * nthreads) {
                uint32_t u[kSplitIlp], d[kSplitIlp], sv[kSplitIlp], stamp_old[kSplitIlp], du[kSplitIlp];
                bool in[kSplitIlp], to_near[kSplitIlp], keep[kSplitIlp], hub[kSplitIlp];
#pragma unroll
                for (uint32_t q = 0; q < kSplitIlp; ++q) {
                    const uint32_t i = base + q * nthreads + threadIdx.x;
                    in[q] = i < far_len;
                    u[q] = in[q] ? __ldcg(a.far[fb] + i) : 0u;
                }
#pragma unroll
                for (uint32_t q = 0; q < kSplitIlp; ++q) {
                    d[q] = in[q] ? __ldcg(a.dist + u[q]) : 0u;
                    sv[q] = in[q] ? __ldcg(a.settled + u[q]) : 0u;
                }
#pragma unroll
                for (uint32_t q = 0; q < kSplitIlp; ++q) {
                    const bool expanded = in[q] && sv[q] == d[q];
                    const bool below = in[q] && !expanded && d[q] < thr;
                    keep[q] = in[q] && !expanded && !below;
                    if (keep[q]) kmin = min(kmin, d[q]);
                    if (expanded || below) a.in_far[u[q]] = 0;
                    stamp_old[q] = below ? atomicExch(a.stamp + u[q], round) : round;
                    du[q] = below ? __ldg(a.outdeg + u[q]) : 1u;
                    to_near[q] = below && stamp_old[q] != round;
                    hub[q] = false;
                }
#pragma unroll
                for (uint32_t q = 0; q < kSplitIlp; ++q) {
                    if (to_near[q]) {
                        if (du[q] > kSsspHubDeg) {
                            hub[q] = true;
                            const unsigned long long h =
                                atomicAdd(&cur->near_hub, (1ull << 32) | sssp_chunks(du[q]));
                            const uint32_t slot = (uint32_t)(h >> 32);
                            a.hv[ib][slot] = u[q];
                            a.hc[ib][slot] = (uint32_t)h;
                        } else if (du[q] == 0) {
                            // nothing to relax: settled right here
                            hub[q] = true;
                            a.settled[u[q]] = d[q];
                        }
                    }
                    wnear.push(u[q], to_near[q] && !hub[q], a.q[ib], &cur->near_len);
                    wfar.push(u[q], keep[q], a.far[fb ^ 1], &cur->far_len);
                }
            }
            wnear.flush(a.q[ib], &cur->near_len);
            wfar.flush(a.far[fb ^ 1], &cur->far_len);
            kmin = warp_min(kmin);
            if (lane == 0 && kmin != 0xFFFFFFFFu) atomicMin(&cur->kept_min, kmin);
        }
        if (!grid_barrier(&st->gs)) { failed = true; break; }
        fetch_counters(cur, &s_cnt);
        qn = s_cnt.near_len;
        unsigned long long hb = s_cnt.near_hub;
        nh = (uint32_t)(hb >> 32);
        nc = (uint32_t)hb;
        far_len = s_cnt.far_len;
        far_lb = s_cnt.kept_min;
        sssp_trace(st, 2, threshold > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)threshold, far_len);
        fb ^= 1;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->rounds = rounds;
        st->relaxed = relaxed;
        st->status = failed ? 1u : 0u;
    }
}

__global__ void sssp_init_kernel(uint32_t *dist, uint32_t *settled, uint32_t *stamp, uint32_t *in_far,
                                 uint32_t *touched, uint32_t V, uint32_t source, const uint32_t *outdeg,
                                 uint32_t *q0, uint32_t *hv0, uint32_t *hc0, SsspRound *r0) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        dist[v] = v == source ? 0u : kSsspInf;
        settled[v] = 0xFFFFFFFFu;
        stamp[v] = v == source ? 1u : 0u;
        in_far[v] = 0;
    }
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < (V + 31) / 32; w += gridDim.x * blockDim.x)
        touched[w] = 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        q0[0] = source;
        hv0[0] = source;
        hc0[0] = 0;
        zero_round(r0, 0);
    }
}

__global__ void sssp_finish_kernel(const uint32_t *dist, const uint32_t *outdeg, uint32_t V, uint32_t *out,
                                   unsigned long long *stats /* reached, edges */) {
    uint32_t reached = 0;
    unsigned long long edges = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        uint32_t d = dist[v];
        out[v] = d;
        if (d != kSsspInf) {
            reached++;
            edges += outdeg[v];
        }
    }
    reached = warp_sum(reached);
    edges = warp_sum(edges);
    if ((threadIdx.x & 31) == 0) {
        if (reached) atomicAdd(&stats[0], (unsigned long long)reached);
        if (edges) atomicAdd(&stats[1], edges);
    }
}

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_sssp(gbx_graph *g, uint32_t source, uint32_t delta, uint32_t *distances,
                        gbx_sssp_result *result, void *stream) {
    clear_error();
    GBX_REQUIRE(g && distances, GBX_ERR_INVALID, "graph or distances is NULL");
    GBX_REQUIRE(source < g->V, GBX_ERR_INVALID, "source %u out of range [0, %u)", source, g->V);
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    if (delta == 0) delta = g->sssp_delta ? g->sssp_delta : (g->weight ? 256u : 1u);
    // working arrays from the graph's scratch arena (plus staging for a
    // host-memory result)
    const int out_dev = is_device_ptr(distances) ? 1 : 0;
    const bool stage = !out_dev;
    const size_t r = Scratch::round_up((size_t)V * 4);
    Scratch sc;
    const uint32_t words = (V + 31) / 32;
    GBX_TRY(sc.take(g, (stage ? 13 : 12) * r + Scratch::round_up((size_t)words * 4) +
                           Scratch::round_up(sizeof(SsspState)) + Scratch::round_up(16),
                    s));
    uint32_t *dist = sc.carve<uint32_t>(V), *settled = sc.carve<uint32_t>(V), *stamp = sc.carve<uint32_t>(V);
    uint32_t *in_far = sc.carve<uint32_t>(V), *q0 = sc.carve<uint32_t>(V), *q1 = sc.carve<uint32_t>(V);
    uint32_t *hv0 = sc.carve<uint32_t>(V), *hv1 = sc.carve<uint32_t>(V), *hc0 = sc.carve<uint32_t>(V);
    uint32_t *hc1 = sc.carve<uint32_t>(V), *f0 = sc.carve<uint32_t>(V), *f1 = sc.carve<uint32_t>(V);
    uint32_t *out_stage = stage ? sc.carve<uint32_t>(V) : nullptr;
    uint32_t *touched = sc.carve<uint32_t>(words);
    SsspState *st = sc.carve<SsspState>(1);
    unsigned long long *fin = sc.carve<unsigned long long>(2);
    GBX_REQUIRE(fin != nullptr, GBX_ERR_CUDA, "SSSP scratch carve overflow");
    OutArray<uint32_t> out;
    GBX_TRY(out.bind(distances, V, s, out_stage, out_dev));
    const unsigned grid1 = std::min<unsigned>(ceil_div(V, 256), (unsigned)num_sms() * 8);
    GBX_CUDA(cudaMemsetAsync(st, 0, sizeof(SsspState), s));
    sssp_init_kernel<<<grid1, 256, 0, s>>>(dist, settled, stamp, in_far, touched, V, source, g->out_degree,
                                           q0, hv0, hc0, &st->r[0]);
    GBX_LAUNCH_CHECK();
    SsspArgs a;
    a.off = g->offsets;
    a.dest = g->dest;
    a.outdeg = g->out_degree;
    a.w = g->weight;
    a.V = V;
    a.delta = delta;
    a.source = source;
    a.dist = dist;
    a.settled = settled;
    a.stamp = stamp;
    a.in_far = in_far;
    a.touched = touched;
    a.words = words;
    a.scan_min = std::max<uint32_t>(4096u, V / 256);
    a.q[0] = q0;
    a.q[1] = q1;
    a.hv[0] = hv0;
    a.hv[1] = hv1;
    a.hc[0] = hc0;
    a.hc[1] = hc1;
    a.far[0] = f0;
    a.far[1] = f1;
    a.st = st;
    int grid = 0;
    static int grid_cache[64] = {0};
    GBX_TRY(coop_grid(sssp_persistent_kernel, kSsspThreads, 0, &grid, &grid_cache));
    void *args[] = {&a};
    GBX_CUDA(cudaLaunchCooperativeKernel((const void *)sssp_persistent_kernel, grid, kSsspThreads, args, 0, s));
    GBX_LAUNCH_CHECK();
    GBX_CUDA(cudaMemsetAsync(fin, 0, 16, s));
    sssp_finish_kernel<<<grid1, 256, 0, s>>>(dist, g->out_degree, V, out.d, fin);
    GBX_LAUNCH_CHECK();
    GBX_TRY(out.finish(s));
    SsspState hs;
    unsigned long long hf[2];
    GBX_CUDA(cudaMemcpyAsync(&hs, st, trace_enabled() ? sizeof(hs) : offsetof(SsspState, trace),
                             cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaMemcpyAsync(hf, fin, 16, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    GBX_REQUIRE(hs.gs.error == 0, GBX_ERR_DEVICE_TIMEOUT, "SSSP grid barrier wait expired");
    GBX_REQUIRE(hs.status == 0, GBX_ERR_ITER_CAP, "SSSP round cap reached");
    if (trace_enabled()) {
        fprintf(stderr, "| gbx_sssp source %u delta %u: %-6s | %-10s | %-12s | %-9s |\n", source, delta, "step",
                "near/thr", "relaxed/far", "us");
        static const char *names[] = {"start", "relax", "bucket"};
        for (unsigned i = 1; i < hs.ntrace && i < kSsspTraceMax; ++i)
            fprintf(stderr, "| %-30s | %-10u | %-12llu | %-9.2f |\n", names[hs.trace[i].kind % 3], hs.trace[i].a,
                    hs.trace[i].b, (hs.trace[i].ns - hs.trace[i - 1].ns) * 1e-3);
    }
    if (result) {
        result->reached = (uint32_t)hf[0];
        result->rounds = hs.rounds;
        result->edges_relaxed = hs.relaxed;
        result->edges_traversed = hf[1];
    }
    return GBX_OK;
}
