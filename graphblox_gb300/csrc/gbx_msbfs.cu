// Multi-source BFS with per-vertex source bitmasks: up to 256 BFS runs over
// one graph in one level-synchronous sweep. No reference counterpart as a
// batch; for every source the distances, processed_nodes and iteration are
// those of the reference's breadthFirstSearchGraphCSR (BFS.c:103-127) from
// that source alone (levels are unique, so the schedule does not change them).
//
// State, NW = ceil(S/32) rounded up to 1, 2, 4 or 8 words per vertex:
//   seen[v][NW]  sources that have reached v
//   F[v][NW]     sources whose frontier holds v (this level)
//   Fn[v][NW]    the next level's bits (before masking with seen)
// Each level either pushes from a compacted frontier list (atomicOr of F[u]
// into Fn of every out-neighbour; few frontier edges) or pulls over in-edges
// (OR of F[u] over v's in-edges, stopping once every bit v still misses is
// found). A group of NW lanes owns one vertex, lane k its k-th mask word, so a
// mask is one 4*NW-byte access. Pull rows above kMsLight in-edges are cut into
// kMsChunk-edge chunks worked by whole warps and OR-ed into Fn with atomics
// (OR is order-free, so the result is deterministic). An update pass then
// sets new = Fn & ~seen, seen |= new, and compacts the next frontier list;
// the new masks of each level are kept (up to kMsMaxStoredLevels of them).
//
// distances is vertex-major: distances[v * S + i] is the level of v from
// sources[i] (0 for sources[i] itself and for unreached vertices, as the
// reference reports). One final pass writes every row of distances from the
// kept level masks (a warp per vertex, whole 16-byte stores) and reduces the
// per-source results; only levels past the kept ones write their distances
// bit by bit during the traversal.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "gbx_internal.cuh"

namespace gbx {

constexpr uint32_t kMsLight = 64;
constexpr uint32_t kMsChunk = 1024;
constexpr int kMsThreads = 256;

// bits of mask word k that belong to one of the S sources
__device__ __forceinline__ uint32_t ms_valid(uint32_t k, uint32_t S) {
    return 32 * k + 32 <= S ? 0xFFFFFFFFu : (S > 32 * k ? (1u << (S - 32 * k)) - 1u : 0u);
}

struct MsCounters {
    uint32_t qn;                // next frontier list length
    uint32_t pad;
    unsigned long long mf;      // out-edges of the next frontier
};

// ---- expansion: push ----------------------------------------------------------
template <int NW>
__global__ void __launch_bounds__(kMsThreads)
    ms_push_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest, const uint32_t *__restrict__ q,
                   uint32_t qn, const uint32_t *__restrict__ F, const uint32_t *__restrict__ seen,
                   uint32_t *__restrict__ Fn) {
    constexpr int GPW = 32 / NW;  // groups per warp
    const uint32_t lane = threadIdx.x & 31, k = lane % NW;
    const uint32_t grp = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * GPW + lane / NW;
    const uint32_t ngrp = ((gridDim.x * blockDim.x) >> 5) * GPW;
    for (uint32_t i = grp; i < qn; i += ngrp) {
        const uint32_t u = q[i];
        const uint32_t fu = F[(size_t)u * NW + k];
        if (!fu) continue;  // lane-local: other lanes of the group may still push
        const uint32_t eb = off[u], ee = off[u + 1];
        for (uint32_t e = eb; e < ee; e += 4) {
            // four out-edges per round: targets, then their seen words
            uint32_t v[4], sw[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = e + q < ee ? __ldg(dest + e + q) : 0u;
#pragma unroll
            for (int q = 0; q < 4; ++q) sw[q] = e + q < ee ? __ldg(seen + (size_t)v[q] * NW + k) : 0xFFFFFFFFu;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t add = fu & ~sw[q];
                if (add) atomicOr(Fn + (size_t)v[q] * NW + k, add);
            }
        }
    }
}

// ---- expansion: pull -----------------------------------------------------------
// Light rows: one NW-lane group per vertex; the warp's groups step through
// their rows together so the early-exit vote is warp-uniform.
template <int NW>
__global__ void __launch_bounds__(kMsThreads)
    ms_pull_light_kernel(const uint32_t *__restrict__ poff, const uint32_t *__restrict__ psrc, uint32_t V, uint32_t S,
                         const uint32_t *__restrict__ F, const uint32_t *__restrict__ seen, uint32_t *__restrict__ Fn) {
    constexpr int GPW = 32 / NW;
    const uint32_t lane = threadIdx.x & 31, k = lane % NW;
    const uint32_t gmask = (NW == 32 ? 0xFFFFFFFFu : ((1u << NW) - 1u)) << (lane / NW * NW);
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarp = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warp0 * GPW; base < V; base += nwarp * GPW) {
        const uint32_t v = base + lane / NW;
        uint32_t b = 0, e = 0, need = 0;
        if (v < V) {
            b = poff[v];
            e = poff[v + 1];
            need = ~seen[(size_t)v * NW + k] & ms_valid(k, S);
            if (e - b > kMsLight) e = b;  // heavy rows are worked by the chunk kernel
        }
        uint32_t acc = 0;
        // group still searching: some lane of it has bits it needs and lacks
        bool open = __ballot_sync(0xFFFFFFFFu, (need & ~acc) != 0 && b < e) & gmask;
        uint32_t j = b;
        while (__any_sync(0xFFFFFFFFu, open)) {
            if (open) {
                // four in-edges per round: their ids, then their mask words,
                // in flight together (the early exit checks once per round)
                uint32_t u[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) u[q] = j + q < e ? __ldg(psrc + j + q) : 0u;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (j + q < e) acc |= __ldg(F + (size_t)u[q] * NW + k);
                j += 4;
            }
            open = __ballot_sync(0xFFFFFFFFu, (need & ~acc) != 0 && j < e) & gmask;
        }
        if (v < V && acc) Fn[(size_t)v * NW + k] = acc;  // heavy rows leave acc 0 here
    }
}

struct MsChunk {
    uint32_t row, eb, ee, pad;
};

// Heavy rows: one warp per chunk, its groups striding the chunk's edges.
template <int NW>
__global__ void __launch_bounds__(kMsThreads)
    ms_pull_heavy_kernel(const MsChunk *__restrict__ chunks, uint32_t n_chunks, const uint32_t *__restrict__ psrc,
                         uint32_t S, const uint32_t *__restrict__ F, const uint32_t *__restrict__ seen,
                         uint32_t *__restrict__ Fn) {
    constexpr int GPW = 32 / NW;
    const uint32_t lane = threadIdx.x & 31, k = lane % NW, gi = lane / NW;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarp = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t c = warp0; c < n_chunks; c += nwarp) {
        const MsChunk ck = chunks[c];
        const uint32_t need = ~seen[(size_t)ck.row * NW + k] & ms_valid(k, S);
        uint32_t acc = 0;
        for (uint32_t j0 = ck.eb; j0 < ck.ee; j0 += 4 * GPW) {
            // four edges per group per round, loads in flight together
            uint32_t u[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t j = j0 + q * GPW + gi;
                u[q] = j < ck.ee ? __ldg(psrc + j) : 0u;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (j0 + q * GPW + gi < ck.ee) acc |= __ldg(F + (size_t)u[q] * NW + k);
            // OR across the groups, then stop once every needed bit is present
            uint32_t all = acc;
#pragma unroll
            for (int o = NW; o < 32; o <<= 1) all |= __shfl_xor_sync(0xFFFFFFFFu, all, o);
            if (!__any_sync(0xFFFFFFFFu, (need & ~all) != 0)) break;
        }
#pragma unroll
        for (int o = NW; o < 32; o <<= 1) acc |= __shfl_xor_sync(0xFFFFFFFFu, acc, o);
        if (gi == 0 && (acc & need)) atomicOr(Fn + (size_t)ck.row * NW + k, acc & need);
    }
}

// ---- update ----------------------------------------------------------------------
// new = Fn & ~seen; seen |= new; F_next = new (written into Fn, which is kept
// as this level's mask while levels are stored); v appended to the next
// frontier list when any bit is new. Past the stored levels (kWriteDist) the
// distances of the new bits are written here, one by one.
template <int NW, bool kWriteDist>
__global__ void __launch_bounds__(kMsThreads)
    ms_update_kernel(uint32_t V, uint32_t S, uint32_t level, const uint32_t *__restrict__ off,
                     uint32_t *__restrict__ seen, uint32_t *__restrict__ Fn, uint32_t *__restrict__ dist,
                     uint32_t *__restrict__ qnext, MsCounters *cnt) {
    // next-frontier appends are staged per warp in shared memory and reserved
    // with one atomic per batch (one per warp step would put V/GPW atomics
    // on the one length counter), the out-degree sum with one per warp
    constexpr uint32_t kCap = 128;
    __shared__ uint32_t s_q[kMsThreads / 32][kCap];
    constexpr int GPW = 32 / NW;
    const uint32_t lane = threadIdx.x & 31, k = lane % NW, gi = lane / NW;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarp = (gridDim.x * blockDim.x) >> 5;
    uint32_t *wq = s_q[threadIdx.x >> 5];
    uint32_t wn = 0;
    unsigned long long mf = 0;
    auto flush = [&]() {
        __syncwarp();
        uint32_t pos = 0;
        if (lane == 0) pos = atomicAdd(&cnt->qn, wn);
        pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
        for (uint32_t i = lane; i < wn; i += 32) qnext[pos + i] = wq[i];
        __syncwarp();
        wn = 0;
    };
    for (uint32_t base = warp0 * GPW; base < V; base += nwarp * GPW) {
        const uint32_t v = base + gi;
        uint32_t nw = 0;
        if (v < V) {
            const size_t i = (size_t)v * NW + k;
            const uint32_t s0 = seen[i];
            nw = Fn[i] & ~s0;
            Fn[i] = nw;
            if (nw) {
                seen[i] = s0 | nw;
                if (kWriteDist) {
                    uint32_t *row = dist + (size_t)v * S + 32 * k;
                    for (uint32_t m = nw; m; m &= m - 1) row[__ffs(m) - 1] = level;
                }
            }
        }
        // one append per vertex with any new bit: the group's lowest lane
        const uint32_t any = __ballot_sync(0xFFFFFFFFu, nw != 0);
        const uint32_t gm = (NW == 32 ? 0xFFFFFFFFu : ((1u << NW) - 1u)) << (gi * NW);
        const bool leader = k == 0 && (any & gm);
        if (leader) mf += off[v + 1] - off[v];
        const uint32_t lm = __ballot_sync(0xFFFFFFFFu, leader);
        if (leader) wq[wn + __popc(lm & ((1u << lane) - 1u))] = v;
        wn += __popc(lm);
        if (wn > kCap - 32) flush();
    }
    if (wn) flush();
    mf = warp_sum(mf);
    if (lane == 0 && mf) atomicAdd(&cnt->mf, mf);
}

__global__ void ms_seed_kernel(const uint32_t *sources, uint32_t S, uint32_t NW, const uint32_t *off, uint32_t *seen,
                               uint32_t *F, uint32_t *q, MsCounters *cnt) {
    for (uint32_t i = threadIdx.x; i < S; i += blockDim.x) {
        const uint32_t s = sources[i];
        atomicOr(seen + (size_t)s * NW + i / 32, 1u << (i % 32));
        atomicOr(F + (size_t)s * NW + i / 32, 1u << (i % 32));
        q[i] = s;  // a repeated source is pushed twice: OR makes that harmless
        atomicAdd(&cnt->mf, (unsigned long long)(off[s + 1] - off[s]));
    }
    if (threadIdx.x == 0) cnt->qn = S;
}

// Level masks kept for the final pass: masks[L][v * NW + k] holds the
// sources (bits of word k) that reached v at level L (level 0: the seeds).
constexpr uint32_t kMsMaxStoredLevels = 32;
struct MsLevels {
    const uint32_t *m[kMsMaxStoredLevels];
    uint32_t n;
};

// The distances and the per-source results in one pass: a warp per vertex,
// lane l owning sources l*NW .. l*NW + NW-1 (NW consecutive bits of mask
// word l*NW/32). A source's level at v is the first stored level whose mask
// holds its bit; a bit that is seen but in no stored mask was reached past
// the stored levels, and its distance was written by the update kernel; the
// rest are unreached (0, as is the source's own entry at level 0). Per
// source: reached vertices (level >= 1), the out-degree sum over them, the
// deepest level.
template <int NW>
__global__ void __launch_bounds__(kMsThreads)
    ms_final_kernel(MsLevels lv, const uint32_t *__restrict__ seen, uint32_t V, uint32_t S,
                    const uint32_t *__restrict__ off, const uint32_t *__restrict__ sources, bool vec_rows,
                    uint32_t *__restrict__ dist, uint32_t *__restrict__ cnt, unsigned long long *__restrict__ edges,
                    uint32_t *__restrict__ depth) {
    __shared__ uint32_t s_cnt[32 * NW], s_depth[32 * NW];
    __shared__ unsigned long long s_edges[32 * NW];
    for (uint32_t i = threadIdx.x; i < 32 * NW; i += blockDim.x) {
        s_cnt[i] = 0;
        s_depth[i] = 0;
        s_edges[i] = 0;
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t k = lane * NW / 32, sh = (lane * NW) % 32;
    const uint32_t bmask = NW == 32 ? 0xFFFFFFFFu : ((1u << NW) - 1u);
    const uint32_t s0 = lane * NW;  // this lane's first source
    uint32_t c[NW], dm[NW];
    unsigned long long ed[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j) c[j] = dm[j] = 0, ed[j] = 0;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarp = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = warp0; v < V; v += nwarp) {
        const size_t w = (size_t)v * NW + k;
        const uint32_t sw = (__ldg(seen + w) >> sh) & bmask;
        const uint32_t deg = __ldg(off + v + 1) - __ldg(off + v);
        uint32_t lvl[NW];
#pragma unroll
        for (int j = 0; j < NW; ++j) lvl[j] = 0;
        uint32_t found = 0;
        for (uint32_t L0 = 0; L0 < lv.n && found != sw; L0 += 8) {
            uint32_t m[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) m[q] = L0 + q < lv.n ? (__ldg(lv.m[L0 + q] + w) >> sh) & bmask : 0u;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const uint32_t nb = m[q] & ~found;
#pragma unroll
                for (int j = 0; j < NW; ++j)
                    if ((nb >> j) & 1u) lvl[j] = L0 + q;
                found |= m[q];
            }
        }
        uint32_t *row = dist + (size_t)v * S + s0;
        const uint32_t deep = sw & ~found;  // written by the update kernel past the stored levels
        if (deep) {
#pragma unroll
            for (int j = 0; j < NW; ++j)
                if ((deep >> j) & 1u) lvl[j] = row[j];
        }
        const bool full = s0 + NW <= S;
        if (NW % 4 == 0 && vec_rows && full) {
#pragma unroll
            for (int q = 0; q < NW / 4; ++q)
                reinterpret_cast<uint4 *>(row)[q] = make_uint4(lvl[4 * q], lvl[4 * q + 1], lvl[4 * q + 2], lvl[4 * q + 3]);
        } else {
#pragma unroll
            for (int j = 0; j < NW; ++j)
                if (s0 + j < S) row[j] = lvl[j];
        }
#pragma unroll
        for (int j = 0; j < NW; ++j) {
            if (lvl[j]) {  // only sources below S can hold a level
                c[j] += 1;
                ed[j] += deg;
                dm[j] = max(dm[j], lvl[j]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NW; ++j) {
        if (s0 + j < S && c[j]) {
            atomicAdd(s_cnt + s0 + j, c[j]);
            atomicAdd(s_edges + s0 + j, ed[j]);
            atomicMax(s_depth + s0 + j, dm[j]);
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < S; i += blockDim.x) {
        // block 0 adds each source's own out-edges
        const unsigned long long own = blockIdx.x == 0 ? __ldg(off + sources[i] + 1) - __ldg(off + sources[i]) : 0u;
        if (s_cnt[i] || own) {
            atomicAdd(cnt + i, s_cnt[i]);
            atomicAdd(edges + i, s_edges[i] + own);
            atomicMax(depth + i, s_depth[i]);
        }
    }
}

}  // namespace gbx

// Chunk list of the heavy pull rows of a graph (cached on the graph).
struct gbx_ms_plan {
    gbx::MsChunk *chunks = nullptr;
    uint32_t n_chunks = 0;
};

void gbx_free_ms_plan(gbx_ms_plan *p) {
    if (!p) return;
    cudaFree(p->chunks);
    delete p;
}

using namespace gbx;

namespace {

int ms_plan(gbx_graph *g, cudaStream_t s, gbx_ms_plan **out) {
    if (!g->ms_plan) {
        const uint32_t V = g->V;
        std::vector<uint32_t> off(V + 1);
        GBX_CUDA(cudaMemcpyAsync(off.data(), g->pull_offsets(), 4 * ((size_t)V + 1), cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        std::vector<MsChunk> ch;
        for (uint32_t v = 0; v < V; ++v)
            if (off[v + 1] - off[v] > kMsLight)
                for (uint32_t c = off[v]; c < off[v + 1]; c += kMsChunk)
                    ch.push_back({v, c, std::min(c + kMsChunk, off[v + 1]), 0});
        gbx_ms_plan *p = new gbx_ms_plan();
        p->n_chunks = (uint32_t)ch.size();
        if (cudaMalloc(&p->chunks, sizeof(MsChunk) * std::max<size_t>(1, ch.size())) != cudaSuccess) {
            (void)cudaGetLastError();
            delete p;
            set_error("multi-source BFS plan allocation failed");
            return GBX_ERR_NOMEM;
        }
        if (!ch.empty()) {
            const cudaError_t e =
                cudaMemcpyAsync(p->chunks, ch.data(), sizeof(MsChunk) * ch.size(), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                gbx_free_ms_plan(p);
                return cuda_fail(e, "cudaMemcpyAsync", __FILE__, __LINE__);
            }
        }
        g->ms_plan = p;
    }
    *out = g->ms_plan;
    return GBX_OK;
}

template <int NW>
int msbfs_impl(gbx_graph *g, uint32_t S, const uint32_t *src_d, uint32_t *dist, gbx_bfs_result *res_host,
               cudaStream_t s) {
    const uint32_t V = g->V;
    gbx_ms_plan *plan = nullptr;
    GBX_TRY(ms_plan(g, s, &plan));
    const size_t words = (size_t)V * NW;
    // the level masks kept for the final pass: as many levels as fit 8 GiB
    // (at least two), at most kMsMaxStoredLevels; deeper levels use the two
    // `deep` buffers in turn and write their distances bit by bit
    const uint32_t max_stored = (uint32_t)std::max<size_t>(
        2, std::min<size_t>(kMsMaxStoredLevels, (8ull << 30) / std::max<size_t>(1, words * 4)));
    std::vector<DevBuf<uint32_t>> lvbuf(max_stored);
    DevBuf<uint32_t> seen, deep[2], q0, q1, rc, rd;
    DevBuf<unsigned long long> re;
    DevBuf<MsCounters> cnt;
    GBX_TRY(seen.alloc(words, s));
    GBX_TRY(lvbuf[0].alloc(words, s));
    GBX_TRY(q0.alloc(std::max(V, S), s));
    GBX_TRY(q1.alloc(std::max(V, S), s));
    GBX_TRY(cnt.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(seen.p, 0, words * 4, s));
    GBX_CUDA(cudaMemsetAsync(lvbuf[0].p, 0, words * 4, s));
    GBX_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(MsCounters), s));
    ms_seed_kernel<<<1, 256, 0, s>>>(src_d, S, NW, g->offsets, seen.p, lvbuf[0].p, q0.p, cnt.p);
    GBX_LAUNCH_CHECK();
    MsCounters h{};
    GBX_CUDA(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    uint32_t *F = lvbuf[0].p, *q = q0.p, *qn = q1.p;
    const unsigned grid = (unsigned)num_sms() * 8;
    const unsigned long long E = g->E;
    uint32_t level = 0, pushes = 0, pulls = 0, stored = 1;
    while (h.qn > 0 && level <= V) {
        const uint32_t next = level + 1;
        const bool keep = next < max_stored;
        uint32_t *Fn;
        if (keep) {
            GBX_TRY(lvbuf[next].alloc(words, s));
            Fn = lvbuf[next].p;
        } else {
            DevBuf<uint32_t> &d = deep[next & 1];
            if (!d.p) GBX_TRY(d.alloc(words, s));
            Fn = d.p;
        }
        GBX_CUDA(cudaMemsetAsync(Fn, 0, words * 4, s));
        if (h.mf * 16 < E) {
            ms_push_kernel<NW><<<grid, kMsThreads, 0, s>>>(g->offsets, g->dest, q, h.qn, F, seen.p, Fn);
            GBX_LAUNCH_CHECK();
            ++pushes;
        } else {
            ms_pull_light_kernel<NW><<<grid, kMsThreads, 0, s>>>(g->pull_offsets(), g->pull_src(), V, S, F, seen.p,
                                                                 Fn);
            GBX_LAUNCH_CHECK();
            if (plan->n_chunks) {
                ms_pull_heavy_kernel<NW><<<grid, kMsThreads, 0, s>>>(plan->chunks, plan->n_chunks, g->pull_src(), S,
                                                                     F, seen.p, Fn);
                GBX_LAUNCH_CHECK();
            }
            ++pulls;
        }
        level = next;
        GBX_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(MsCounters), s));
        if (keep) {
            ms_update_kernel<NW, false><<<grid, kMsThreads, 0, s>>>(V, S, level, g->offsets, seen.p, Fn, dist, qn,
                                                                    cnt.p);
            stored = next + 1;
        } else {
            ms_update_kernel<NW, true><<<grid, kMsThreads, 0, s>>>(V, S, level, g->offsets, seen.p, Fn, dist, qn,
                                                                   cnt.p);
        }
        GBX_LAUNCH_CHECK();
        GBX_CUDA(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        F = Fn;
        std::swap(q, qn);
    }
    GBX_REQUIRE(h.qn == 0, GBX_ERR_ITER_CAP, "multi-source BFS level cap reached");
    // distances of the stored levels, zeros for unreached pairs, and the
    // per-source results, in one pass
    MsLevels lv{};
    lv.n = stored;
    for (uint32_t L = 0; L < stored; ++L) lv.m[L] = lvbuf[L].p;
    GBX_TRY(rc.alloc(S, s));
    GBX_TRY(rd.alloc(S, s));
    GBX_TRY(re.alloc(S, s));
    GBX_CUDA(cudaMemsetAsync(rc.p, 0, 4 * (size_t)S, s));
    GBX_CUDA(cudaMemsetAsync(rd.p, 0, 4 * (size_t)S, s));
    GBX_CUDA(cudaMemsetAsync(re.p, 0, 8 * (size_t)S, s));
    const bool vec_rows = S % 4 == 0 && (reinterpret_cast<uintptr_t>(dist) & 15u) == 0;
    ms_final_kernel<NW><<<(unsigned)num_sms() * 4, kMsThreads, 0, s>>>(lv, seen.p, V, S, g->offsets, src_d,
                                                                       vec_rows, dist, rc.p, re.p, rd.p);
    GBX_LAUNCH_CHECK();
    if (res_host) {
        std::vector<uint32_t> hc(S), hd(S);
        std::vector<unsigned long long> he(S);
        GBX_CUDA(cudaMemcpyAsync(hc.data(), rc.p, 4 * (size_t)S, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaMemcpyAsync(hd.data(), rd.p, 4 * (size_t)S, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaMemcpyAsync(he.data(), re.p, 8 * (size_t)S, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        for (uint32_t i = 0; i < S; ++i) {
            gbx_bfs_result r{};
            r.processed_nodes = hc[i] + 1;
            r.depth = hd[i];
            r.iteration = hd[i] + 2;
            r.top_down_steps = pushes;
            r.bottom_up_steps = pulls;
            r.edges_traversed = he[i];
            res_host[i] = r;
        }
    } else {
        GBX_CUDA(cudaStreamSynchronize(s));
    }
    return GBX_OK;
}

}  // namespace

extern "C" int gbx_bfs_multisource(gbx_graph *g, uint32_t num_sources, const uint32_t *sources, uint32_t *distances,
                                   gbx_bfs_result *results, void *stream) {
    clear_error();
    GBX_REQUIRE(g && sources && distances, GBX_ERR_INVALID, "graph, sources or distances is NULL");
    GBX_REQUIRE(num_sources >= 1 && num_sources <= 256, GBX_ERR_INVALID, "num_sources must be 1..256 (got %u)",
                num_sources);
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<uint32_t> hs(num_sources);
    GBX_CUDA(cudaMemcpyAsync(hs.data(), sources, 4 * (size_t)num_sources, cudaMemcpyDefault, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    for (uint32_t i = 0; i < num_sources; ++i)
        GBX_REQUIRE(hs[i] < g->V, GBX_ERR_INVALID, "source %u (index %u) is not below %u vertices", hs[i], i, g->V);
    DevBuf<uint32_t> src_d;
    GBX_TRY(src_d.alloc(num_sources, s));
    GBX_CUDA(cudaMemcpyAsync(src_d.p, hs.data(), 4 * (size_t)num_sources, cudaMemcpyHostToDevice, s));
    OutArray<uint32_t> dist;
    GBX_TRY(dist.bind(distances, (size_t)g->V * num_sources, s));
    std::vector<gbx_bfs_result> hr;
    if (results) hr.resize(num_sources);
    const uint32_t nw = (num_sources + 31) / 32;
    int st;
    if (nw == 1)
        st = msbfs_impl<1>(g, num_sources, src_d.p, dist.d, results ? hr.data() : nullptr, s);
    else if (nw == 2)
        st = msbfs_impl<2>(g, num_sources, src_d.p, dist.d, results ? hr.data() : nullptr, s);
    else if (nw <= 4)
        st = msbfs_impl<4>(g, num_sources, src_d.p, dist.d, results ? hr.data() : nullptr, s);
    else
        st = msbfs_impl<8>(g, num_sources, src_d.p, dist.d, results ? hr.data() : nullptr, s);
    GBX_TRY(st);
    GBX_TRY(dist.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    if (results) std::copy(hr.begin(), hr.end(), results);
    return GBX_OK;
}
