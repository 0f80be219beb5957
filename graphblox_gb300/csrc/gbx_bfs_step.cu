// Single BFS steps for callers that drive the traversal themselves: the
// reference's topDownStepGraphCSR (BFS.c:498-546) and bottomUpStepGraphCSR
// (BFS.c:562-613) over a frontier the caller holds, with the parents and
// distances arrays of its BFSStats. gbx_bfs runs whole traversals in one
// persistent kernel; these entry points run one step per call.
//
// Top-down: a warp per frontier vertex v walks its out-edges; an edge to u
// whose parent is still negative (unvisited: -out_degree or -1) claims u by a
// compare-and-swap of that value to v, as the reference does, sets
// distances[u] = distances[v] + 1, appends u to the next frontier and adds
// -parents_old(u) to mf. Which frontier vertex wins u is a race, as in the
// reference; distances are not.
//
// Bottom-up: a thread per vertex v whose parent is negative scans its pull
// in-edges in order; the first in-neighbour u set in the current frontier
// bitmap becomes the parent, distances[v] = distances[u] + 1, and v is set in
// the next frontier bitmap (OR-ed in). Both parent and distance are
// deterministic, like the reference's.
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {
namespace {

constexpr uint32_t kIdMask = 0x3FFFFFFFu;  // EXTRACT_VALUE (reorder.h): mask-mode bits cleared

__global__ void td_step_kernel(const uint32_t *__restrict__ off, const uint32_t *__restrict__ dest, uint32_t V,
                               const uint32_t *__restrict__ frontier, uint32_t n, int32_t *parents,
                               uint32_t *distances, uint32_t *next, uint32_t next_cap, uint32_t *next_len,
                               unsigned long long *mf, uint32_t *overflow, uint32_t *bad_id) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long my_mf = 0;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nw) {
        const uint32_t v = frontier[i];
        if (v >= V) {  // not a vertex: reported, never dereferenced
            if (lane == 0) atomicExch(bad_id, 1u);
            continue;
        }
        const uint32_t b = off[v], e = off[v + 1];
        const uint32_t dnext = distances[v] + 1;
        for (uint32_t j0 = b; j0 < e; j0 += 32) {
            const uint32_t j = j0 + lane;
            bool won = false;
            uint32_t u = 0;
            if (j < e) {
                u = __ldg(dest + j) & kIdMask;
                const int32_t up = *((volatile int32_t *)parents + u);
                if (up < 0 && atomicCAS(parents + u, up, (int32_t)v) == up) {
                    won = true;
                    distances[u] = dnext;
                    my_mf += (unsigned long long)(uint32_t)(-up);
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, won);
            if (m) {
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(next_len, (uint32_t)__popc(m));
                base = __shfl_sync(0xffffffffu, base, 0);
                const uint32_t slot = base + __popc(m & ((1u << lane) - 1u));
                if (won) {
                    if (slot < next_cap) next[slot] = u;
                    else atomicExch(overflow, 1u);
                }
            }
        }
    }
    my_mf = warp_sum(my_mf);
    if (lane == 0 && my_mf) atomicAdd(mf, my_mf);
}

__global__ void bu_step_kernel(const uint32_t *__restrict__ poff, const uint32_t *__restrict__ psrc, uint32_t V,
                               const uint32_t *__restrict__ curr, uint32_t *next, int32_t *parents,
                               uint32_t *distances, uint32_t *nf) {
    uint32_t found = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        if (parents[v] >= 0) continue;
        const uint32_t b = poff[v], e = poff[v + 1];
        for (uint32_t j = b; j < e; ++j) {
            const uint32_t u = __ldg(psrc + j) & kIdMask;
            if ((__ldg(curr + (u >> 5)) >> (u & 31)) & 1u) {
                parents[v] = (int32_t)u;
                distances[v] = distances[u] + 1;
                atomicOr(next + (v >> 5), 1u << (v & 31));
                ++found;
                break;
            }
        }
    }
    found = warp_sum(found);
    if ((threadIdx.x & 31) == 0 && found) atomicAdd(nf, found);
}

// An in/out array: the caller's device memory as is, or a device copy of its
// host memory, copied back by finish().
template <typename T>
struct InOutArray {
    T *d = nullptr;
    T *host = nullptr;
    size_t n = 0;
    DevBuf<T> owned;
    int bind(T *p, size_t count, cudaStream_t s, bool upload = true) {
        n = count;
        if (is_device_ptr(p)) {
            d = p;
            return GBX_OK;
        }
        host = p;
        GBX_TRY(owned.alloc(count ? count : 1, s));
        d = owned.p;
        if (upload && count) GBX_CUDA(cudaMemcpyAsync(d, p, count * sizeof(T), cudaMemcpyHostToDevice, s));
        return GBX_OK;
    }
    int finish(cudaStream_t s, size_t count) {
        if (host && count) GBX_CUDA(cudaMemcpyAsync(host, d, count * sizeof(T), cudaMemcpyDeviceToHost, s));
        return GBX_OK;
    }
};

}  // namespace
}  // namespace gbx

using namespace gbx;

extern "C" int gbx_bfs_top_down_step(gbx_graph *g, const uint32_t *frontier, uint32_t frontier_len,
                                     int32_t *parents, uint32_t *distances, uint32_t *next, uint32_t next_capacity,
                                     uint32_t *next_len, uint32_t *mf, void *stream) {
    clear_error();
    GBX_REQUIRE(g, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(parents && distances && next_len && mf, GBX_ERR_INVALID, "NULL array argument");
    GBX_REQUIRE(frontier_len == 0 || (frontier && next), GBX_ERR_INVALID, "NULL frontier or next array");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    InArray<uint32_t> fr;
    GBX_TRY(fr.bind(frontier, frontier_len, s));
    if (frontier_len && !is_device_ptr(frontier)) {
        // ids outside the graph would index past parents[]: check them here
        for (uint32_t i = 0; i < frontier_len; ++i)
            GBX_REQUIRE(frontier[i] < V, GBX_ERR_INVALID, "frontier vertex %u out of range [0, %u)", frontier[i], V);
    }
    InOutArray<int32_t> par;
    InOutArray<uint32_t> dist;
    InOutArray<uint32_t> nx;
    GBX_TRY(par.bind(parents, V, s));
    GBX_TRY(dist.bind(distances, V, s));
    GBX_TRY(nx.bind(next, next_capacity, s, false));
    DevBuf<unsigned long long> ctr;  // [0] next_len, [1] mf, [2] overflow, [3] frontier id out of range
    GBX_TRY(ctr.alloc(4, s));
    GBX_CUDA(cudaMemsetAsync(ctr.p, 0, 4 * sizeof(unsigned long long), s));
    uint32_t *len_d = reinterpret_cast<uint32_t *>(ctr.p);
    uint32_t *ovf_d = reinterpret_cast<uint32_t *>(ctr.p + 2);
    uint32_t *bad_d = reinterpret_cast<uint32_t *>(ctr.p + 3);
    if (frontier_len) {
        const unsigned grid = std::min<unsigned>(ceil_div((uint64_t)frontier_len * 32, 256), (unsigned)num_sms() * 8);
        td_step_kernel<<<grid, 256, 0, s>>>(g->offsets, g->dest, V, fr.d, frontier_len, par.d, dist.d, nx.d,
                                            next_capacity, len_d, ctr.p + 1, ovf_d, bad_d);
        GBX_LAUNCH_CHECK();
    }
    unsigned long long h[4];
    GBX_CUDA(cudaMemcpyAsync(h, ctr.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    const uint32_t got = (uint32_t)(h[0] & 0xFFFFFFFFull);
    GBX_REQUIRE((uint32_t)(h[3] & 0xFFFFFFFFull) == 0, GBX_ERR_INVALID, "a frontier vertex is out of range [0, %u)",
                V);
    GBX_REQUIRE((uint32_t)(h[2] & 0xFFFFFFFFull) == 0, GBX_ERR_INVALID,
                "next frontier holds %u vertices, more than its capacity %u", got, next_capacity);
    GBX_TRY(par.finish(s, V));
    GBX_TRY(dist.finish(s, V));
    GBX_TRY(nx.finish(s, std::min(got, next_capacity)));
    GBX_CUDA(cudaStreamSynchronize(s));
    *next_len = got;
    *mf = (uint32_t)h[1];
    return GBX_OK;
}

extern "C" int gbx_bfs_bottom_up_step(gbx_graph *g, const uint32_t *bitmap_curr, uint32_t *bitmap_next,
                                      int32_t *parents, uint32_t *distances, uint32_t *nf, void *stream) {
    clear_error();
    GBX_REQUIRE(g, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(bitmap_curr && bitmap_next && parents && distances && nf, GBX_ERR_INVALID, "NULL array argument");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V, words = (V + 31) / 32;
    InArray<uint32_t> cur;
    GBX_TRY(cur.bind(bitmap_curr, words, s));
    InOutArray<uint32_t> nxt;
    InOutArray<int32_t> par;
    InOutArray<uint32_t> dist;
    GBX_TRY(nxt.bind(bitmap_next, words, s));
    GBX_TRY(par.bind(parents, V, s));
    GBX_TRY(dist.bind(distances, V, s));
    DevBuf<uint32_t> cnt;
    GBX_TRY(cnt.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(cnt.p, 0, 4, s));
    if (V) {
        const unsigned grid = std::min<unsigned>(ceil_div(V, 256), (unsigned)num_sms() * 8);
        bu_step_kernel<<<grid, 256, 0, s>>>(g->pull_offsets(), g->pull_src(), V, cur.d, nxt.d, par.d, dist.d,
                                            cnt.p);
        GBX_LAUNCH_CHECK();
    }
    uint32_t h = 0;
    GBX_CUDA(cudaMemcpyAsync(&h, cnt.p, 4, cudaMemcpyDeviceToHost, s));
    GBX_TRY(nxt.finish(s, words));
    GBX_TRY(par.finish(s, V));
    GBX_TRY(dist.finish(s, V));
    GBX_CUDA(cudaStreamSynchronize(s));
    *nf = h;
    return GBX_OK;
}
