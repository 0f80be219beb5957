// Single-source shortest paths (the reference's SSSPDataDrivenPushGraphCSR,
// SSSP.c:514-653, with its relaxation SSSPAtomicRelax, :180-254).
//
// Near/far delta-stepping: vertices whose tentative distance is below the
// current threshold form the "near" queue and are relaxed round after round
// (edge-balanced expansion, atomicMin on dist[]); improvements at or above
// the threshold go to the "far" pile (each vertex at most once, flagged).
// When near drains, the threshold jumps past the smallest far distance
// (empty buckets cost nothing, unlike the reference's full-V bucket scans),
// and far entries that fall below it move to near. A vertex is re-expanded
// only if its distance changed since it was last expanded, so the result is
// the unique fixed point dist[u] = min over (v->u) of (uint32)((float)dist[v] + w),
// identical to the reference's distances.
#include <algorithm>

#include "gbx_frontier.cuh"

namespace gbx {

__global__ void gather_queue_degrees_kernel(const uint32_t *q, uint32_t qlen, const uint32_t *deg,
                                            uint32_t *out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < qlen; i += gridDim.x * blockDim.x)
        out[i] = deg[q[i]];
}

struct SsspCounters {
    uint32_t near_len;
    uint32_t far_len;
    uint32_t far_min;
    uint32_t pad;
    unsigned long long relaxed;
};

__device__ __forceinline__ uint32_t sssp_add(uint32_t d, float w) {
    // SSSP.c:204: uint32 + float evaluated in float, truncated back to uint32
    return __float2uint_rz(__fadd_rn(__uint2float_rn(d), w));
}

struct RelaxVisitor {
    uint32_t *dist;
    const uint32_t *settled;  // distance each queued vertex was expanded with
    const float *w;
    uint32_t threshold;
    uint32_t round;
    uint32_t *stamp;
    uint32_t *in_far;
    uint32_t *near_next;
    uint32_t *far;
    SsspCounters *cnt;
    unsigned long long relaxed;
    __device__ __forceinline__ void operator()(uint32_t v, uint32_t e, uint32_t u, bool active) {
        bool to_near = false, to_far = false;
        if (active) {
            uint32_t d = __ldg(settled + v);
            float wt = w ? __ldg(w + e) : 1.0f;
            uint32_t nd = sssp_add(d, wt);
            relaxed++;
            if (nd < __ldcg(dist + u)) {
                uint32_t old = atomicMin(dist + u, nd);
                if (nd < old) {
                    if (nd < threshold) to_near = atomicExch(stamp + u, round) != round;
                    else to_far = atomicExch(in_far + u, 1u) == 0u;
                }
            }
        }
        warp_append(near_next, &cnt->near_len, u, to_near);
        warp_append(far, &cnt->far_len, u, to_far);
    }
    __device__ __forceinline__ void finish() {
        unsigned long long r = warp_sum(relaxed);
        if ((threadIdx.x & 31) == 0 && r) atomicAdd(&cnt->relaxed, r);
    }
};

// degrees of the near queue + snapshot of the distances used to expand it
__global__ void sssp_prepare_kernel(const uint32_t *q, uint32_t qlen, const uint32_t *deg,
                                    const uint32_t *dist, uint32_t *settled, uint32_t *degs) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < qlen; i += gridDim.x * blockDim.x) {
        uint32_t v = q[i];
        degs[i] = deg[v];
        settled[v] = dist[v];
    }
}

__global__ void far_min_kernel(const uint32_t *far, uint32_t n, const uint32_t *dist,
                               const uint32_t *settled, SsspCounters *cnt) {
    uint32_t m = 0xFFFFFFFFu;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t u = far[i];
        uint32_t d = dist[u];
        if (settled[u] != d) m = min(m, d);
    }
    m = __reduce_min_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0 && m != 0xFFFFFFFFu) atomicMin(&cnt->far_min, m);
}

__global__ void far_split_kernel(const uint32_t *far, uint32_t n, const uint32_t *dist,
                                 const uint32_t *settled, uint32_t threshold, uint32_t round,
                                 uint32_t *stamp, uint32_t *in_far, uint32_t *near, uint32_t *far2,
                                 SsspCounters *cnt) {
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        uint32_t i = base + threadIdx.x;
        bool to_near = false, keep = false;
        uint32_t u = 0;
        if (i < n) {
            u = far[i];
            uint32_t d = dist[u];
            if (settled[u] == d) {
                in_far[u] = 0;  // already expanded at this distance
            } else if (d < threshold) {
                in_far[u] = 0;
                to_near = atomicExch(stamp + u, round) != round;
            } else {
                keep = true;
            }
        }
        warp_append(near, &cnt->near_len, u, to_near);
        warp_append(far2, &cnt->far_len, u, keep);
    }
}

__global__ void sssp_init_kernel(uint32_t *dist, uint32_t *settled, uint32_t *stamp, uint32_t *in_far,
                                 uint32_t V, uint32_t source) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        dist[v] = v == source ? 0u : kSsspInf;
        settled[v] = 0xFFFFFFFFu;
        stamp[v] = v == source ? 1u : 0u;
        in_far[v] = 0;
    }
}

__global__ void sssp_finish_kernel(const uint32_t *dist, const uint32_t *outdeg, uint32_t V,
                                   uint32_t *out, unsigned long long *stats /* reached, edges */) {
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
    if (delta == 0) delta = g->weight ? 256u : 1u;
    DevBuf<uint32_t> dist, settled, stamp, in_far, qa, qb, fa, fb, degs, pre, total;
    DevBuf<SsspCounters> cnt;
    DevBuf<unsigned long long> fin;
    GBX_TRY(dist.alloc(V, s));
    GBX_TRY(settled.alloc(V, s));
    GBX_TRY(stamp.alloc(V, s));
    GBX_TRY(in_far.alloc(V, s));
    GBX_TRY(qa.alloc(V, s));
    GBX_TRY(qb.alloc(V, s));
    GBX_TRY(fa.alloc(V, s));
    GBX_TRY(fb.alloc(V, s));
    GBX_TRY(degs.alloc(V, s));
    GBX_TRY(pre.alloc(V, s));
    GBX_TRY(total.alloc(1, s));
    GBX_TRY(cnt.alloc(1, s));
    GBX_TRY(fin.alloc(2, s));
    OutArray<uint32_t> out;
    GBX_TRY(out.bind(distances, V, s));
    const unsigned grid = std::min<unsigned>(ceil_div(V, 256), (unsigned)num_sms() * 8);
    sssp_init_kernel<<<grid, 256, 0, s>>>(dist.p, settled.p, stamp.p, in_far.p, V, source);
    GBX_LAUNCH_CHECK();
    GBX_CUDA(cudaMemcpyAsync(qa.p, &source, 4, cudaMemcpyHostToDevice, s));
    uint32_t *nearq = qa.p, *nextq = qb.p, *farq = fa.p, *far2 = fb.p;
    uint32_t near_len = 1, far_len = 0, round = 1, rounds = 0;
    uint64_t threshold = delta;
    unsigned long long relaxed = 0;
    SsspCounters h;
    const uint32_t max_rounds = 4u * V + 64u;  // hard cap: every round settles >= 1 vertex
    for (;;) {
        while (near_len > 0) {
            GBX_REQUIRE(rounds < max_rounds, GBX_ERR_ITER_CAP, "SSSP round cap reached");
            GBX_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(SsspCounters), s));
            GBX_CUDA(cudaMemcpyAsync(&cnt.p->far_len, &far_len, 4, cudaMemcpyHostToDevice, s));
            unsigned pg = std::min<unsigned>(ceil_div(near_len, 256), (unsigned)num_sms() * 8);
            sssp_prepare_kernel<<<pg, 256, 0, s>>>(nearq, near_len, g->out_degree, dist.p, settled.p, degs.p);
            GBX_LAUNCH_CHECK();
            GBX_TRY(exclusive_scan_u32(degs.p, pre.p, near_len, s, total.p));
            round++;
            uint32_t thr = threshold > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)threshold;
            RelaxVisitor vis{dist.p, settled.p, g->weight, thr, round, stamp.p, in_far.p,
                             nextq, farq, cnt.p, 0ull};
            expand_kernel<RelaxVisitor><<<num_sms() * 8, kExpThreads, 0, s>>>(
                nearq, pre.p, near_len, total.p, g->offsets, g->dest, vis);
            GBX_LAUNCH_CHECK();
            GBX_CUDA(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
            GBX_CUDA(cudaStreamSynchronize(s));
            relaxed += h.relaxed;
            near_len = h.near_len;
            far_len = h.far_len;
            std::swap(nearq, nextq);
            rounds++;
        }
        if (far_len == 0) break;
        // next threshold: one delta past the smallest pending far distance
        GBX_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(SsspCounters), s));
        uint32_t big = 0xFFFFFFFFu;
        GBX_CUDA(cudaMemcpyAsync(&cnt.p->far_min, &big, 4, cudaMemcpyHostToDevice, s));
        unsigned fg = std::min<unsigned>(ceil_div(far_len, 256), (unsigned)num_sms() * 8);
        far_min_kernel<<<fg, 256, 0, s>>>(farq, far_len, dist.p, settled.p, cnt.p);
        GBX_LAUNCH_CHECK();
        GBX_CUDA(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        if (h.far_min == 0xFFFFFFFFu) break;  // every far entry is already expanded
        threshold = ((uint64_t)h.far_min / delta + 1) * delta;
        round++;
        GBX_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(SsspCounters), s));
        uint32_t thr = threshold > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)threshold;
        far_split_kernel<<<fg, 256, 0, s>>>(farq, far_len, dist.p, settled.p, thr, round, stamp.p,
                                            in_far.p, nearq, far2, cnt.p);
        GBX_LAUNCH_CHECK();
        GBX_CUDA(cudaMemcpyAsync(&h, cnt.p, sizeof(h), cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        near_len = h.near_len;
        far_len = h.far_len;
        std::swap(farq, far2);
        // the near queue was filled under `round`; expansion rounds continue from there
    }
    GBX_CUDA(cudaMemsetAsync(fin.p, 0, 16, s));
    sssp_finish_kernel<<<grid, 256, 0, s>>>(dist.p, g->out_degree, V, out.d, fin.p);
    GBX_LAUNCH_CHECK();
    GBX_TRY(out.finish(s));
    unsigned long long hf[2];
    GBX_CUDA(cudaMemcpyAsync(hf, fin.p, 16, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    if (result) {
        result->reached = (uint32_t)hf[0];
        result->rounds = rounds;
        result->edges_relaxed = relaxed;
        result->edges_traversed = hf[1];
    }
    return GBX_OK;
}
