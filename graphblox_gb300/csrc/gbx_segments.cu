// CSR segments: the reference's cache-blocked form of a graph (csrSegmentsNew,
// csrSegments.c:157-578). The vertex range is cut into num_segments ranges
// (getSegmentID, csrSegments.c:555-570: equal sizes, the first V % S ranges
// one longer), and every edge goes to the segment of its destination, so a
// segment's edges read sources from anywhere but write only into one
// destination range. This file builds the partition on the GPU:
//   out_degree / in_degree     per vertex over all edges
//                              (graphCSRSegmentsProcessInOutDegrees)
//   vertex_segment_index[v]    the segment of v for every destination v, 0
//                              for vertices that are no edge's destination
//                              (csrSegmentsSegmentEdgeListSizePreprocessing)
//   segment_num_edges[s]       edges of segment s
//   segment_max_id[s]          largest id among its edges' ends
//                              (csrSegmentsSegmentVertexSizePreprocessing)
//   seg_src / seg_dst / seg_weight
//                              the edges grouped by segment, in input order
//                              inside a segment (the order the reference's
//                              population loop gives with one thread)
// A stable radix sort of the edges' segment ids gives the grouping. The
// per-segment GraphCSR the reference then builds is the library's own
// preprocessing applied to each segment's edge list (graph.py,
// csr_segments).
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {
namespace {

__host__ __device__ __forceinline__ uint32_t segment_of(uint32_t V, uint32_t S, uint32_t id) {
    uint32_t size = V / S;
    if (V % S == 0) return id / size;
    size += 1;
    const uint32_t split = (V % S) * size;
    return id < split ? id / size : (id - split) / (size - 1) + V % S;
}

unsigned grid_for(uint64_t n) { return std::max(1u, std::min<unsigned>(ceil_div(n, 256), (unsigned)num_sms() * 8)); }

__global__ void seg_degrees_kernel(const uint32_t *src, const uint32_t *dst, uint32_t E, uint32_t V, uint32_t S,
                                   uint32_t *out_degree, uint32_t *in_degree, uint32_t *vsi, uint32_t *key,
                                   uint32_t *perm, uint32_t *bad) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const uint32_t s = src[i], d = dst[i];
        if (s >= V || d >= V) {  // reported to the host, never used as an index
            atomicExch(bad, 1u);
            key[i] = 0;
            perm[i] = i;
            continue;
        }
        atomicAdd(out_degree + s, 1u);
        atomicAdd(in_degree + d, 1u);
        const uint32_t seg = segment_of(V, S, d);
        vsi[d] = seg;
        key[i] = seg;
        perm[i] = i;
    }
}

// per-segment edge counts and largest ids, gathered in shared memory when
// the segments fit (nseg <= kSmemSegs), else straight into global memory
constexpr uint32_t kSmemSegs = 4096;
__global__ void seg_counts_kernel(const uint32_t *src, const uint32_t *dst, const uint32_t *key, uint32_t E,
                                  uint32_t S, uint32_t *count, uint32_t *max_id) {
    __shared__ uint32_t s_cnt[kSmemSegs], s_max[kSmemSegs];
    const bool smem = S <= kSmemSegs;
    if (smem) {
        for (uint32_t j = threadIdx.x; j < S; j += blockDim.x) s_cnt[j] = s_max[j] = 0;
        __syncthreads();
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const uint32_t k = key[i], m = max(src[i], dst[i]);
        if (smem) {
            atomicAdd(s_cnt + k, 1u);
            atomicMax(s_max + k, m);
        } else {
            atomicAdd(count + k, 1u);
            atomicMax(max_id + k, m);
        }
    }
    if (smem) {
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < S; j += blockDim.x) {
            if (s_cnt[j]) {
                atomicAdd(count + j, s_cnt[j]);
                atomicMax(max_id + j, s_max[j]);
            }
        }
    }
}

__global__ void seg_gather_kernel(const uint32_t *src, const uint32_t *dst, const float *w, const uint32_t *perm,
                                  uint32_t E, uint32_t *osrc, uint32_t *odst, float *ow) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const uint32_t p = perm[i];
        osrc[i] = src[p];
        odst[i] = dst[p];
        if (ow) ow[i] = w[p];
    }
}

}  // namespace
}  // namespace gbx

using namespace gbx;

extern "C" uint32_t gbx_csr_segments_count(uint32_t num_vertices, uint32_t cache_size) {
    // csrSegmentsCalculateSegments (csrSegments.c:538-553): 8 bytes per vertex
    // over the cache size, at least 4; in 32-bit arithmetic like the reference
    if (cache_size == 0) return 4;
    const uint32_t n = (num_vertices * 8u + cache_size - 1) / cache_size;
    return n < 4 ? 4 : n;
}

extern "C" int gbx_csr_segments(uint32_t num_edges, const uint32_t *src, const uint32_t *dst, const float *weight,
                                uint32_t num_vertices, uint32_t num_segments, uint32_t *out_degree,
                                uint32_t *in_degree, uint32_t *vertex_segment_index, uint32_t *segment_num_edges,
                                uint32_t *segment_max_id, uint32_t *seg_src, uint32_t *seg_dst, float *seg_weight,
                                void *stream) {
    clear_error();
    GBX_REQUIRE(num_vertices > 0, GBX_ERR_INVALID, "num_vertices must be > 0");
    GBX_REQUIRE(num_segments > 0, GBX_ERR_INVALID, "num_segments must be > 0");
    GBX_REQUIRE(num_edges == 0 || (src && dst && seg_src && seg_dst), GBX_ERR_INVALID, "NULL edge array");
    GBX_REQUIRE(out_degree && in_degree && vertex_segment_index && segment_num_edges && segment_max_id,
                GBX_ERR_INVALID, "NULL output array");
    GBX_REQUIRE(!seg_weight || weight, GBX_ERR_INVALID, "seg_weight needs weight");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t E = num_edges, V = num_vertices, S = num_segments;
    InArray<uint32_t> is, id;
    InArray<float> iw;
    GBX_TRY(is.bind(src, E, s));
    GBX_TRY(id.bind(dst, E, s));
    GBX_TRY(iw.bind(seg_weight ? weight : nullptr, E, s));
    OutArray<uint32_t> od, ideg, vsi, cnt, mx, os, odst;
    OutArray<float> ow;
    GBX_TRY(od.bind(out_degree, V, s));
    GBX_TRY(ideg.bind(in_degree, V, s));
    GBX_TRY(vsi.bind(vertex_segment_index, V, s));
    GBX_TRY(cnt.bind(segment_num_edges, S, s));
    GBX_TRY(mx.bind(segment_max_id, S, s));
    GBX_TRY(os.bind(seg_src, E, s));
    GBX_TRY(odst.bind(seg_dst, E, s));
    GBX_TRY(ow.bind(seg_weight, E, s));
    GBX_CUDA(cudaMemsetAsync(od.d, 0, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(ideg.d, 0, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(vsi.d, 0, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(cnt.d, 0, (size_t)S * 4, s));
    GBX_CUDA(cudaMemsetAsync(mx.d, 0, (size_t)S * 4, s));
    DevBuf<uint32_t> key, perm, bad;
    GBX_TRY(key.alloc(E ? E : 1, s));
    GBX_TRY(perm.alloc(E ? E : 1, s));
    GBX_TRY(bad.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
    if (E) {
        seg_degrees_kernel<<<grid_for(E), 256, 0, s>>>(is.d, id.d, E, V, S, od.d, ideg.d, vsi.d, key.p, perm.p,
                                                       bad.p);
        GBX_LAUNCH_CHECK();
        uint32_t hb = 0;
        GBX_CUDA(cudaMemcpyAsync(&hb, bad.p, 4, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        GBX_REQUIRE(hb == 0, GBX_ERR_INVALID, "an edge has an end outside [0, %u)", V);
        seg_counts_kernel<<<grid_for(E), 256, 0, s>>>(is.d, id.d, key.p, E, S, cnt.d, mx.d);
        GBX_LAUNCH_CHECK();
        int bits = 1;
        while (bits < 32 && ((S - 1) >> bits)) ++bits;
        GBX_TRY(radix_sort_pairs(key.p, perm.p, E, bits, s));  // stable: input order inside a segment
        seg_gather_kernel<<<grid_for(E), 256, 0, s>>>(is.d, id.d, iw.d, perm.p, E, os.d, odst.d,
                                                      seg_weight ? ow.d : nullptr);
        GBX_LAUNCH_CHECK();
    }
    GBX_TRY(od.finish(s));
    GBX_TRY(ideg.finish(s));
    GBX_TRY(vsi.finish(s));
    GBX_TRY(cnt.finish(s));
    GBX_TRY(mx.finish(s));
    GBX_TRY(os.finish(s));
    GBX_TRY(odst.finish(s));
    GBX_TRY(ow.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}
