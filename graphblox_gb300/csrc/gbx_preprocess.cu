// Device preprocessing: the CSR build from an edge list and the degree
// reordering, i.e. the GPU form of graphCSRPreProcessingStep's sort / dedup /
// map steps (graphCSR.c:243-327) and of reorderGraphProcessDegree
// (reorder.c:275-380).
#include <algorithm>

#include "gbx_internal.cuh"

namespace gbx {

static unsigned grid1d(uint64_t n) {
    uint64_t b = (n + 255) / 256;
    uint64_t cap = (uint64_t)num_sms() * 8;
    return (unsigned)std::max<uint64_t>(1, std::min(b, cap));
}

__global__ void iota_kernel(uint32_t *a, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

// symmetric: second half holds every edge reversed (edgeList.c:559-576)
__global__ void stage_edges_kernel(const uint32_t *src, const uint32_t *dst, const float *w,
                                   uint32_t E, int symmetric, uint32_t *s, uint32_t *d, float *wo) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        uint32_t a = src[i], b = dst[i];
        s[i] = a;
        d[i] = b;
        if (wo) wo[i] = w ? w[i] : 1.0f;
        if (symmetric) {
            s[i + E] = b;
            d[i + E] = a;
            if (wo) wo[i + E] = w ? w[i] : 1.0f;
        }
    }
}

__global__ void max_id_kernel(const uint32_t *s, const uint32_t *d, uint32_t n, uint32_t *out) {
    uint32_t m = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        m = max(m, max(s[i], d[i]));
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// out[0] = largest id, out[1] = largest id without the mask bits
__global__ void id_range_kernel(const uint32_t *s, const uint32_t *d, uint32_t n, uint32_t *out) {
    uint32_t m = 0, mm = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t a = s[i], b = d[i];
        m = max(m, max(a, b));
        mm = max(mm, max(a & kIdMask, b & kIdMask));
    }
    m = __reduce_max_sync(0xffffffffu, m);
    mm = __reduce_max_sync(0xffffffffu, mm);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, m);
        atomicMax(out + 1, mm);
    }
}

// Largest id of an edge list (device scalar read back), 0 for no edges.
static int max_edge_id(const uint32_t *s, const uint32_t *d, uint32_t n, cudaStream_t st, uint32_t *full,
                       uint32_t *masked) {
    *full = *masked = 0;
    if (!n) return GBX_OK;
    DevBuf<uint32_t> r;
    GBX_TRY(r.alloc(2, st));
    GBX_CUDA(cudaMemsetAsync(r.p, 0, 8, st));
    id_range_kernel<<<grid1d(n), 256, 0, st>>>(s, d, n, r.p);
    GBX_LAUNCH_CHECK();
    uint32_t h[2];
    GBX_CUDA(cudaMemcpyAsync(h, r.p, 8, cudaMemcpyDeviceToHost, st));
    GBX_CUDA(cudaStreamSynchronize(st));
    *full = h[0];
    *masked = h[1];
    return GBX_OK;
}

__global__ void gather_u32_kernel(const uint32_t *in, const uint32_t *perm, uint32_t n, uint32_t *out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = in[perm[i]];
}

__global__ void gather_f32_kernel(const float *in, const uint32_t *perm, uint32_t n, float *out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = in[perm[i]];
}

// removeDulpicatesSelfLoopEdges on a (src,dst)-sorted list: keep edge i when
// it is not a self loop and differs from edge i-1 (edgeList.c:255-321)
__global__ void dedup_flags_kernel(const uint32_t *s, const uint32_t *d, uint32_t n, uint32_t *keep) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t a = s[i], b = d[i];
        bool k = a != b && (i == 0 || a != s[i - 1] || b != d[i - 1]);
        keep[i] = k ? 1u : 0u;
    }
}

// compaction; kept weights are truncated through uint32 as the reference's
// uint32_t tempWeight does (edgeList.c:260,273)
__global__ void compact_edges_kernel(const uint32_t *s, const uint32_t *d, const float *w,
                                     const uint32_t *keep, const uint32_t *pos, uint32_t n,
                                     uint32_t *so, uint32_t *dout, float *wo) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        uint32_t p = pos[i];
        so[p] = s[i];
        dout[p] = d[i];
        if (wo) wo[p] = (float)(uint32_t)w[i];
    }
}

// mapVerticesWithInOutDegree_base (vertex.c:204-328) on a source-sorted edge
// list: each run of equal sources writes its first position (idx) and its end
// (into deg); degrees_from_runs_kernel turns the end into the run length. No
// atomics: a hub's run would otherwise take one atomic per edge on one address.
__global__ void map_vertices_kernel(const uint32_t *s, uint32_t n, uint32_t *deg, uint32_t *idx) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t v = s[i] & kIdMask;
        if (i == 0 || v != (s[i - 1] & kIdMask)) idx[v] = i;
        if (i + 1 == n || v != (s[i + 1] & kIdMask)) deg[v] = i + 1;
    }
}

__global__ void degrees_from_runs_kernel(uint32_t *deg, const uint32_t *idx, uint32_t V) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        if (deg[v]) deg[v] -= idx[v];
}

// deg[key] += 1 for the active lanes, one atomic per distinct key in the warp
// (edge lists sorted by source repeat a key along the warp; hubs repeat
// everywhere, and one address taking every increment serialises the atomics)
__device__ __forceinline__ void count_keys(uint32_t *deg, uint32_t key, unsigned active) {
    const uint32_t lane = threadIdx.x & 31;
    if ((active >> lane) & 1u) {
        const unsigned peers = __match_any_sync(active, key);
        if (lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(deg + key, (uint32_t)__popc(peers));
    }
}

__global__ void degree_count_kernel(const uint32_t *s, const uint32_t *d, uint32_t n, int lmode,
                                    uint32_t *deg) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;  // a multiple of 32
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < n; base += stride) {
        const uint32_t i = base + lane;
        const unsigned active = __ballot_sync(0xffffffffu, i < n);
        if (lmode == 2 || lmode == 3) count_keys(deg, i < n ? d[i] : 0u, active);
        if (lmode != 2) count_keys(deg, i < n ? s[i] : 0u, active);
    }
}

__global__ void new_labels_kernel(const uint32_t *sorted_ids, uint32_t V, uint32_t *newlab) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x)
        newlab[sorted_ids[i]] = V - 1 - i;
}

__global__ void relabel_edges_kernel(uint32_t *s, uint32_t *d, uint32_t n, const uint32_t *newlab) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        s[i] = newlab[s[i]];
        d[i] = newlab[d[i]];
    }
}

// label_array[v] = labels[label_array[v]]; inverse[label_array[v]] = v  (reorder.c:368-373)
__global__ void compose_labels_kernel(uint32_t *labels, uint32_t *inv, uint32_t V, const uint32_t *newlab) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        uint32_t l = newlab[labels[v]];
        labels[v] = l;
        inv[l] = v;
    }
}

// ---- bucketed reorder modes (DBG, HUBSort, HUBCluster, Corder) -------------
struct BucketThresholds {
    uint32_t t[11];
    uint32_t n;
};

// key[v] = n-1 - bucket(v): a stable ascending sort of (key, id) lists the
// highest bucket first, ids ascending inside a bucket (reorder.c:439-572)
__global__ void bucket_key_kernel(const uint32_t *deg, uint32_t V, BucketThresholds th, uint32_t *key) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        uint32_t i = 0;
        while (deg[v] > th.t[i]) ++i;  // th.t[th.n-1] = UINT32_MAX ends the scan
        key[v] = th.n - 1 - i;
    }
}

// newlab[sorted[i]] = i
__global__ void rank_labels_kernel(const uint32_t *sorted, uint32_t n, uint32_t *newlab) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        newlab[sorted[i]] = i;
}

// HUBSort: hot flag (degree above t0) per vertex
__global__ void hot_flag_kernel(const uint32_t *deg, uint32_t V, uint32_t t0, uint32_t *flag) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        flag[v] = deg[v] > t0 ? 1u : 0u;
}

// hot vertices (ascending ids) and their degrees at their rank; cold vertices
// labelled H + (their rank among cold vertices) = H + v - (hot before v)
__global__ void hot_split_kernel(const uint32_t *deg, const uint32_t *flag, const uint32_t *pos, uint32_t V,
                                 const uint32_t *hot_total, uint32_t *hot_ids, uint32_t *hot_deg,
                                 uint32_t *newlab) {
    const uint32_t H = *hot_total;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        if (flag[v]) {
            hot_ids[pos[v]] = v;
            hot_deg[pos[v]] = deg[v];
        } else {
            newlab[v] = H + v - pos[v];
        }
    }
}

// bad[0] counts labels out of range or taken twice (seen[] starts zeroed)
__global__ void permutation_check_kernel(const uint32_t *lab, uint32_t V, uint32_t *seen, unsigned *bad) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const uint32_t l = lab[v];
        if (l >= V || atomicExch(seen + l, 1u) != 0u) atomicAdd(bad, 1u);
    }
}

// ---- mask mode (maskGraphProcess, reorder.c:1164-1475) --------------------
// The vertex at position i of the bucket order takes the first region with
// room left (reorder.c:1408-1436): HOT below e0, WARM below e1, LUKEWARM
// below e2 (cumulative region ends), COLD after.
__global__ void mask_hints_kernel(const uint32_t *sorted, uint32_t V, uint64_t e0, uint64_t e1, uint64_t e2,
                                  uint32_t *mask) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x)
        mask[sorted[i]] = i < e0 ? 0xC0000000u : i < e1 ? 0x80000000u : i < e2 ? 0x40000000u : 0u;
}

// maskEdgeList (reorder.c:1639-1657): every id ORed with its vertex's hint
__global__ void mask_edges_kernel(uint32_t *s, uint32_t *d, uint32_t n, const uint32_t *mask) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t a = s[i], b = d[i];
        s[i] = a | mask[a];
        d[i] = b | mask[b];
    }
}

static int bits_for(uint32_t maxv) {
    int b = 0;
    while (b < 32 && (maxv >> b)) ++b;
    return b;
}

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_csr_build(uint32_t num_edges, const uint32_t *src, const uint32_t *dst,
                             const float *w, int symmetric, int dedup, int sort_mode,
                             uint32_t num_vertices, uint32_t *out_degree, uint32_t *edges_idx,
                             uint32_t *src_out, uint32_t *dst_out, float *w_out,
                             uint32_t *num_edges_out, void *stream) {
    clear_error();
    GBX_REQUIRE(num_edges == 0 || (src && dst), GBX_ERR_INVALID, "src/dst is NULL");
    GBX_REQUIRE(out_degree && edges_idx && num_edges_out, GBX_ERR_INVALID, "output is NULL");
    GBX_REQUIRE(num_vertices > 0, GBX_ERR_INVALID, "num_vertices must be > 0");
    GBX_REQUIRE(!dedup || sort_mode == 1 || sort_mode == 3, GBX_ERR_INVALID,
                "dedup needs a (source,destination) sort (sort_mode 1)");
    GBX_REQUIRE(!symmetric || num_edges <= 0x7FFFFFFFu, GBX_ERR_INVALID, "too many edges");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t E = num_edges, E2 = symmetric ? 2 * num_edges : num_edges, V = num_vertices;
    InArray<uint32_t> isrc, idst;
    InArray<float> iw;
    GBX_TRY(isrc.bind(src, E, s));
    GBX_TRY(idst.bind(dst, E, s));
    GBX_TRY(iw.bind(w, E, s));
    const bool want_w = w_out != nullptr;
    DevBuf<uint32_t> es, ed, perm, keys;
    DevBuf<float> ew;
    GBX_TRY(es.alloc(E2, s));
    GBX_TRY(ed.alloc(E2, s));
    GBX_TRY(perm.alloc(E2, s));
    GBX_TRY(keys.alloc(E2, s));
    if (want_w) GBX_TRY(ew.alloc(E2, s));
    if (E) {
        stage_edges_kernel<<<grid1d(E), 256, 0, s>>>(isrc.d, idst.d, iw.d, E, symmetric, es.p, ed.p,
                                                     want_w ? ew.p : nullptr);
        GBX_LAUNCH_CHECK();
    }
    // ids may carry the mask bits of mask mode: the vertex is the id without
    // them, the sort key the whole id (the reference radix-sorts all 32 bits)
    uint32_t hmax = 0, hmasked = 0;
    GBX_TRY(max_edge_id(es.p, ed.p, E2, s, &hmax, &hmasked));
    GBX_REQUIRE(E2 == 0 || hmasked < V, GBX_ERR_INVALID, "vertex id %u >= num_vertices %u", hmasked, V);
    const int bits = bits_for(hmax);
    // stable sort: destination pass(es) first, then source (LSD on the pair)
    iota_kernel<<<grid1d(E2), 256, 0, s>>>(perm.p, E2);
    GBX_LAUNCH_CHECK();
    if (sort_mode == 1 || sort_mode == 3) {
        GBX_CUDA(cudaMemcpyAsync(keys.p, ed.p, (size_t)E2 * 4, cudaMemcpyDeviceToDevice, s));
        GBX_TRY(radix_sort_pairs(keys.p, perm.p, E2, bits, s));
    }
    gather_u32_kernel<<<grid1d(E2), 256, 0, s>>>(es.p, perm.p, E2, keys.p);
    GBX_LAUNCH_CHECK();
    GBX_TRY(radix_sort_pairs(keys.p, perm.p, E2, bits, s));
    // apply the permutation
    DevBuf<uint32_t> ss, sd, keep, pos, tot;
    DevBuf<float> sw;
    GBX_TRY(ss.alloc(E2, s));
    GBX_TRY(sd.alloc(E2, s));
    if (want_w) GBX_TRY(sw.alloc(E2, s));
    GBX_CUDA(cudaMemcpyAsync(ss.p, keys.p, (size_t)E2 * 4, cudaMemcpyDeviceToDevice, s));
    gather_u32_kernel<<<grid1d(E2), 256, 0, s>>>(ed.p, perm.p, E2, sd.p);
    if (want_w) gather_f32_kernel<<<grid1d(E2), 256, 0, s>>>(ew.p, perm.p, E2, sw.p);
    GBX_LAUNCH_CHECK();
    uint32_t Eout = E2;
    OutArray<uint32_t> os, od, odeg, oidx;
    OutArray<float> ow;
    const uint32_t *fs = ss.p, *fd = sd.p;
    const float *fw = sw.p;
    if (dedup && E2) {
        GBX_TRY(keep.alloc(E2, s));
        GBX_TRY(pos.alloc(E2, s));
        GBX_TRY(tot.alloc(1, s));
        dedup_flags_kernel<<<grid1d(E2), 256, 0, s>>>(ss.p, sd.p, E2, keep.p);
        GBX_LAUNCH_CHECK();
        GBX_TRY(exclusive_scan_u32(keep.p, pos.p, E2, s, tot.p));
        GBX_CUDA(cudaMemcpyAsync(&Eout, tot.p, 4, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        // compact into es/ed/ew (free now)
        compact_edges_kernel<<<grid1d(E2), 256, 0, s>>>(ss.p, sd.p, sw.p, keep.p, pos.p, E2, es.p,
                                                        ed.p, want_w ? ew.p : nullptr);
        GBX_LAUNCH_CHECK();
        fs = es.p;
        fd = ed.p;
        fw = ew.p;
    }
    GBX_TRY(odeg.bind(out_degree, V, s));
    GBX_TRY(oidx.bind(edges_idx, V, s));
    GBX_CUDA(cudaMemsetAsync(odeg.d, 0, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(oidx.d, 0, (size_t)V * 4, s));
    if (Eout) {
        map_vertices_kernel<<<grid1d(Eout), 256, 0, s>>>(fs, Eout, odeg.d, oidx.d);
        GBX_LAUNCH_CHECK();
        degrees_from_runs_kernel<<<grid1d(V), 256, 0, s>>>(odeg.d, oidx.d, V);
        GBX_LAUNCH_CHECK();
    }
    GBX_TRY(odeg.finish(s));
    GBX_TRY(oidx.finish(s));
    if (src_out) {
        GBX_TRY(os.bind(src_out, Eout, s));
        GBX_CUDA(cudaMemcpyAsync(os.d, fs, (size_t)Eout * 4, cudaMemcpyDeviceToDevice, s));
        GBX_TRY(os.finish(s));
    }
    if (dst_out) {
        GBX_TRY(od.bind(dst_out, Eout, s));
        GBX_CUDA(cudaMemcpyAsync(od.d, fd, (size_t)Eout * 4, cudaMemcpyDeviceToDevice, s));
        GBX_TRY(od.finish(s));
    }
    if (want_w) {
        GBX_TRY(ow.bind(w_out, Eout, s));
        GBX_CUDA(cudaMemcpyAsync(ow.d, fw, (size_t)Eout * 4, cudaMemcpyDeviceToDevice, s));
        GBX_TRY(ow.finish(s));
    }
    GBX_CUDA(cudaStreamSynchronize(s));
    *num_edges_out = Eout;
    return GBX_OK;
}

extern "C" int gbx_degree_reorder(uint32_t num_vertices, uint32_t num_edges, uint32_t *src,
                                  uint32_t *dst, int lmode, uint32_t *labels,
                                  uint32_t *inverse_labels, void *stream) {
    clear_error();
    GBX_REQUIRE(num_vertices > 0, GBX_ERR_INVALID, "num_vertices must be > 0");
    GBX_REQUIRE(num_edges == 0 || (src && dst), GBX_ERR_INVALID, "src/dst is NULL");
    GBX_REQUIRE(labels && inverse_labels, GBX_ERR_INVALID, "labels is NULL");
    GBX_REQUIRE(lmode != 10, GBX_ERR_UNSUPPORTED,
                "lmode 10 (random order) draws per-thread random degrees in the reference and is not "
                "reproducible; relabel with explicit labels (gbx_relabel) instead");
    GBX_REQUIRE(lmode != 11, GBX_ERR_INVALID, "lmode 11 (labels from a file): call gbx_relabel with the labels");
    GBX_REQUIRE((lmode >= 1 && lmode <= 9) || lmode == 12 || lmode == 13, GBX_ERR_INVALID,
                "lmode must be 1-9, 12 or 13");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = num_vertices, E = num_edges;
    OutArray<uint32_t> os, od, ol, oi;
    GBX_TRY(os.bind(src, E, s));
    GBX_TRY(od.bind(dst, E, s));
    GBX_TRY(ol.bind(labels, V, s));
    GBX_TRY(oi.bind(inverse_labels, V, s));
    if (os.to_host() && E) GBX_CUDA(cudaMemcpyAsync(os.d, src, (size_t)E * 4, cudaMemcpyHostToDevice, s));
    if (od.to_host() && E) GBX_CUDA(cudaMemcpyAsync(od.d, dst, (size_t)E * 4, cudaMemcpyHostToDevice, s));
    if (ol.to_host()) GBX_CUDA(cudaMemcpyAsync(ol.d, labels, (size_t)V * 4, cudaMemcpyHostToDevice, s));
    uint32_t id_max = 0, id_masked = 0;
    GBX_TRY(max_edge_id(os.d, od.d, E, s, &id_max, &id_masked));
    GBX_REQUIRE(E == 0 || id_max < V, GBX_ERR_INVALID, "vertex id %u >= num_vertices %u", id_max, V);
    DevBuf<uint32_t> deg, ids, newlab, mx;
    GBX_TRY(deg.alloc(V, s));
    GBX_TRY(ids.alloc(V, s));
    GBX_TRY(newlab.alloc(V, s));
    GBX_TRY(mx.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(deg.p, 0, (size_t)V * 4, s));
    // reorderGraphGenerateInOutDegrees (reorder.c:1483-1552): in-degrees for
    // 2, 5, 7, 9, in + out for 3, out-degrees for every other mode
    const bool in_deg = lmode == 2 || lmode == 5 || lmode == 7 || lmode == 9;
    const int count_mode = in_deg ? 2 : (lmode == 3 ? 3 : 1);
    if (E) {
        degree_count_kernel<<<grid1d(E), 256, 0, s>>>(os.d, od.d, E, count_mode, deg.p);
        GBX_LAUNCH_CHECK();
    }
    GBX_CUDA(cudaMemsetAsync(mx.p, 0, 4, s));
    max_id_kernel<<<grid1d(V), 256, 0, s>>>(deg.p, deg.p, V, mx.p);
    GBX_LAUNCH_CHECK();
    uint32_t hmax = 0;
    GBX_CUDA(cudaMemcpyAsync(&hmax, mx.p, 4, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    // thresholds of the bucketed modes: t0 = avg <= 1 ? 1 : avg/2 (HUBCluster:
    // avg), doubling, last UINT32_MAX; avg = E/V in uint32 as the reference's
    // EdgeList.avg_degree
    BucketThresholds th{};
    th.n = (lmode == 4 || lmode == 5 || lmode == 12 || lmode == 13) ? 11u : (lmode >= 6 && lmode <= 9 ? 2u : 0u);
    if (th.n) {
        const uint32_t avg = E / V;
        th.t[0] = (lmode == 8 || lmode == 9) ? avg : (avg <= 1 ? 1u : avg / 2);
        for (uint32_t i = 1; i + 1 < th.n; ++i) th.t[i] = th.t[i - 1] * 2u;
        th.t[th.n - 1] = 0xFFFFFFFFu;
    }
    if (th.n == 0) {
        // reorderGraphListDegree (reorder.c:296-380): stable ascending sort of
        // (degree, id), label N-1-rank
        iota_kernel<<<grid1d(V), 256, 0, s>>>(ids.p, V);
        GBX_LAUNCH_CHECK();
        GBX_TRY(radix_sort_pairs(deg.p, ids.p, V, bits_for(hmax), s));
        new_labels_kernel<<<grid1d(V), 256, 0, s>>>(ids.p, V, newlab.p);
        GBX_LAUNCH_CHECK();
    } else if (lmode == 6 || lmode == 7) {
        // HUBSort (reorder.c:814-982): hot vertices (degree above t0) stably
        // sorted by degree and labelled in reverse, cold ones after, in id order
        DevBuf<uint32_t> flag, pos, hot_deg, tot;
        GBX_TRY(flag.alloc(V, s));
        GBX_TRY(pos.alloc(V, s));
        GBX_TRY(hot_deg.alloc(V, s));
        GBX_TRY(tot.alloc(1, s));
        hot_flag_kernel<<<grid1d(V), 256, 0, s>>>(deg.p, V, th.t[0], flag.p);
        GBX_LAUNCH_CHECK();
        GBX_TRY(exclusive_scan_u32(flag.p, pos.p, V, s, tot.p));
        hot_split_kernel<<<grid1d(V), 256, 0, s>>>(deg.p, flag.p, pos.p, V, tot.p, ids.p, hot_deg.p, newlab.p);
        GBX_LAUNCH_CHECK();
        uint32_t H = 0;
        GBX_CUDA(cudaMemcpyAsync(&H, tot.p, 4, cudaMemcpyDeviceToHost, s));
        GBX_CUDA(cudaStreamSynchronize(s));
        GBX_TRY(radix_sort_pairs(hot_deg.p, ids.p, H, bits_for(hmax), s));
        if (H) {
            new_labels_kernel<<<grid1d(H), 256, 0, s>>>(ids.p, H, newlab.p);
            GBX_LAUNCH_CHECK();
        }
    } else {
        // DBG / Corder (11 buckets) and HUBCluster (2): buckets from the
        // highest, ids ascending inside a bucket
        bucket_key_kernel<<<grid1d(V), 256, 0, s>>>(deg.p, V, th, deg.p);
        GBX_LAUNCH_CHECK();
        iota_kernel<<<grid1d(V), 256, 0, s>>>(ids.p, V);
        GBX_LAUNCH_CHECK();
        GBX_TRY(radix_sort_pairs(deg.p, ids.p, V, bits_for(th.n - 1), s));
        rank_labels_kernel<<<grid1d(V), 256, 0, s>>>(ids.p, V, newlab.p);
        GBX_LAUNCH_CHECK();
    }
    if (E) {
        relabel_edges_kernel<<<grid1d(E), 256, 0, s>>>(os.d, od.d, E, newlab.p);
        GBX_LAUNCH_CHECK();
    }
    compose_labels_kernel<<<grid1d(V), 256, 0, s>>>(ol.d, oi.d, V, newlab.p);
    GBX_LAUNCH_CHECK();
    GBX_TRY(os.finish(s));
    GBX_TRY(od.finish(s));
    GBX_TRY(ol.finish(s));
    GBX_TRY(oi.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}

extern "C" int gbx_relabel(uint32_t num_vertices, uint32_t num_edges, uint32_t *src, uint32_t *dst,
                           const uint32_t *new_labels, uint32_t *labels, uint32_t *inverse_labels, void *stream) {
    clear_error();
    GBX_REQUIRE(num_vertices > 0, GBX_ERR_INVALID, "num_vertices must be > 0");
    GBX_REQUIRE(num_edges == 0 || (src && dst), GBX_ERR_INVALID, "src/dst is NULL");
    GBX_REQUIRE(new_labels && labels && inverse_labels, GBX_ERR_INVALID, "labels is NULL");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = num_vertices, E = num_edges;
    InArray<uint32_t> nl;
    GBX_TRY(nl.bind(new_labels, V, s));
    DevBuf<uint32_t> seen;
    DevBuf<unsigned> bad;
    GBX_TRY(seen.alloc(V, s));
    GBX_TRY(bad.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(seen.p, 0, (size_t)V * 4, s));
    GBX_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
    permutation_check_kernel<<<grid1d(V), 256, 0, s>>>(nl.d, V, seen.p, bad.p);
    GBX_LAUNCH_CHECK();
    unsigned hbad = 0;
    GBX_CUDA(cudaMemcpyAsync(&hbad, bad.p, 4, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    GBX_REQUIRE(hbad == 0, GBX_ERR_INVALID, "new_labels is not a permutation of [0, %u): %u bad entries", V,
                hbad);
    OutArray<uint32_t> os, od, ol, oi;
    GBX_TRY(os.bind(src, E, s));
    GBX_TRY(od.bind(dst, E, s));
    GBX_TRY(ol.bind(labels, V, s));
    GBX_TRY(oi.bind(inverse_labels, V, s));
    if (os.to_host() && E) GBX_CUDA(cudaMemcpyAsync(os.d, src, (size_t)E * 4, cudaMemcpyHostToDevice, s));
    if (od.to_host() && E) GBX_CUDA(cudaMemcpyAsync(od.d, dst, (size_t)E * 4, cudaMemcpyHostToDevice, s));
    if (ol.to_host()) GBX_CUDA(cudaMemcpyAsync(ol.d, labels, (size_t)V * 4, cudaMemcpyHostToDevice, s));
    uint32_t id_max = 0, id_masked = 0;
    GBX_TRY(max_edge_id(os.d, od.d, E, s, &id_max, &id_masked));
    GBX_REQUIRE(E == 0 || id_max < V, GBX_ERR_INVALID, "vertex id %u >= num_vertices %u", id_max, V);
    if (E) {
        relabel_edges_kernel<<<grid1d(E), 256, 0, s>>>(os.d, od.d, E, nl.d);
        GBX_LAUNCH_CHECK();
    }
    compose_labels_kernel<<<grid1d(V), 256, 0, s>>>(ol.d, oi.d, V, nl.d);
    GBX_LAUNCH_CHECK();
    GBX_TRY(os.finish(s));
    GBX_TRY(od.finish(s));
    GBX_TRY(ol.finish(s));
    GBX_TRY(oi.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}

extern "C" int gbx_mask_graph(uint32_t num_vertices, uint32_t num_edges, uint32_t *src, uint32_t *dst,
                              int mmode, uint32_t cache_size, uint32_t *mask_array, void *stream) {
    clear_error();
    GBX_REQUIRE(num_vertices > 0, GBX_ERR_INVALID, "num_vertices must be > 0");
    GBX_REQUIRE(num_edges == 0 || (src && dst), GBX_ERR_INVALID, "src/dst is NULL");
    GBX_REQUIRE(mask_array, GBX_ERR_INVALID, "mask_array is NULL");
    GBX_REQUIRE(mmode >= 1 && mmode <= 6, GBX_ERR_INVALID, "mmode must be 1-6");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = num_vertices, E = num_edges;
    OutArray<uint32_t> os, od, om;
    GBX_TRY(os.bind(src, E, s));
    GBX_TRY(od.bind(dst, E, s));
    GBX_TRY(om.bind(mask_array, V, s));
    if (os.to_host() && E) GBX_CUDA(cudaMemcpyAsync(os.d, src, (size_t)E * 4, cudaMemcpyHostToDevice, s));
    if (od.to_host() && E) GBX_CUDA(cudaMemcpyAsync(od.d, dst, (size_t)E * 4, cudaMemcpyHostToDevice, s));
    uint32_t id_max = 0, id_masked = 0;
    GBX_TRY(max_edge_id(os.d, od.d, E, s, &id_max, &id_masked));
    GBX_REQUIRE(E == 0 || id_max < V, GBX_ERR_INVALID,
                "vertex id %u >= num_vertices %u (ids must not carry mask bits yet)", id_max, V);
    DevBuf<uint32_t> key, ids;
    GBX_TRY(key.alloc(V, s));
    GBX_TRY(ids.alloc(V, s));
    GBX_CUDA(cudaMemsetAsync(key.p, 0, (size_t)V * 4, s));
    // maskGraphProcessGenerateInOutDegrees (reorder.c:1260-1306): in-degrees
    // for 2, 4, in + out for 5, 6, out-degrees otherwise
    const int count_mode = (mmode == 2 || mmode == 4) ? 2 : (mmode == 5 || mmode == 6) ? 3 : 1;
    if (E) {
        degree_count_kernel<<<grid1d(E), 256, 0, s>>>(os.d, od.d, E, count_mode, key.p);
        GBX_LAUNCH_CHECK();
    }
    // DBG's 11 buckets (reorder.c:1214-1228), highest first, ids ascending
    BucketThresholds th{};
    th.n = 11;
    const uint32_t avg = E / V;
    th.t[0] = avg <= 1 ? 1u : avg / 2;
    for (uint32_t i = 1; i + 1 < th.n; ++i) th.t[i] = th.t[i - 1] * 2u;
    th.t[th.n - 1] = 0xFFFFFFFFu;
    bucket_key_kernel<<<grid1d(V), 256, 0, s>>>(key.p, V, th, key.p);
    GBX_LAUNCH_CHECK();
    iota_kernel<<<grid1d(V), 256, 0, s>>>(ids.p, V);
    GBX_LAUNCH_CHECK();
    GBX_TRY(radix_sort_pairs(key.p, ids.p, V, bits_for(th.n - 1), s));
    // region sizes (reorder.c:1329-1345) with cs = cache_size / 4: V/4 each
    // when V - cs < 2 cs, else cs*8, *4, *4 in uint32 as the reference
    const uint32_t cs = cache_size >> 2;
    uint32_t r0, r1, r2;
    if ((int64_t)V - (int64_t)cs < 2 * (int64_t)cs) {
        r0 = r1 = r2 = V / 4;
    } else {
        r0 = cs * 8u;
        r1 = r0 * 4u;
        r2 = r1 * 4u;
    }
    const uint64_t e0 = r0, e1 = e0 + r1, e2 = e1 + r2;
    mask_hints_kernel<<<grid1d(V), 256, 0, s>>>(ids.p, V, e0, e1, e2, om.d);
    GBX_LAUNCH_CHECK();
    GBX_TRY(om.finish(s));
    if ((mmode == 1 || mmode == 2) && E) {
        mask_edges_kernel<<<grid1d(E), 256, 0, s>>>(os.d, od.d, E, om.d);
        GBX_LAUNCH_CHECK();
        GBX_TRY(os.finish(s));
        GBX_TRY(od.finish(s));
    }
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}
