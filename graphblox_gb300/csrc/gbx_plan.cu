// Degree classes for the pull engine (gbx_gather.cuh), built once per graph
// and direction with an ordered compaction (flags -> exclusive scan ->
// scatter), so the row lists are in ascending vertex order.
#include <algorithm>
#include <vector>

#include "gbx_gather.cuh"

namespace gbx {


__global__ void classify_rows_kernel(const uint32_t *off, uint32_t V, uint32_t heavy_min,
                                     uint32_t *is_med, uint32_t *is_heavy) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        uint32_t d = off[v + 1] - off[v];
        is_med[v] = (d > kLightMax && d <= heavy_min) ? 1u : 0u;
        is_heavy[v] = d > heavy_min ? 1u : 0u;
    }
}

__global__ void scatter_rows_kernel(const uint32_t *flag, const uint32_t *pos, uint32_t V,
                                    uint32_t *out) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        if (flag[v]) out[pos[v]] = v;
}

// out[2i], out[2i+1] = off[rows[i]], off[rows[i]+1]
__global__ void row_bounds_kernel(const uint32_t *off, const uint32_t *rows, uint32_t n, uint32_t *out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out[2 * i] = off[rows[i]];
        out[2 * i + 1] = off[rows[i] + 1];
    }
}

// rows above heavy_min edges get whole CTAs (chunks of kHeavyChunk)
static int build_plan(const uint32_t *off, uint32_t V, uint32_t heavy_min, cudaStream_t s, gbx_gather_plan **out) {
    gbx_gather_plan *p = new gbx_gather_plan();
    p->V = V;
    p->heavy_min = heavy_min;
    DevBuf<uint32_t> fm, fh, pm, ph, tot;
    int st = GBX_OK;
    do {
        if ((st = fm.alloc(V, s)) || (st = fh.alloc(V, s)) || (st = pm.alloc(V, s)) ||
            (st = ph.alloc(V, s)) || (st = tot.alloc(2, s)))
            break;
        int grid = (int)std::min<uint64_t>((V + 255) / 256, (uint64_t)num_sms() * 8);
        classify_rows_kernel<<<grid, 256, 0, s>>>(off, V, p->heavy_min, fm.p, fh.p);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) { st = GBX_ERR_CUDA; break; }
        if ((st = exclusive_scan_u32(fm.p, pm.p, V, s, tot.p))) break;
        if ((st = exclusive_scan_u32(fh.p, ph.p, V, s, tot.p + 1))) break;
        uint32_t h[2];
        if (cudaMemcpyAsync(h, tot.p, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            st = GBX_ERR_CUDA;
            break;
        }
        p->n_medium = h[0];
        p->n_heavy = h[1];
        if (cudaMalloc(&p->medium_rows, (size_t)(h[0] ? h[0] : 1) * 4) != cudaSuccess ||
            cudaMalloc(&p->heavy_rows, (size_t)(h[1] ? h[1] : 1) * 4) != cudaSuccess) {
            st = GBX_ERR_NOMEM;
            break;
        }
        scatter_rows_kernel<<<grid, 256, 0, s>>>(fm.p, pm.p, V, p->medium_rows);
        scatter_rows_kernel<<<grid, 256, 0, s>>>(fh.p, ph.p, V, p->heavy_rows);
        note_launch();
        note_launch();
        if (cudaGetLastError() != cudaSuccess) { st = GBX_ERR_CUDA; break; }
        // heavy rows -> chunks of kHeavyChunk edges (host side: the list is short)
        const uint32_t nh = p->n_heavy;
        std::vector<uint32_t> hoff(2 * (size_t)nh), first(nh + 1);
        if (nh) {
            DevBuf<uint32_t> hb;
            if ((st = hb.alloc(2 * (size_t)nh, s))) break;
            row_bounds_kernel<<<(nh + 255) / 256, 256, 0, s>>>(off, p->heavy_rows, nh, hb.p);
            note_launch();
            if (cudaGetLastError() != cudaSuccess ||
                cudaMemcpyAsync(hoff.data(), hb.p, 8 * (size_t)nh, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess) {
                st = GBX_ERR_CUDA;
                break;
            }
        }
        first[0] = 0;
        for (uint32_t i = 0; i < nh; ++i) {
            uint32_t d = hoff[2 * i + 1] - hoff[2 * i];
            first[i + 1] = first[i] + (d + kHeavyChunk - 1) / kHeavyChunk;
        }
        p->n_chunks = first[nh];
        std::vector<uint32_t> chunk_heavy(p->n_chunks ? p->n_chunks : 1);
        for (uint32_t i = 0; i < nh; ++i)
            for (uint32_t c = first[i]; c < first[i + 1]; ++c) chunk_heavy[c] = i;
        size_t nc = p->n_chunks ? p->n_chunks : 1;
        if (cudaMalloc(&p->heavy_first, (size_t)(nh + 1) * 4) != cudaSuccess ||
            cudaMalloc(&p->chunk_heavy, nc * 4) != cudaSuccess ||
            cudaMalloc(&p->partials, nc * 4) != cudaSuccess ||
            cudaMalloc(&p->tickets, (size_t)(nh ? nh : 1) * 4) != cudaSuccess) {
            st = GBX_ERR_NOMEM;
            break;
        }
        if (cudaMemcpyAsync(p->heavy_first, first.data(), (size_t)(nh + 1) * 4, cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            cudaMemcpyAsync(p->chunk_heavy, chunk_heavy.data(), nc * 4, cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            cudaMemsetAsync(p->tickets, 0, (size_t)(nh ? nh : 1) * 4, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            st = GBX_ERR_CUDA;
            break;
        }
    } while (0);
    if (st != GBX_OK) {
        (void)cudaGetLastError();
        if (!gbx_last_error()[0]) set_error("building the pull plan failed");
        free_plan(p);
        return st;
    }
    *out = p;
    return GBX_OK;
}

int get_pull_plan(gbx_graph *g, cudaStream_t s, gbx_gather_plan **plan) {
    gbx_gather_plan **slot = g->has_inverse() ? &g->plan_inv : &g->plan_fwd;
    if (!*slot) GBX_TRY(build_plan(g->pull_offsets(), g->V, g->pull_heavy_min, s, slot));
    *plan = *slot;
    return GBX_OK;
}

void free_plan(gbx_gather_plan *p) {
    if (!p) return;
    cudaFree(p->medium_rows);
    cudaFree(p->heavy_rows);
    cudaFree(p->heavy_first);
    cudaFree(p->chunk_heavy);
    cudaFree(p->partials);
    cudaFree(p->tickets);
    delete p;
}

}  // namespace gbx
