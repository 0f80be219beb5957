// Personalised PageRank over K teleport vectors and its hand-written adjoint.
// No reference counterpart: the reference has no personalised or
// differentiable PageRank. The recurrence is the reference's pull PageRank
// (01_host/src/algorithms/openmp/pageRank.c:245-368) with a teleport block
// and a column-stochastic P built from edge weights:
//
//   P[v,u] = w_e / s_u  for edge e = (u -> v), s_u = sum of u's out-weights
//   forward : R = (1-d) T + d P R          (fixed point, FP32 block [V][K])
//   loss    : L = sum_{v,k} W[v,k] R[v,k]  (FP64 dot)
//   adjoint : Lam = W + d P^T Lam          (fixed point, the same sweep kernel
//                                           pulling over out-edges)
//   dL/dT[v,k] = (1-d) Lam[v,k]
//   g_e = dL/dP_e = d * <Lam[v,:], R[u,:]>
//   dL/dw_e = (g_e - sum_{e' out of u} g_e' P_e') / s_u
//
// Only the converged R enters the adjoint, so no forward iterate is stored.
// A source with no out-weight (s_u = 0) has a zero column: its mass is
// dropped, as the reference drops dangling mass (pageRank.c:298-301).
//
// Layout: R, Lam, T, W are [V][K] row-major, K = 32*KPL (32..256), so one
// gathered neighbour row is K*4 contiguous bytes read by one warp with a
// KPL-float vector load per lane. Rows are dealt as chunks of at most
// kPprChunk edges, one warp per chunk (a per-direction chunk table); a row
// cut into several chunks writes K-wide partial sums that a second kernel
// adds in chunk order, so every result is deterministic. The iteration loop
// runs without host round trips: a one-block check kernel turns the
// per-column L1 residual (reduced in FP64) into a device flag that the
// following sweeps test before doing any work, and the host reads the flag
// every kPprPoll iterations.
//
// Stopping rule: max over columns of ||X_new - X_old||_1 / ||S||_1 < tol,
// with S the column's source term (T forward, W adjoint; a zero column counts
// as norm 1). For teleport columns that sum to 1 this is the plain L1
// residual; for the adjoint it makes the sweep count independent of the
// scale of W (Lam scales with W).
#include <algorithm>
#include <cmath>
#include <vector>

#include "gbx_internal.cuh"

namespace gbx {

constexpr uint32_t kPprChunk = 256;
constexpr int kPprThreads = 256;
constexpr int kPprWarps = kPprThreads / 32;
constexpr uint32_t kNoSlot = 0xFFFFFFFFu;
constexpr uint32_t kPprPoll = 8;

struct PprChunk {
    uint32_t row, eb, ee, slot;  // slot: partial-sum slot, kNoSlot when the chunk is the whole row
};

// Chunk table of one CSR direction: whole rows up to kPprChunk edges, longer
// rows cut into kPprChunk pieces with one partial slot each.
struct PprPlan {
    PprChunk *chunks = nullptr;       // device
    uint32_t *split_rows = nullptr;   // device: rows cut into several chunks
    uint32_t *split_first = nullptr;  // device [n_split+1]: first slot of each split row
    uint32_t n_chunks = 0, n_split = 0, n_slots = 0;
    void release() {
        cudaFree(chunks);
        cudaFree(split_rows);
        cudaFree(split_first);
        chunks = nullptr;
        split_rows = split_first = nullptr;
    }
};

// convergence state of one fixed-point solve
struct PprCtl {
    uint32_t done;
    uint32_t iterations;
    double residual;
};

static int build_ppr_plan(const uint32_t *d_off, uint32_t V, cudaStream_t s, PprPlan *p) {
    std::vector<uint32_t> off(V + 1);
    GBX_CUDA(cudaMemcpyAsync(off.data(), d_off, (size_t)(V + 1) * 4, cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    std::vector<PprChunk> ch;
    std::vector<uint32_t> srows, sfirst;
    ch.reserve(V + off[V] / kPprChunk + 1);
    uint32_t slot = 0;
    for (uint32_t v = 0; v < V; ++v) {
        const uint32_t b = off[v], e = off[v + 1];
        if (e - b <= kPprChunk) {
            ch.push_back({v, b, e, kNoSlot});
        } else {
            srows.push_back(v);
            sfirst.push_back(slot);
            for (uint32_t c = b; c < e; c += kPprChunk) ch.push_back({v, c, std::min(c + kPprChunk, e), slot++});
        }
    }
    sfirst.push_back(slot);
    p->n_chunks = (uint32_t)ch.size();
    p->n_split = (uint32_t)srows.size();
    p->n_slots = slot;
    GBX_CUDA(cudaMalloc(&p->chunks, sizeof(PprChunk) * std::max<size_t>(1, ch.size())));
    GBX_CUDA(cudaMalloc(&p->split_rows, 4 * std::max<size_t>(1, srows.size())));
    GBX_CUDA(cudaMalloc(&p->split_first, 4 * sfirst.size()));
    if (!ch.empty())
        GBX_CUDA(cudaMemcpyAsync(p->chunks, ch.data(), sizeof(PprChunk) * ch.size(), cudaMemcpyHostToDevice, s));
    if (!srows.empty())
        GBX_CUDA(cudaMemcpyAsync(p->split_rows, srows.data(), 4 * srows.size(), cudaMemcpyHostToDevice, s));
    GBX_CUDA(cudaMemcpyAsync(p->split_first, sfirst.data(), 4 * sfirst.size(), cudaMemcpyHostToDevice, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}

template <int KPL>
struct Vec {
    float v[KPL];
};

template <int KPL>
__device__ __forceinline__ Vec<KPL> load_row(const float *__restrict__ X, uint32_t row, uint32_t lane) {
    Vec<KPL> r;
    const float *p = X + (size_t)row * (32 * KPL) + lane * KPL;
    if constexpr (KPL % 4 == 0) {
#pragma unroll
        for (int i = 0; i < KPL; i += 4) {
            const float4 t = __ldg(reinterpret_cast<const float4 *>(p + i));
            r.v[i] = t.x;
            r.v[i + 1] = t.y;
            r.v[i + 2] = t.z;
            r.v[i + 3] = t.w;
        }
    } else if constexpr (KPL == 2) {
        const float2 t = __ldg(reinterpret_cast<const float2 *>(p));
        r.v[0] = t.x;
        r.v[1] = t.y;
    } else {
        r.v[0] = __ldg(p);
    }
    return r;
}

template <int KPL>
__device__ __forceinline__ void store_row(float *__restrict__ X, uint32_t row, uint32_t lane, const float (&a)[KPL]) {
    float *p = X + (size_t)row * (32 * KPL) + lane * KPL;
    if constexpr (KPL % 4 == 0) {
#pragma unroll
        for (int i = 0; i < KPL; i += 4)
            *reinterpret_cast<float4 *>(p + i) = make_float4(a[i], a[i + 1], a[i + 2], a[i + 3]);
    } else if constexpr (KPL == 2) {
        *reinterpret_cast<float2 *>(p) = make_float2(a[0], a[1]);
    } else {
        p[0] = a[0];
    }
}

// Epilogue of one row: Xn = bscale*B + d*acc; per-column |Xn - X| into res.
template <int KPL>
__device__ __forceinline__ void ppr_finish_row(uint32_t row, uint32_t lane, const float (&acc)[KPL],
                                               const float *__restrict__ X, float *__restrict__ Xn,
                                               const float *__restrict__ B, float bscale, float d,
                                               float (&res)[KPL]) {
    const Vec<KPL> b = load_row<KPL>(B, row, lane);
    const Vec<KPL> old = load_row<KPL>(X, row, lane);
    float out[KPL];
#pragma unroll
    for (int i = 0; i < KPL; ++i) {
        out[i] = __fadd_rn(__fmul_rn(bscale, b.v[i]), __fmul_rn(d, acc[i]));
        res[i] += fabsf(out[i] - old.v[i]);
    }
    store_row<KPL>(Xn, row, lane, out);
}

// Per-column residual of a block: each lane's FP32 partial (the rows its warp
// finished) is widened to FP64 and summed across the block, then added to the
// device-wide FP64 column sums.
template <int KPL>
__device__ __forceinline__ void flush_residual(const float (&res)[KPL], double *res_out) {
    __shared__ double sres[kPprWarps][32 * KPL];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < KPL; ++i) sres[wid][lane * KPL + i] = (double)res[i];
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < 32 * KPL; c += blockDim.x) {
        double t = 0.0;
        for (int w = 0; w < kPprWarps; ++w) t += sres[w][c];
        if (t != 0.0) atomicAdd(res_out + c, t);
    }
}

__device__ __forceinline__ bool ppr_done(const PprCtl *ctl) {
    return *reinterpret_cast<const volatile uint32_t *>(&ctl->done) != 0;
}

// One sweep: each chunk's P-weighted sum of neighbour rows; whole-row chunks
// finish their row, chunks of split rows leave partials.
template <int KPL>
__global__ void __launch_bounds__(kPprThreads)
    ppr_sweep_kernel(const PprChunk *__restrict__ chunks, uint32_t n_chunks, const uint32_t *__restrict__ col,
                     const float *__restrict__ P, const float *__restrict__ X, float *__restrict__ Xn,
                     const float *__restrict__ B, float bscale, float d, float *__restrict__ partials,
                     double *res_out, const PprCtl *ctl) {
    if (ppr_done(ctl)) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    float res[KPL];
#pragma unroll
    for (int i = 0; i < KPL; ++i) res[i] = 0.f;
    for (uint32_t c = gw; c < n_chunks; c += nw) {
        const PprChunk ck = chunks[c];
        float acc[KPL];
#pragma unroll
        for (int i = 0; i < KPL; ++i) acc[i] = 0.f;
        uint32_t e = ck.eb;
        for (; e + 4 <= ck.ee; e += 4) {
            uint32_t u[4];
            float p[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                u[q] = __ldg(col + e + q);
                p[q] = __ldg(P + e + q);
            }
            Vec<KPL> x[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) x[q] = load_row<KPL>(X, u[q], lane);
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int i = 0; i < KPL; ++i) acc[i] = __fmaf_rn(p[q], x[q].v[i], acc[i]);
        }
        for (; e < ck.ee; ++e) {
            const uint32_t u = __ldg(col + e);
            const float p = __ldg(P + e);
            const Vec<KPL> x = load_row<KPL>(X, u, lane);
#pragma unroll
            for (int i = 0; i < KPL; ++i) acc[i] = __fmaf_rn(p, x.v[i], acc[i]);
        }
        if (ck.slot == kNoSlot)
            ppr_finish_row<KPL>(ck.row, lane, acc, X, Xn, B, bscale, d, res);
        else
            store_row<KPL>(partials, ck.slot, lane, acc);
    }
    flush_residual<KPL>(res, res_out);
}

// Split rows: add the partials in chunk order, then the row epilogue.
template <int KPL>
__global__ void __launch_bounds__(kPprThreads)
    ppr_combine_kernel(const uint32_t *__restrict__ split_rows, const uint32_t *__restrict__ split_first,
                       uint32_t n_split, const float *__restrict__ partials, const float *__restrict__ X,
                       float *__restrict__ Xn, const float *__restrict__ B, float bscale, float d, double *res_out,
                       const PprCtl *ctl) {
    if (ppr_done(ctl)) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    float res[KPL];
#pragma unroll
    for (int i = 0; i < KPL; ++i) res[i] = 0.f;
    for (uint32_t h = gw; h < n_split; h += nw) {
        float acc[KPL];
#pragma unroll
        for (int i = 0; i < KPL; ++i) acc[i] = 0.f;
        for (uint32_t s = split_first[h]; s < split_first[h + 1]; ++s) {
            const Vec<KPL> p = load_row<KPL>(partials, s, lane);
#pragma unroll
            for (int i = 0; i < KPL; ++i) acc[i] = __fadd_rn(acc[i], p.v[i]);
        }
        ppr_finish_row<KPL>(split_rows[h], lane, acc, X, Xn, B, bscale, d, res);
    }
    flush_residual<KPL>(res, res_out);
}

// After a sweep: the max over columns of the relative L1 residual decides
// convergence; also clears the residual buffer the next sweep accumulates into.
__global__ void ppr_check_kernel(const double *res_cur, double *res_next, const double *norms, uint32_t K,
                                 double tol, PprCtl *ctl) {
    __shared__ double sh[32];
    double m = 0.0;
    for (uint32_t c = threadIdx.x; c < K; c += blockDim.x) {
        const double n = norms[c];
        m = fmax(m, res_cur[c] / (n > 0.0 ? n : 1.0));
        res_next[c] = 0.0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0 && !ctl->done) {
        for (uint32_t w = 1; w < blockDim.x / 32; ++w) m = fmax(m, sh[w]);
        ctl->iterations += 1;
        ctl->residual = m;
        if (m < tol) ctl->done = 1;
    }
}

// Per-column L1 norms of a [V][K] block (FP32 partials per thread, FP64 sums).
__global__ void ppr_col_norm_kernel(const float *__restrict__ B, uint32_t V, uint32_t K, double *norms) {
    // thread t of the grid owns column t % K and rows t / K, t / K + stride, ...
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t c = tid % K, r0 = tid / K, rs = (gridDim.x * blockDim.x) / K;
    if (r0 >= rs) return;  // grid is a multiple of K; spare threads do nothing
    float s = 0.f;
    for (uint32_t r = r0; r < V; r += rs) s += fabsf(B[(size_t)r * K + c]);
    if (s != 0.f) atomicAdd(norms + c, (double)s);
}

// Per-source out-weight sums and the normalised forward weights P_e = w_e/s_u.
__global__ void ppr_normalise_kernel(const uint32_t *__restrict__ off, const float *__restrict__ w, uint32_t V,
                                     float *__restrict__ s_out, float *__restrict__ P) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t u = gw; u < V; u += nw) {
        const uint32_t b = off[u], e = off[u + 1];
        float s = 0.f;
        for (uint32_t j = b + lane; j < e; j += 32) s += w[j];
        s = warp_sum(s);
        if (lane == 0) s_out[u] = s;
        for (uint32_t j = b + lane; j < e; j += 32) P[j] = s > 0.f ? __fdiv_rn(w[j], s) : 0.f;
    }
}

// row_of[e] = source of forward edge e
__global__ void ppr_row_of_kernel(const uint32_t *__restrict__ off, uint32_t V, uint32_t *__restrict__ row_of) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t u = gw; u < V; u += nw)
        for (uint32_t j = off[u] + lane; j < off[u + 1]; j += 32) row_of[j] = u;
}

// sort input (key = destination, value = forward position) and in-degrees
__global__ void ppr_sort_input_kernel(const uint32_t *__restrict__ dest, uint32_t E, uint32_t *__restrict__ keys,
                                      uint32_t *__restrict__ vals, uint32_t *__restrict__ counts) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const uint32_t v = dest[i];
        keys[i] = v;
        vals[i] = i;
        atomicAdd(counts + v, 1u);
    }
}

__global__ void ppr_gather_u32_kernel(const uint32_t *__restrict__ in, const uint32_t *__restrict__ map, uint32_t n,
                                      uint32_t *__restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = in[map[i]];
}

__global__ void ppr_gather_f32_kernel(const float *__restrict__ in, const uint32_t *__restrict__ map, uint32_t n,
                                      float *__restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = in[map[i]];
}

__global__ void ppr_scale_kernel(const float *__restrict__ in, float a, size_t n, float *__restrict__ out) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __fmul_rn(a, in[i]);
}

// loss = sum W*R, FP64
__global__ void ppr_loss_kernel(const float *__restrict__ W, const float *__restrict__ R, size_t n, double *loss) {
    __shared__ double sh[32];
    double s = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        s += (double)W[i] * (double)R[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) atomicAdd(loss, s);
}

// Edge gradient, first pass, one warp per forward chunk of source u:
// g_e = d * <Lam[v,:], R[u,:]> for each edge, and the chunk's Kahan sum of
// g_e * P_e (to the row directly, or to its partial slot).
template <int KPL>
__global__ void __launch_bounds__(kPprThreads)
    ppr_edge_dot_kernel(const PprChunk *__restrict__ chunks, uint32_t n_chunks, const uint32_t *__restrict__ dest,
                        const float *__restrict__ P, const float *__restrict__ R, const float *__restrict__ Lam,
                        float d, float *__restrict__ g, float *__restrict__ wsum_row,
                        float *__restrict__ wsum_part) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t c = gw; c < n_chunks; c += nw) {
        const PprChunk ck = chunks[c];
        const Vec<KPL> r = load_row<KPL>(R, ck.row, lane);
        float sum = 0.f, comp = 0.f;
        for (uint32_t e0 = ck.eb; e0 < ck.ee; e0 += 4) {
            const uint32_t n = min(4u, ck.ee - e0);
            Vec<KPL> l[4];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (q < (int)n) l[q] = load_row<KPL>(Lam, __ldg(dest + e0 + q), lane);
            float t[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float a = 0.f;
                if (q < (int)n) {
#pragma unroll
                    for (int i = 0; i < KPL; ++i) a = __fmaf_rn(l[q].v[i], r.v[i], a);
                }
                t[q] = warp_sum(a);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (q < (int)n) {
                    const float ge = __fmul_rn(d, t[q]);
                    if (lane == (uint32_t)q) g[e0 + q] = ge;
                    // Kahan step, identical on every lane
                    const float y = __fsub_rn(__fmul_rn(ge, __ldg(P + e0 + q)), comp);
                    const float s2 = __fadd_rn(sum, y);
                    comp = __fsub_rn(__fsub_rn(s2, sum), y);
                    sum = s2;
                }
            }
        }
        if (lane == 0) {
            if (ck.slot == kNoSlot)
                wsum_row[ck.row] = sum;
            else
                wsum_part[ck.slot] = sum;
        }
    }
}

// split rows: chunk partials of sum g_e P_e added in chunk order
__global__ void ppr_wsum_combine_kernel(const uint32_t *__restrict__ split_rows,
                                        const uint32_t *__restrict__ split_first, uint32_t n_split,
                                        const float *__restrict__ wsum_part, float *__restrict__ wsum_row) {
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < n_split; h += gridDim.x * blockDim.x) {
        float sum = 0.f, comp = 0.f;
        for (uint32_t s = split_first[h]; s < split_first[h + 1]; ++s) {
            const float y = __fsub_rn(wsum_part[s], comp);
            const float s2 = __fadd_rn(sum, y);
            comp = __fsub_rn(__fsub_rn(s2, sum), y);
            sum = s2;
        }
        wsum_row[split_rows[h]] = sum;
    }
}

// dL/dw_e = (g_e - sum_{e' out of u} g_e' P_e') / s_u
__global__ void ppr_grad_w_kernel(const uint32_t *__restrict__ row_of, const float *__restrict__ g,
                                  const float *__restrict__ wsum_row, const float *__restrict__ ssum, uint32_t E,
                                  float *__restrict__ grad_w) {
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        const uint32_t u = row_of[e];
        const float s = ssum[u];
        grad_w[e] = s > 0.f ? __fdiv_rn(__fsub_rn(g[e], wsum_row[u]), s) : 0.f;
    }
}

}  // namespace gbx

// Per-graph PPR state: the in-edge order of the forward edges (a stable sort
// by destination), the in-edge CSR it implies, and the chunk tables of both
// directions. Built from the forward CSR alone, so undirected graphs, graphs
// without an inverse CSR and rows with repeated neighbours all work.
struct gbx_ppr_cache {
    gbx::PprPlan fwd, inv;
    uint32_t *row_of = nullptr;   // E: source of each forward edge
    uint32_t *perm = nullptr;     // E: forward edge at each in-edge position
    uint32_t *inv_off = nullptr;  // V+1
    uint32_t *inv_src = nullptr;  // E
};

using namespace gbx;

void gbx_free_ppr_cache(gbx_ppr_cache *c) {
    if (!c) return;
    c->fwd.release();
    c->inv.release();
    cudaFree(c->row_of);
    cudaFree(c->perm);
    cudaFree(c->inv_off);
    cudaFree(c->inv_src);
    delete c;
}

namespace {

int bits_for_ids(uint32_t V) {
    int b = 1;
    while (b < 32 && ((uint64_t)(V - 1) >> b)) ++b;
    return b;
}

int build_ppr_cache(gbx_graph *g, cudaStream_t s, gbx_ppr_cache *c) {
    const uint32_t V = g->V, E = g->E;
    const size_t e1 = std::max<uint32_t>(E, 1);
    GBX_CUDA(cudaMalloc(&c->row_of, e1 * 4));
    GBX_CUDA(cudaMalloc(&c->perm, e1 * 4));
    GBX_CUDA(cudaMalloc(&c->inv_src, e1 * 4));
    GBX_CUDA(cudaMalloc(&c->inv_off, ((size_t)V + 1) * 4));
    const unsigned wg = std::max(1u, std::min<unsigned>(ceil_div((uint64_t)V * 32, 256), (unsigned)num_sms() * 8));
    const unsigned eg = (unsigned)num_sms() * 8;
    ppr_row_of_kernel<<<wg, 256, 0, s>>>(g->offsets, V, c->row_of);
    GBX_LAUNCH_CHECK();
    DevBuf<uint32_t> keys, counts;
    GBX_TRY(keys.alloc(e1, s));
    GBX_TRY(counts.alloc(V, s));
    GBX_CUDA(cudaMemsetAsync(counts.p, 0, (size_t)V * 4, s));
    if (E) {
        ppr_sort_input_kernel<<<eg, 256, 0, s>>>(g->dest, E, keys.p, c->perm, counts.p);
        GBX_LAUNCH_CHECK();
        GBX_TRY(radix_sort_pairs(keys.p, c->perm, E, bits_for_ids(V), s));
        ppr_gather_u32_kernel<<<eg, 256, 0, s>>>(c->row_of, c->perm, E, c->inv_src);
        GBX_LAUNCH_CHECK();
    }
    GBX_TRY(exclusive_scan_u32(counts.p, c->inv_off, V, s, c->inv_off + V));
    GBX_TRY(build_ppr_plan(g->offsets, V, s, &c->fwd));
    GBX_TRY(build_ppr_plan(c->inv_off, V, s, &c->inv));
    return GBX_OK;
}

int ppr_cache(gbx_graph *g, cudaStream_t s, gbx_ppr_cache **out) {
    if (!g->ppr) {
        gbx_ppr_cache *c = new gbx_ppr_cache();
        const int st = build_ppr_cache(g, s, c);
        if (st != GBX_OK) {
            cudaStreamSynchronize(s);
            gbx_free_ppr_cache(c);
            return st;
        }
        g->ppr = c;
    }
    *out = g->ppr;
    return GBX_OK;
}

// Fixed point X = bscale*B + d*A X with A given by (plan, col, P), from
// X0 = bscale*B. On return *result points at the last iterate (X0 or X1).
template <int KPL>
int ppr_solve(const PprPlan &plan, const uint32_t *col, const float *P, const float *B, float bscale, float d,
              double tol, uint32_t max_it, float *X0, float *X1, float *partials, uint32_t V, cudaStream_t s,
              float **result, uint32_t *iters, double *resid) {
    const uint32_t K = 32 * KPL;
    const unsigned grid = (unsigned)num_sms() * 8;
    DevBuf<double> resb;
    DevBuf<PprCtl> ctl;
    GBX_TRY(resb.alloc(3 * (size_t)K, s));
    GBX_TRY(ctl.alloc(1, s));
    GBX_CUDA(cudaMemsetAsync(resb.p, 0, sizeof(double) * 3 * K, s));
    GBX_CUDA(cudaMemsetAsync(ctl.p, 0, sizeof(PprCtl), s));
    double *norms = resb.p + 2 * K;
    // 1024 rows at a time per column: grid * 256 threads = 1024 * K
    ppr_col_norm_kernel<<<4 * K, 256, 0, s>>>(B, V, K, norms);
    GBX_LAUNCH_CHECK();
    ppr_scale_kernel<<<grid, 256, 0, s>>>(B, bscale, (size_t)V * K, X0);
    GBX_LAUNCH_CHECK();
    float *X[2] = {X0, X1};
    PprCtl h{};
    const unsigned cgrid = std::max(1u, std::min<unsigned>(grid, ceil_div((uint64_t)plan.n_split * 32, 256)));
    for (uint32_t it = 0; it < max_it; ++it) {
        double *rc = resb.p + (it & 1) * K, *rn = resb.p + ((it + 1) & 1) * K;
        ppr_sweep_kernel<KPL><<<grid, kPprThreads, 0, s>>>(plan.chunks, plan.n_chunks, col, P, X[it & 1],
                                                           X[(it + 1) & 1], B, bscale, d, partials, rc, ctl.p);
        GBX_LAUNCH_CHECK();
        if (plan.n_split) {
            ppr_combine_kernel<KPL><<<cgrid, kPprThreads, 0, s>>>(plan.split_rows, plan.split_first, plan.n_split,
                                                                  partials, X[it & 1], X[(it + 1) & 1], B, bscale,
                                                                  d, rc, ctl.p);
            GBX_LAUNCH_CHECK();
        }
        ppr_check_kernel<<<1, 256, 0, s>>>(rc, rn, norms, K, tol, ctl.p);
        GBX_LAUNCH_CHECK();
        if ((it + 1) % kPprPoll == 0 || it + 1 == max_it) {
            GBX_CUDA(cudaMemcpyAsync(&h, ctl.p, sizeof(PprCtl), cudaMemcpyDeviceToHost, s));
            GBX_CUDA(cudaStreamSynchronize(s));
            if (h.done) break;
        }
    }
    if (max_it == 0) GBX_CUDA(cudaStreamSynchronize(s));
    *result = X[h.iterations & 1];
    *iters = h.iterations;
    *resid = h.residual;
    return h.done ? GBX_OK : GBX_ERR_ITER_CAP;
}

template <int KPL>
int ppr_forward_impl(gbx_graph *g, const float *w, const float *T, float d, double tol, uint32_t max_it, float *ranks,
                     gbx_ppr_result *res, cudaStream_t s) {
    const uint32_t V = g->V, E = g->E, K = 32 * KPL;
    gbx_ppr_cache *c = nullptr;
    GBX_TRY(ppr_cache(g, s, &c));
    InArray<float> win, tin;
    GBX_TRY(win.bind(w, E, s));
    GBX_TRY(tin.bind(T, (size_t)V * K, s));
    DevBuf<float> ssum, Pf, Pi, X0, X1, part;
    const size_t e1 = std::max<uint32_t>(E, 1);
    GBX_TRY(ssum.alloc(V, s));
    GBX_TRY(Pf.alloc(e1, s));
    GBX_TRY(Pi.alloc(e1, s));
    GBX_TRY(X0.alloc((size_t)V * K, s));
    GBX_TRY(X1.alloc((size_t)V * K, s));
    GBX_TRY(part.alloc((size_t)std::max<uint32_t>(c->inv.n_slots, 1) * K, s));
    const unsigned wg = std::max(1u, std::min<unsigned>(ceil_div((uint64_t)V * 32, 256), (unsigned)num_sms() * 8));
    if (E) {
        ppr_normalise_kernel<<<wg, 256, 0, s>>>(g->offsets, win.d, V, ssum.p, Pf.p);
        GBX_LAUNCH_CHECK();
        ppr_gather_f32_kernel<<<num_sms() * 8, 256, 0, s>>>(Pf.p, c->perm, E, Pi.p);
        GBX_LAUNCH_CHECK();
    }
    float *out = nullptr;
    uint32_t iters = 0;
    double resid = 0.0;
    const int st = ppr_solve<KPL>(c->inv, c->inv_src, Pi.p, tin.d, 1.0f - d, d, tol, max_it, X0.p, X1.p, part.p, V,
                                  s, &out, &iters, &resid);
    if (st != GBX_OK && st != GBX_ERR_ITER_CAP) return st;
    OutArray<float> o;
    GBX_TRY(o.bind(ranks, (size_t)V * K, s));
    GBX_CUDA(cudaMemcpyAsync(o.d, out, sizeof(float) * (size_t)V * K, cudaMemcpyDeviceToDevice, s));
    GBX_TRY(o.finish(s));
    GBX_CUDA(cudaStreamSynchronize(s));
    if (res) {
        res->iterations = iters;
        res->residual = resid;
    }
    GBX_REQUIRE(st == GBX_OK, GBX_ERR_ITER_CAP, "PPR did not reach L1 residual %g in %u iterations (residual %g)", tol,
                max_it, resid);
    return GBX_OK;
}

template <int KPL>
int ppr_adjoint_impl(gbx_graph *g, const float *w, const float *R, const float *W, float d, double tol,
                     uint32_t max_it, float *grad_w, float *grad_t, gbx_ppr_result *res, cudaStream_t s) {
    const uint32_t V = g->V, E = g->E, K = 32 * KPL;
    gbx_ppr_cache *c = nullptr;
    GBX_TRY(ppr_cache(g, s, &c));
    InArray<float> win, rin, lw;
    GBX_TRY(win.bind(w, E, s));
    GBX_TRY(rin.bind(R, (size_t)V * K, s));
    GBX_TRY(lw.bind(W, (size_t)V * K, s));
    const size_t e1 = std::max<uint32_t>(E, 1);
    DevBuf<double> loss;
    DevBuf<float> ssum, Pf, X0, X1, part, gbuf, wrow, wpart;
    GBX_TRY(loss.alloc(1, s));
    GBX_TRY(ssum.alloc(V, s));
    GBX_TRY(Pf.alloc(e1, s));
    GBX_TRY(X0.alloc((size_t)V * K, s));
    GBX_TRY(X1.alloc((size_t)V * K, s));
    GBX_TRY(part.alloc((size_t)std::max<uint32_t>(c->fwd.n_slots, 1) * K, s));
    const unsigned wg = std::max(1u, std::min<unsigned>(ceil_div((uint64_t)V * 32, 256), (unsigned)num_sms() * 8));
    if (E) {
        ppr_normalise_kernel<<<wg, 256, 0, s>>>(g->offsets, win.d, V, ssum.p, Pf.p);
        GBX_LAUNCH_CHECK();
    }
    // Lam = W + d P^T Lam: the sweep over out-edges with forward-order weights
    float *lam = nullptr;
    uint32_t iters = 0;
    double resid = 0.0;
    const int st = ppr_solve<KPL>(c->fwd, g->dest, Pf.p, lw.d, 1.0f, d, tol, max_it, X0.p, X1.p, part.p, V, s, &lam,
                                  &iters, &resid);
    if (st != GBX_OK && st != GBX_ERR_ITER_CAP) return st;
    OutArray<float> gw_out, gt_out;
    GBX_TRY(gw_out.bind(grad_w, E, s));
    GBX_TRY(gt_out.bind(grad_t, (size_t)V * K, s));
    const unsigned eg = (unsigned)num_sms() * 8;
    if (gt_out.d) {
        ppr_scale_kernel<<<eg, 256, 0, s>>>(lam, 1.0f - d, (size_t)V * K, gt_out.d);
        GBX_LAUNCH_CHECK();
    }
    if (gw_out.d && E) {
        GBX_TRY(gbuf.alloc(e1, s));
        GBX_TRY(wrow.alloc(V, s));
        GBX_TRY(wpart.alloc(std::max<uint32_t>(c->fwd.n_slots, 1), s));
        GBX_CUDA(cudaMemsetAsync(wrow.p, 0, (size_t)V * 4, s));
        ppr_edge_dot_kernel<KPL><<<eg, kPprThreads, 0, s>>>(c->fwd.chunks, c->fwd.n_chunks, g->dest, Pf.p, rin.d, lam,
                                                            d, gbuf.p, wrow.p, wpart.p);
        GBX_LAUNCH_CHECK();
        if (c->fwd.n_split) {
            ppr_wsum_combine_kernel<<<ceil_div(c->fwd.n_split, 256), 256, 0, s>>>(
                c->fwd.split_rows, c->fwd.split_first, c->fwd.n_split, wpart.p, wrow.p);
            GBX_LAUNCH_CHECK();
        }
        ppr_grad_w_kernel<<<eg, 256, 0, s>>>(c->row_of, gbuf.p, wrow.p, ssum.p, E, gw_out.d);
        GBX_LAUNCH_CHECK();
    }
    GBX_CUDA(cudaMemsetAsync(loss.p, 0, sizeof(double), s));
    ppr_loss_kernel<<<eg, 256, 0, s>>>(lw.d, rin.d, (size_t)V * K, loss.p);
    GBX_LAUNCH_CHECK();
    GBX_TRY(gw_out.finish(s));
    GBX_TRY(gt_out.finish(s));
    double hl = 0.0;
    GBX_CUDA(cudaMemcpyAsync(&hl, loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    GBX_CUDA(cudaStreamSynchronize(s));
    if (res) {
        res->adjoint_iterations = iters;
        res->adjoint_residual = resid;
        res->loss = hl;
    }
    GBX_REQUIRE(st == GBX_OK, GBX_ERR_ITER_CAP,
                "PPR adjoint did not reach L1 residual %g in %u iterations (residual %g)", tol, max_it, resid);
    return GBX_OK;
}

int check_ppr_args(const gbx_graph *g, uint32_t K, double damping, double tol) {
    GBX_REQUIRE(g, GBX_ERR_INVALID, "graph is NULL");
    GBX_REQUIRE(K == 32 || K == 64 || K == 128 || K == 256, GBX_ERR_INVALID, "K must be 32, 64, 128 or 256 (got %u)",
                K);
    GBX_REQUIRE(damping > 0.0 && damping < 1.0, GBX_ERR_INVALID, "damping must be in (0, 1)");
    GBX_REQUIRE(tol > 0.0, GBX_ERR_INVALID, "tolerance must be > 0");
    GBX_REQUIRE(g->V > 0, GBX_ERR_INVALID, "graph has no vertices");
    return GBX_OK;
}

}  // namespace

extern "C" int gbx_ppr_forward(gbx_graph *g, uint32_t K, const float *weights, const float *teleport, double damping,
                               double tol, uint32_t max_iterations, float *ranks, gbx_ppr_result *result,
                               void *stream) {
    clear_error();
    if (result) *result = gbx_ppr_result{};
    GBX_TRY(check_ppr_args(g, K, damping, tol));
    GBX_REQUIRE((weights || g->E == 0) && teleport && ranks, GBX_ERR_INVALID, "NULL array argument");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const float d = (float)damping;
    switch (K) {
    case 32: return ppr_forward_impl<1>(g, weights, teleport, d, tol, max_iterations, ranks, result, s);
    case 64: return ppr_forward_impl<2>(g, weights, teleport, d, tol, max_iterations, ranks, result, s);
    case 128: return ppr_forward_impl<4>(g, weights, teleport, d, tol, max_iterations, ranks, result, s);
    default: return ppr_forward_impl<8>(g, weights, teleport, d, tol, max_iterations, ranks, result, s);
    }
}

extern "C" int gbx_ppr_adjoint(gbx_graph *g, uint32_t K, const float *weights, const float *ranks,
                               const float *loss_weights, double damping, double tol, uint32_t max_iterations,
                               float *grad_weights, float *grad_teleport, gbx_ppr_result *result, void *stream) {
    clear_error();
    if (result) *result = gbx_ppr_result{};
    GBX_TRY(check_ppr_args(g, K, damping, tol));
    GBX_REQUIRE((weights || g->E == 0) && ranks && loss_weights, GBX_ERR_INVALID, "NULL array argument");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const float d = (float)damping;
    switch (K) {
    case 32: return ppr_adjoint_impl<1>(g, weights, ranks, loss_weights, d, tol, max_iterations, grad_weights,
                                        grad_teleport, result, s);
    case 64: return ppr_adjoint_impl<2>(g, weights, ranks, loss_weights, d, tol, max_iterations, grad_weights,
                                        grad_teleport, result, s);
    case 128: return ppr_adjoint_impl<4>(g, weights, ranks, loss_weights, d, tol, max_iterations, grad_weights,
                                         grad_teleport, result, s);
    default: return ppr_adjoint_impl<8>(g, weights, ranks, loss_weights, d, tol, max_iterations, grad_weights,
                                        grad_teleport, result, s);
    }
}
