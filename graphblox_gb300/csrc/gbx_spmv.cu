// SpMV pull (the reference's SPMVPullGraphCSR, SPMV.c:117-215):
// y[v] += sum over pull edges (u->v) of w_uv * x[u], repeated `iterations`
// times with y never reset. The pull engine (gbx_gather.cuh) computes each
// row's sum (Kahan-compensated on medium and heavy rows) and adds it to y.
#include "gbx_gather.cuh"

namespace gbx {

struct SpmvTerm {
    const uint32_t *__restrict__ src;
    const float *__restrict__ val;  // may be null
    float dflt;
    const float *__restrict__ x;
    // index and value streams are read once: evict-first, keeping x in L2
    __device__ __forceinline__ uint32_t src_of(uint32_t e) const { return __ldcs(src + e); }
    __device__ __forceinline__ float value(uint32_t e, uint32_t u) const {
        float w = val ? __ldcs(val + e) : dflt;
        return __fmul_rn(w, __ldg(x + u));
    }
};

struct SpmvEpi {
    float *__restrict__ y;
    __device__ __forceinline__ void operator()(uint32_t v, float sum) { y[v] = __fadd_rn(y[v], sum); }
    __device__ __forceinline__ void block_finish() {}
};

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_spmv(gbx_graph *g, const float *values, float default_value, const float *x,
                        float *y, uint32_t iterations, void *stream) {
    clear_error();
    GBX_REQUIRE(g && x && y, GBX_ERR_INVALID, "graph, x or y is NULL");
    GBX_TRY(ensure_device());
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t V = g->V;
    gbx_gather_plan *plan = nullptr;
    GBX_TRY(get_pull_plan(g, s, &plan));
    InArray<float> xin, vin;
    GBX_TRY(xin.bind(x, V, s));
    const float *vals = nullptr;
    if (values) {
        GBX_TRY(vin.bind(values, g->E, s));
        vals = vin.d;
    } else {
        vals = g->pull_weight();
    }
    // y is read and written: stage host y in and out
    OutArray<float> yout;
    GBX_TRY(yout.bind(y, V, s));
    if (yout.to_host()) GBX_CUDA(cudaMemcpyAsync(yout.d, y, (size_t)V * 4, cudaMemcpyHostToDevice, s));
    SpmvTerm term{g->pull_src(), vals, default_value, xin.d};
    SpmvEpi epi{yout.d};
    for (uint32_t it = 0; it < iterations; ++it)
        GBX_TRY(launch_gather(g->pull_offsets(), V, *plan, term, epi, s));
    GBX_TRY(yout.finish(s));
    if (yout.to_host()) GBX_CUDA(cudaStreamSynchronize(s));
    return GBX_OK;
}
