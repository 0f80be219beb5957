/* cuda integration: same Stats struct and entry points as the reference's
 * 01_host/include/algorithms/openmp/SPMV.h:17-42, backed by gbx_spmv. */
#ifndef SPMV_H
#define SPMV_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
#include "graphConfig.h"
#include "graphCSR.h"
struct SPMVStats {
    uint32_t iterations;
    struct Arguments *arguments;
    uint32_t num_vertices;
    float *vector_output;
    float *vector_input;
    double time_total;
};
struct SPMVStats *newSPMVStatsGraphCSR(struct GraphCSR *graph);
void freeSPMVStats(struct SPMVStats *stats);
struct SPMVStats *SPMVGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
#ifdef __cplusplus
}
#endif
#endif
