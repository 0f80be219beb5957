/* cuda integration: same Stats struct and entry points as the reference's
 * 01_host/include/algorithms/openmp/triangleCount.h:16-43, backed by gbx_tc. */
#ifndef TRIANGLECOUNT_H
#define TRIANGLECOUNT_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
#include "graphConfig.h"
#include "graphCSR.h"
struct TCStats {
    uint32_t num_vertices;
    uint64_t *counts;
    uint64_t total_counts;
    double time_total;
};
struct TCStats *newTCStatsGraphCSR(struct GraphCSR *graph);
void freeTCStats(struct TCStats *stats);
struct TCStats *triangleCountGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
#ifdef __cplusplus
}
#endif
#endif
