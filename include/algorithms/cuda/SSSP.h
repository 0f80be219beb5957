/* cuda integration: same Stats struct and entry points as the reference's
 * 01_host/include/algorithms/openmp/SSSP.h:18-54, backed by gbx_sssp. */
#ifndef SSSP_H
#define SSSP_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
#include "graphConfig.h"
#include "graphCSR.h"
struct SSSPStats {
    uint32_t *distances;
    uint32_t *parents;
    uint32_t *buckets_map;
    uint32_t bucket_counter;
    uint32_t bucket_current;
    uint32_t buckets_total;
    uint32_t processed_nodes;
    uint32_t delta;
    uint32_t num_vertices;
    double time_total;
};
struct SSSPStats *newSSSPStatsGraphCSR(struct GraphCSR *graph, uint32_t delta);
void freeSSSPStats(struct SSSPStats *stats);
struct SSSPStats *SSSPGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
#ifdef __cplusplus
}
#endif
#endif
