/* cuda integration: same Stats struct and entry points as the reference's
 * 01_host/include/algorithms/openmp/connectedComponents.h:22-59, backed by gbx_cc. */
#ifndef CONNECTEDCOMPONENTS_H
#define CONNECTEDCOMPONENTS_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
#include "graphConfig.h"
#include "graphCSR.h"
struct CCStats {
    uint32_t iterations;
    uint32_t neighbor_rounds;
    struct Arguments *arguments;
    uint32_t num_vertices;
    uint32_t *components;
    uint32_t *counts;
    uint32_t *labels;
    double time_total;
};
struct CCStats *newCCStatsGraphCSR(struct GraphCSR *graph);
void freeCCStats(struct CCStats *stats);
struct CCStats *connectedComponentsGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct CCStats *connectedComponentsAfforestGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct CCStats *connectedComponentsShiloachVishkinGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct CCStats *connectedComponentsWeaklyGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
#ifdef __cplusplus
}
#endif
#endif
