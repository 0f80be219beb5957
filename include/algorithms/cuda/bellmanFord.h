/* cuda integration: the reference's Bellman-Ford Stats and entry points
 * (01_host/include/algorithms/openmp/bellmanFord.h:19-54). Every variant
 * (pull, push, randomized push) runs gbx_bellman_ford on the GPU: they
 * reach the same distances; parents are the smallest valid ones. */
#ifndef BELLMANFORD_H
#define BELLMANFORD_H

#ifdef __cplusplus
extern "C" {
#endif

#include <stdint.h>
#include "graphConfig.h"
#include "graphCSR.h"

struct BellmanFordStats {
    uint32_t *distances;
    uint32_t *parents;
    uint32_t processed_nodes;
    uint32_t num_vertices;
    double time_total;
};

struct BellmanFordStats *newBellmanFordStatsGraphCSR(struct GraphCSR *graph);
void freeBellmanFordStats(struct BellmanFordStats *stats);
uint32_t bellmanFordCompareDistanceArrays(struct BellmanFordStats *stats1, struct BellmanFordStats *stats2);

struct BellmanFordStats *bellmanFordGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct BellmanFordStats *bellmanFordDataDrivenPullGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct BellmanFordStats *bellmanFordDataDrivenPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct BellmanFordStats *bellmanFordRandomizedDataDrivenPushGraphCSR(struct Arguments *arguments,
                                                                     struct GraphCSR *graph);

#ifdef __cplusplus
}
#endif

#endif
