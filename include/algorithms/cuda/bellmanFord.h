/* cuda integration: the reference's Bellman-Ford Stats and entry points
 * (01_host/include/algorithms/openmp/bellmanFord.h:19-47); not part of the
 * GPU backend: the entry point reports that and returns NULL. */
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
void freeBellmanFordStats(struct BellmanFordStats *stats);
struct BellmanFordStats *bellmanFordGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
#ifdef __cplusplus
}
#endif
#endif
