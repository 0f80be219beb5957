/* cuda integration: the reference's cluster Stats and entry points
 * (01_host/include/algorithms/openmp/cluster.h:23-73); not part of the GPU
 * backend: the entry point reports that and returns NULL. */
#ifndef CLUSTER_H
#define CLUSTER_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
#include "graphConfig.h"
#include "graphCSR.h"
struct ClusterStats {
    uint32_t *partitions;
    uint32_t processed_nodes;
    uint32_t num_vertices;
    uint32_t iteration;
    long double total_weight;
    double time_total;
};
void freeClusterStats(struct ClusterStats *stats);
struct ClusterStats *clusterGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
#ifdef __cplusplus
}
#endif
#endif
