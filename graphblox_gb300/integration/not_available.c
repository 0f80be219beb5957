/* Symbols graphRun.c links for the algorithm outside the GPU backend
 * (clustering, cluster.c): it reports that it is not available and returns
 * NULL, which graphRun.c treats as a failed run (graphRun.c:473-477); the
 * free function accepts NULL. */
#include <stdio.h>
#include <stdlib.h>

#include "cluster.h"
#include "gbx_shim.h"

void freeClusterStats(struct ClusterStats *stats) { free(stats); }

struct ClusterStats *clusterGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    (void)arguments; (void)graph;
    gbx_shim_not_available("Clustering");
    return NULL;
}
