/* Symbols graphRun.c links for algorithms outside the GPU backend (DFS,
 * Bellman-Ford, betweenness centrality, clustering): they report that they
 * are not available and return NULL, which graphRun.c treats as a failed
 * run (graphRun.c:473-477); the free functions accept NULL. */
#include <stdio.h>
#include <stdlib.h>

#include "DFS.h"
#include "bellmanFord.h"
#include "betweennessCentrality.h"
#include "cluster.h"
#include "gbx_shim.h"

void freeDFSStats(struct DFSStats *stats) { free(stats); }
void freeBellmanFordStats(struct BellmanFordStats *stats) { free(stats); }
void freeBetweennessCentralityStats(struct BetweennessCentralityStats *stats) { free(stats); }
void freeClusterStats(struct ClusterStats *stats) { free(stats); }
void printRanksBetweennessCentralityStats(struct BetweennessCentralityStats *stats) { (void)stats; }

struct DFSStats *depthFirstSearchGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    (void)arguments; (void)graph;
    gbx_shim_not_available("DFS");
    return NULL;
}
struct BellmanFordStats *bellmanFordGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    (void)arguments; (void)graph;
    gbx_shim_not_available("Bellman-Ford");
    return NULL;
}
struct BetweennessCentralityStats *betweennessCentralityGraphCSR(struct Arguments *arguments,
                                                                 struct GraphCSR *graph) {
    (void)arguments; (void)graph;
    gbx_shim_not_available("Betweenness centrality");
    return NULL;
}
struct ClusterStats *clusterGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    (void)arguments; (void)graph;
    gbx_shim_not_available("Clustering");
    return NULL;
}
