/* cuda integration: the reference's DFS Stats and entry points
 * (01_host/include/algorithms/openmp/DFS.h:18-36), which graphRun.c links;
 * DFS is not part of the GPU backend, so the entry point reports that and
 * returns NULL (graphRun.c treats NULL Stats as a failed run). */
#ifndef DFS_H
#define DFS_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
#include "graphConfig.h"
#include "graphCSR.h"
struct DFSStats {
    uint32_t *distances;
    int *parents;
    uint32_t processed_nodes;
    uint32_t num_vertices;
    double time_total;
};
void freeDFSStats(struct DFSStats *stats);
struct DFSStats *depthFirstSearchGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
#ifdef __cplusplus
}
#endif
#endif
