/* cuda integration: the reference's DFS Stats and entry points
 * (01_host/include/algorithms/openmp/DFS.h:18-39). All of them run
 * gbx_dfs, the reference's stack traversal, on the GPU. */
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

struct DFSStats *newDFSStatsGraphCSR(struct GraphCSR *graph);
void freeDFSStats(struct DFSStats *stats);

struct DFSStats *depthFirstSearchGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct DFSStats *depthFirstSearchGraphCSRBase(struct Arguments *arguments, struct GraphCSR *graph);
struct DFSStats *pDepthFirstSearchGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);

#ifdef __cplusplus
}
#endif

#endif
