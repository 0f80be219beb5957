/* cuda integration of depthFirstSearchGraphCSR and its Stats
 * (the reference's 01_host/src/algorithms/openmp/DFS.c:42-265). */
#include <stdio.h>
#include <stdlib.h>

#include "DFS.h"
#include "gbx_shim.h"

struct DFSStats *newDFSStatsGraphCSR(struct GraphCSR *graph) {
    struct DFSStats *stats = (struct DFSStats *)gbx_shim_alloc(sizeof(struct DFSStats));
    uint32_t V = graph->num_vertices;
    stats->distances = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    stats->parents = (int *)gbx_shim_alloc(V * sizeof(int));
    stats->processed_nodes = 0;
    stats->num_vertices = V;
    stats->time_total = 0.0;
    for (uint32_t v = 0; v < V; ++v) {
        stats->distances[v] = 0;
        stats->parents[v] = -1;
    }
    return stats;
}

void freeDFSStats(struct DFSStats *stats) {
    if (!stats) return;
    free(stats->distances);
    free(stats->parents);
    free(stats);
}

/* DFS uses arguments->source as given (no label remapping, DFS.c:156-170) */
struct DFSStats *depthFirstSearchGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    struct DFSStats *stats = newDFSStatsGraphCSR(graph);
    if (arguments->source >= graph->num_vertices) {
        printf(" -----------------------------------------------------\n");
        printf("| %-51s | \n", "ERROR!! CHECK SOURCE RANGE");
        printf(" -----------------------------------------------------\n");
        return stats;
    }
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) {
        freeDFSStats(stats);
        return NULL;
    }
    double t0 = gbx_shim_now();
    int st = gbx_dfs(g, arguments->source, stats->distances, stats->parents, &stats->processed_nodes, NULL);
    stats->time_total = gbx_shim_now() - t0;
    if (st != GBX_OK) {
        freeDFSStats(stats);
        return (struct DFSStats *)gbx_shim_fail("gbx_dfs", st);
    }
    return stats;
}

struct DFSStats *depthFirstSearchGraphCSRBase(struct Arguments *arguments, struct GraphCSR *graph) {
    return depthFirstSearchGraphCSR(arguments, graph);
}

/* the reference's task-parallel variant claims vertices by compare-and-swap
 * in a schedule-dependent order; the sequential traversal is one valid
 * outcome of it */
struct DFSStats *pDepthFirstSearchGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return depthFirstSearchGraphCSR(arguments, graph);
}
