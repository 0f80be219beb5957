/* cuda integration of bellmanFordGraphCSR and its Stats
 * (the reference's 01_host/src/algorithms/openmp/bellmanFord.c:46-738). */
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>

#include "bellmanFord.h"
#include "gbx_shim.h"

struct BellmanFordStats *newBellmanFordStatsGraphCSR(struct GraphCSR *graph) {
    struct BellmanFordStats *stats = (struct BellmanFordStats *)gbx_shim_alloc(sizeof(struct BellmanFordStats));
    uint32_t V = graph->num_vertices;
    stats->processed_nodes = 0;
    stats->time_total = 0.0;
    stats->num_vertices = V;
    stats->distances = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    stats->parents = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    for (uint32_t v = 0; v < V; ++v) {
        stats->distances[v] = UINT_MAX / 2;
        stats->parents[v] = UINT_MAX;
    }
    return stats;
}

void freeBellmanFordStats(struct BellmanFordStats *stats) {
    if (!stats) return;
    free(stats->distances);
    free(stats->parents);
    free(stats);
}

uint32_t bellmanFordCompareDistanceArrays(struct BellmanFordStats *stats1, struct BellmanFordStats *stats2) {
    for (uint32_t v = 0; v < stats1->num_vertices; ++v)
        if (stats1->distances[v] != stats2->distances[v]) return 0;
    return 1;
}

/* the source is already remapped through label_array; every variant of the
 * reference sets arguments->iterations = V - 1 first (bellmanFord.c:449) */
static struct BellmanFordStats *run(struct Arguments *arguments, struct GraphCSR *graph) {
    arguments->iterations = graph->num_vertices - 1;
    struct BellmanFordStats *stats = newBellmanFordStatsGraphCSR(graph);
    if (arguments->source >= graph->num_vertices) {
        printf(" -----------------------------------------------------\n");
        printf("| %-51s | \n", "ERROR!! CHECK arguments->SOURCE RANGE");
        printf(" -----------------------------------------------------\n");
        return stats;
    }
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) {
        freeBellmanFordStats(stats);
        return NULL;
    }
    gbx_sssp_result r;
    double t0 = gbx_shim_now();
    int st = gbx_bellman_ford(g, arguments->source, stats->distances, stats->parents, &r, NULL);
    stats->time_total = gbx_shim_now() - t0;
    if (st != GBX_OK) {
        freeBellmanFordStats(stats);
        return (struct BellmanFordStats *)gbx_shim_fail("gbx_bellman_ford", st);
    }
    stats->processed_nodes = r.reached;
    return stats;
}

struct BellmanFordStats *bellmanFordGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    /* bellmanFord.c:422: the source is remapped before the variant runs */
    if (arguments->source < graph->num_vertices)
        arguments->source = graph->sorted_edges_array->label_array[arguments->source];
    return run(arguments, graph);
}

struct BellmanFordStats *bellmanFordDataDrivenPullGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return run(arguments, graph);
}

struct BellmanFordStats *bellmanFordDataDrivenPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return run(arguments, graph);
}

struct BellmanFordStats *bellmanFordRandomizedDataDrivenPushGraphCSR(struct Arguments *arguments,
                                                                     struct GraphCSR *graph) {
    return run(arguments, graph);
}
