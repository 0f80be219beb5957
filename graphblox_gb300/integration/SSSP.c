/* cuda integration of SSSPGraphCSR and its Stats
 * (the reference's 01_host/src/algorithms/openmp/SSSP.c:76-511). */
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>

#include "SSSP.h"
#include "gbx_shim.h"

struct SSSPStats *newSSSPStatsGraphCSR(struct GraphCSR *graph, uint32_t delta) {
    struct SSSPStats *stats = (struct SSSPStats *)gbx_shim_alloc(sizeof(struct SSSPStats));
    uint32_t V = graph->num_vertices;
    stats->bucket_counter = 0;
    stats->delta = delta;
    stats->bucket_current = 0;
    stats->processed_nodes = 0;
    stats->buckets_total = 0;
    stats->time_total = 0.0;
    stats->num_vertices = V;
    stats->distances = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    stats->parents = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    stats->buckets_map = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    for (uint32_t v = 0; v < V; ++v) {
        stats->buckets_map[v] = UINT_MAX / 2;
        stats->distances[v] = UINT_MAX / 2;
        stats->parents[v] = UINT_MAX;
    }
    return stats;
}

void freeSSSPStats(struct SSSPStats *stats) {
    if (!stats) return;
    free(stats->distances);
    free(stats->parents);
    free(stats->buckets_map);
    free(stats);
}

struct SSSPStats *SSSPGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    /* SSSP.c:493: the source is remapped before the range check */
    if (arguments->source < graph->num_vertices)
        arguments->source = graph->sorted_edges_array->label_array[arguments->source];
    struct SSSPStats *stats = newSSSPStatsGraphCSR(graph, arguments->delta);
    if (arguments->source >= graph->num_vertices) {
        printf(" -----------------------------------------------------\n");
        printf("| %-51s | \n", "ERROR!! CHECK SOURCE RANGE");
        printf(" -----------------------------------------------------\n");
        return stats;
    }
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) {
        freeSSSPStats(stats);
        return NULL;
    }
    gbx_sssp_result r;
    double t0 = gbx_shim_now();
    /* the delta-stepping bucket width changes only the schedule; 0 = tuned */
    int st = gbx_sssp(g, arguments->source, 0, stats->distances, &r, NULL);
    stats->time_total = gbx_shim_now() - t0;
    if (st != GBX_OK) {
        freeSSSPStats(stats);
        return (struct SSSPStats *)gbx_shim_fail("gbx_sssp", st);
    }
    stats->parents[arguments->source] = arguments->source;
    stats->processed_nodes = r.reached;
    return stats;
}
