/* cuda integration of triangleCountGraphCSR and its Stats
 * (the reference's 01_host/src/algorithms/openmp/triangleCount.c:36-182). */
#include <stdio.h>
#include <stdlib.h>

#include "gbx_shim.h"
#include "triangleCount.h"

struct TCStats *newTCStatsGraphCSR(struct GraphCSR *graph) {
    struct TCStats *stats = (struct TCStats *)gbx_shim_alloc(sizeof(struct TCStats));
    stats->total_counts = 0;
    stats->num_vertices = graph->num_vertices;
    stats->time_total = 0.0;
    stats->counts = (uint64_t *)gbx_shim_alloc(graph->num_vertices * sizeof(uint64_t));
    return stats;
}

void freeTCStats(struct TCStats *stats) {
    if (!stats) return;
    free(stats->counts);
    free(stats);
}

struct TCStats *triangleCountGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    (void)arguments;  /* every variant (basic/pull/push/binary) reports the same total */
    struct TCStats *stats = newTCStatsGraphCSR(graph);
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) {
        freeTCStats(stats);
        return NULL;
    }
    uint64_t total = 0;
    double t0 = gbx_shim_now();
    int st = gbx_tc(g, &total, NULL);
    stats->time_total = gbx_shim_now() - t0;
    if (st != GBX_OK) {
        freeTCStats(stats);
        return (struct TCStats *)gbx_shim_fail("gbx_tc", st);
    }
    stats->total_counts = total;
    return stats;
}
