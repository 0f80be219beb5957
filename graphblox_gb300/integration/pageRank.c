/* cuda integration of pageRankGraphCSR and its Stats
 * (the reference's 01_host/src/algorithms/openmp/pageRank.c:47-242). */
#include <stdio.h>
#include <stdlib.h>

#include "gbx_shim.h"
#include "pageRank.h"

struct PageRankStats *newPageRankStatsGraphCSR(struct GraphCSR *graph) {
    struct PageRankStats *stats = (struct PageRankStats *)gbx_shim_alloc(sizeof(struct PageRankStats));
    stats->damp = Damp;
    stats->base_pr = 1.0f - stats->damp;
    stats->iterations = 0;
    stats->num_vertices = graph->num_vertices;
    stats->time_total = 0.0;
    stats->error_total = 0.0;
    stats->realRanks = (uint32_t *)gbx_shim_alloc(graph->num_vertices * sizeof(uint32_t));
    stats->pageRanks = (float *)gbx_shim_alloc(graph->num_vertices * sizeof(float));
    for (uint32_t v = 0; v < graph->num_vertices; ++v) {
        stats->pageRanks[v] = stats->base_pr;
        stats->realRanks[v] = v;
    }
    return stats;
}

void freePageRankStats(struct PageRankStats *stats) {
    if (!stats) return;
    free(stats->realRanks);
    free(stats->pageRanks);
    free(stats);
}

struct PageRankStats *pageRankPullGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    struct PageRankStats *stats = newPageRankStatsGraphCSR(graph);
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) {
        freePageRankStats(stats);
        return NULL;
    }
    gbx_pr_result r;
    double t0 = gbx_shim_now();
    int st = gbx_pagerank_pull(g, arguments->iterations, arguments->epsilon, stats->pageRanks, &r, NULL);
    stats->time_total = gbx_shim_now() - t0;
    if (st != GBX_OK) {
        freePageRankStats(stats);
        return (struct PageRankStats *)gbx_shim_fail("gbx_pagerank_pull", st);
    }
    stats->iterations = r.iterations;
    stats->activeVertices = r.active_last;
    stats->error_total = r.error_total;
    return stats;
}

/* The push form (pageRank.c:370-492) computes the same FP32 recurrence. */
struct PageRankStats *pageRankPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return pageRankPullGraphCSR(arguments, graph);
}

struct PageRankStats *pageRankGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    switch (arguments->pushpull) {
    case 0: case 1: case 6: case 7: case 8:
        /* FP32 pull / push / data-driven forms: same recurrence */
        return pageRankPullGraphCSR(arguments, graph);
    default:
        /* fixed-point and quantised forms are not part of the GPU backend */
        gbx_shim_not_available("PageRank fixed-point/quantised variant");
        return NULL;
    }
}
