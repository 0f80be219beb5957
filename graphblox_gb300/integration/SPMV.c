/* cuda integration of SPMVGraphCSR and its Stats
 * (the reference's 01_host/src/algorithms/openmp/SPMV.c:44-215). */
#include <stdio.h>
#include <stdlib.h>

#include "SPMV.h"
#include "gbx_shim.h"

struct SPMVStats *newSPMVStatsGraphCSR(struct GraphCSR *graph) {
    struct SPMVStats *stats = (struct SPMVStats *)gbx_shim_alloc(sizeof(struct SPMVStats));
    stats->iterations = 0;
    stats->num_vertices = graph->num_vertices;
    stats->time_total = 0.0;
    stats->vector_output = (float *)gbx_shim_alloc(graph->num_vertices * sizeof(float));
    stats->vector_input = (float *)gbx_shim_alloc(graph->num_vertices * sizeof(float));
    return stats;
}

void freeSPMVStats(struct SPMVStats *stats) {
    if (!stats) return;
    free(stats->vector_output);
    free(stats->vector_input);
    free(stats);
}

struct SPMVStats *SPMVGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    switch (arguments->pushpull) {
    case 0: case 1: break;  /* FP32 pull and push compute the same product */
    default:
        gbx_shim_not_available("SpMV fixed-point variant");
        return NULL;
    }
    struct SPMVStats *stats = newSPMVStatsGraphCSR(graph);
    stats->arguments = arguments;
    /* SPMV.c:156-163: x = 1/out_degree, or 0.001 for dangling vertices */
    for (uint32_t v = 0; v < graph->num_vertices; ++v) {
        uint32_t d = graph->vertices->out_degree[v];
        stats->vector_input[v] = d ? 1.0f / d : 0.001f;
    }
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) {
        freeSPMVStats(stats);
        return NULL;
    }
    double t0 = gbx_shim_now();
    /* values: the graph's weights (WEIGHTED build) or the constant 0.0001f */
    int st = gbx_spmv(g, NULL, 0.0001f, stats->vector_input, stats->vector_output, arguments->iterations, NULL);
    stats->time_total = gbx_shim_now() - t0;
    if (st != GBX_OK) {
        freeSPMVStats(stats);
        return (struct SPMVStats *)gbx_shim_fail("gbx_spmv", st);
    }
    stats->iterations = arguments->iterations;
    return stats;
}
