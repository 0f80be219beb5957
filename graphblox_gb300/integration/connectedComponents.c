/* cuda integration of connectedComponentsGraphCSR and its Stats
 * (the reference's 01_host/src/algorithms/openmp/connectedComponents.c:49-629). */
#include <stdio.h>
#include <stdlib.h>

#include "connectedComponents.h"
#include "gbx_shim.h"

struct CCStats *newCCStatsGraphCSR(struct GraphCSR *graph) {
    struct CCStats *stats = (struct CCStats *)gbx_shim_alloc(sizeof(struct CCStats));
    uint32_t V = graph->num_vertices;
    stats->iterations = 0;
    stats->neighbor_rounds = 2;
    stats->num_vertices = V;
    stats->time_total = 0.0;
    stats->components = (uint32_t *)gbx_shim_alloc((V + 1) * sizeof(uint32_t));
    stats->counts = (uint32_t *)gbx_shim_alloc((V + 1) * sizeof(uint32_t));
    stats->labels = (uint32_t *)gbx_shim_alloc((V + 1) * sizeof(uint32_t));
    for (uint32_t v = 0; v < V; ++v) {
        stats->components[v] = v;
        stats->labels[v] = v;
    }
    return stats;
}

void freeCCStats(struct CCStats *stats) {
    if (!stats) return;
    free(stats->components);
    free(stats->counts);
    free(stats->labels);
    free(stats);
}

static struct CCStats *run_cc(struct Arguments *arguments, struct GraphCSR *graph, int variant) {
    struct CCStats *stats = newCCStatsGraphCSR(graph);
    stats->arguments = arguments;
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) {
        freeCCStats(stats);
        return NULL;
    }
    double t0 = gbx_shim_now();
    uint32_t iters = 0;
    int st = gbx_cc(g, variant, stats->components, &iters, NULL);
    stats->time_total = gbx_shim_now() - t0;
    if (st != GBX_OK) {
        freeCCStats(stats);
        return (struct CCStats *)gbx_shim_fail("gbx_cc", st);
    }
    stats->iterations = iters;
    return stats;
}

struct CCStats *connectedComponentsShiloachVishkinGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return run_cc(arguments, graph, 0);
}
struct CCStats *connectedComponentsAfforestGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return run_cc(arguments, graph, 1);
}
struct CCStats *connectedComponentsWeaklyGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return run_cc(arguments, graph, 2);
}
struct CCStats *connectedComponentsGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    switch (arguments->pushpull) {
    case 0: return connectedComponentsShiloachVishkinGraphCSR(arguments, graph);
    case 2: return connectedComponentsWeaklyGraphCSR(arguments, graph);
    default: return connectedComponentsAfforestGraphCSR(arguments, graph);
    }
}
