/* cuda integration of betweennessCentralityGraphCSR and its Stats
 * (the reference's 01_host/src/algorithms/openmp/betweennessCentrality.c:44-466). */
#include <stdio.h>
#include <stdlib.h>

#include "betweennessCentrality.h"
#include "gbx_shim.h"

/* One value of the generator in the caller's state: gbx_mt19937_next steps
 * the reference's mt19937state (01_host/include/utils_graph/mt19937.h:58-62)
 * in place, so the stream continues exactly as the reference's
 * generateRandInt would continue it. */
static unsigned long mt_next(mt19937state *m) { return gbx_mt19937_next(m->mt, &m->mti); }

/* betweennessCentrality.c:172-189: draw until a vertex with out-degree above
 * the average */
uint32_t generateRandomRootBetweennessCentrality(mt19937state *mt19937var, struct GraphCSR *graph) {
    for (;;) {
        const unsigned long r = mt_next(mt19937var);
        if (r < graph->num_vertices && graph->vertices->out_degree[r] > graph->avg_degree) return (uint32_t)r;
    }
}

struct BetweennessCentralityStats *newBetweennessCentralityStatsGraphCSR(struct GraphCSR *graph) {
    uint32_t V = graph->num_vertices;
    struct BetweennessCentralityStats *stats =
        (struct BetweennessCentralityStats *)gbx_shim_alloc(sizeof(struct BetweennessCentralityStats));
    stats->betweennessCentrality = (float *)gbx_shim_alloc(V * sizeof(float));
    stats->stack = (struct Predecessor *)gbx_shim_alloc(sizeof(struct Predecessor));
    stats->stack->nodes = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    stats->stack->degree = 0;
    stats->distances = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    stats->realRanks = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    stats->parents = (int *)gbx_shim_alloc(V * sizeof(int));
    stats->sigma = (int *)gbx_shim_alloc(V * sizeof(int));
    stats->dependency = (float *)gbx_shim_alloc(V * sizeof(float));
    /* predecessor lists are not materialised (degree 0): the GPU walks the
     * successor CSR instead */
    stats->predecessors = (struct Predecessor *)gbx_shim_alloc(V * sizeof(struct Predecessor));
    stats->processed_nodes = 0;
    stats->iteration = 0;
    stats->num_vertices = V;
    stats->time_total = 0.0;
    for (uint32_t v = 0; v < V; ++v) {
        stats->distances[v] = UINT32_MAX;
        stats->realRanks[v] = v;
        stats->parents[v] = graph->vertices->out_degree[v] ? -(int)graph->vertices->out_degree[v] : -1;
    }
    return stats;
}

void clearBetweennessCentralityStats(struct BetweennessCentralityStats *stats) {
    stats->stack->degree = 0;
    stats->processed_nodes = 0;
    for (uint32_t v = 0; v < stats->num_vertices; ++v) {
        stats->distances[v] = UINT32_MAX;
        stats->dependency[v] = 0.0f;
        stats->sigma[v] = 0;
        stats->stack->nodes[v] = 0;
        stats->predecessors[v].degree = 0;
        stats->parents[v] = -1;
    }
}

void freeBetweennessCentralityStats(struct BetweennessCentralityStats *stats) {
    if (!stats) return;
    free(stats->distances);
    free(stats->parents);
    free(stats->dependency);
    free(stats->sigma);
    free(stats->betweennessCentrality);
    free(stats->realRanks);
    if (stats->stack) free(stats->stack->nodes);
    free(stats->stack);
    if (stats->predecessors) {
        for (uint32_t v = 0; v < stats->num_vertices; ++v) free(stats->predecessors[v].nodes);
        free(stats->predecessors);
    }
    free(stats);
}

void printRanksBetweennessCentralityStats(struct BetweennessCentralityStats *stats) { (void)stats; }

struct BetweennessCentralityStats *betweennessCentralityBrandesGraphCSR(struct Arguments *arguments,
                                                                       struct GraphCSR *graph) {
    struct BetweennessCentralityStats *stats = newBetweennessCentralityStatsGraphCSR(graph);
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) {
        freeBetweennessCentralityStats(stats);
        return NULL;
    }
    const uint32_t n = arguments->iterations, V = graph->num_vertices;
    uint32_t *roots = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    if (!roots) {
        freeBetweennessCentralityStats(stats);
        return NULL;
    }
    for (uint32_t i = 0; i < n; ++i) roots[i] = generateRandomRootBetweennessCentrality(&arguments->mt19937var, graph);
    if (n) clearBetweennessCentralityStats(stats);
    gbx_bc_result r;
    double t0 = gbx_shim_now();
    int st = gbx_betweenness(g, n, roots, stats->betweennessCentrality, stats->distances, stats->sigma,
                             stats->dependency, &r, NULL);
    stats->time_total = gbx_shim_now() - t0;
    if (st != GBX_OK) {
        free(roots);
        freeBetweennessCentralityStats(stats);
        return (struct BetweennessCentralityStats *)gbx_shim_fail("gbx_betweenness", st);
    }
    stats->iteration = r.iteration;
    stats->processed_nodes = r.processed_nodes;
    if (n) {
        /* the last root's stack: levels in order, ids ascending inside a level
         * (copyBitmapToStack, betweennessCentrality.c:205-217) */
        const uint32_t levels = r.levels;
        uint32_t *start = (uint32_t *)calloc((size_t)levels + 1, sizeof(uint32_t));
        if (start) {
            for (uint32_t v = 0; v < V; ++v)
                if (stats->distances[v] < levels) start[stats->distances[v] + 1]++;
            for (uint32_t l = 0; l < levels; ++l) start[l + 1] += start[l];
            for (uint32_t v = 0; v < V; ++v)
                if (stats->distances[v] < levels) stats->stack->nodes[start[stats->distances[v]]++] = v;
            stats->stack->degree = levels ? start[levels - 1] : 0;
            free(start);
        }
        stats->parents[roots[n - 1]] = (int)roots[n - 1];
    }
    free(roots);
    return stats;
}

struct BetweennessCentralityStats *betweennessCentralityGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return betweennessCentralityBrandesGraphCSR(arguments, graph);
}
