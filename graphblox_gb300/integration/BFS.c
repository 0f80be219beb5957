/* cuda integration of breadthFirstSearchGraphCSR and its Stats
 * (the reference's 01_host/src/algorithms/openmp/BFS.c:42-127). */
#include <stdio.h>
#include <stdlib.h>

#include "BFS.h"
#include "gbx_shim.h"

struct BFSStats *newBFSStatsGraphCSR(struct GraphCSR *graph) {
    /* BFS.c:42-78: distances 0, parents -out_degree (or -1) */
    struct BFSStats *stats = (struct BFSStats *)gbx_shim_alloc(sizeof(struct BFSStats));
    uint32_t V = graph->num_vertices;
    stats->distances = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    stats->distances_DualOrder = (uint32_t *)gbx_shim_alloc(V * sizeof(uint32_t));
    stats->parents = (int *)gbx_shim_alloc(V * sizeof(int));
    stats->parents_DualOrder = (int *)gbx_shim_alloc(V * sizeof(int));
    stats->processed_nodes = 0;
    stats->iteration = 0;
    stats->num_vertices = V;
    stats->time_total = 0.0;
    for (uint32_t v = 0; v < V; ++v) {
        uint32_t d = graph->vertices->out_degree[v];
        stats->parents[v] = d ? -(int)d : -1;
        stats->parents_DualOrder[v] = stats->parents[v];
    }
    return stats;
}

void freeBFSStats(struct BFSStats *stats) {
    if (!stats) return;
    free(stats->distances);
    free(stats->parents);
    free(stats->distances_DualOrder);
    free(stats->parents_DualOrder);
    free(stats);
}

static struct BFSStats *run_bfs(struct Arguments *arguments, struct GraphCSR *graph, int mode) {
    struct BFSStats *stats = newBFSStatsGraphCSR(graph);
    if (arguments->source >= graph->num_vertices) {
        printf(" -----------------------------------------------------\n");
        printf("| %-51s | \n", "ERROR!! CHECK SOURCE RANGE");
        printf(" -----------------------------------------------------\n");
        return stats;
    }
    /* BFS.c:153: the source is given in original ids */
    arguments->source = graph->sorted_edges_array->label_array[arguments->source];
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) {
        freeBFSStats(stats);
        return NULL;
    }
    gbx_bfs_result r;
    double t0 = gbx_shim_now();
    int st = gbx_bfs(g, arguments->source, mode, stats->distances, stats->parents, &r, NULL);
    stats->time_total = gbx_shim_now() - t0;
    if (st != GBX_OK) {
        freeBFSStats(stats);
        return (struct BFSStats *)gbx_shim_fail("gbx_bfs", st);
    }
    stats->processed_nodes = r.processed_nodes;
    stats->iteration = r.iteration;
    return stats;
}

struct BFSStats *breadthFirstSearchPullGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return run_bfs(arguments, graph, 0);
}

struct BFSStats *breadthFirstSearchPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return run_bfs(arguments, graph, 1);
}

struct BFSStats *breadthFirstSearchDirectionOptimizedGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    return run_bfs(arguments, graph, 2);
}

struct BFSStats *breadthFirstSearchGraphCSR(struct Arguments *arguments, struct GraphCSR *graph) {
    switch (arguments->pushpull) {
    case 0: return breadthFirstSearchPullGraphCSR(arguments, graph);
    case 1: return breadthFirstSearchPushGraphCSR(arguments, graph);
    default: return breadthFirstSearchDirectionOptimizedGraphCSR(arguments, graph);
    }
}

/* BFS.c:498-546: expand the shared queue's current frontier [head, tail);
 * the vertices claimed are appended from tail_next on. The reference
 * gathers them in the per-thread queues and flushes those into the shared
 * one, which leaves them empty; here they are not used, so they stay as the
 * caller passed them (empty between steps). Returns mf, the sum of -parent
 * over the claimed vertices. A failure prints the library's message and
 * returns 0 with nothing appended. */
uint32_t topDownStepGraphCSR(struct GraphCSR *graph, struct ArrayQueue *sharedFrontierQueue,
                             struct ArrayQueue **localFrontierQueues, struct BFSStats *stats) {
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) return 0;
    struct ArrayQueue *q = sharedFrontierQueue;
    const uint32_t n = q->tail - q->head;
    uint32_t next_len = 0, mf = 0;
    const uint32_t cap = q->size > q->tail_next ? q->size - q->tail_next : 0;
    int st = gbx_bfs_top_down_step(g, q->queue + q->head, n, stats->parents, stats->distances,
                                   q->queue + q->tail_next, cap, &next_len, &mf, NULL);
    if (st != GBX_OK) {
        gbx_shim_fail("gbx_bfs_top_down_step", st);
        return 0;
    }
    q->tail_next += next_len;
    return mf;
}

/* BFS.c:562-613: every vertex without a parent looks for an in-neighbour in
 * bitmapCurr; the found ones are set in bitmapNext. Returns nf, the number
 * found; a failure prints the library's message and returns 0. */
uint32_t bottomUpStepGraphCSR(struct GraphCSR *graph, struct Bitmap *bitmapCurr, struct Bitmap *bitmapNext,
                              struct BFSStats *stats) {
    gbx_graph *g = gbx_shim_graph(graph);
    if (!g) return 0;
    uint32_t nf = 0;
    int st = gbx_bfs_bottom_up_step(g, bitmapCurr->bitarray, bitmapNext->bitarray, stats->parents,
                                    stats->distances, &nf, NULL);
    if (st != GBX_OK) {
        gbx_shim_fail("gbx_bfs_bottom_up_step", st);
        return 0;
    }
    return nf;
}
