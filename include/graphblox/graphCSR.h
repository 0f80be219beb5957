/* Layout-identical struct GraphCSR (01_host/include/structures/graphCSR.h:14-31):
 * fields depend on the WEIGHTED and DIRECTED build macros exactly as there. */
#ifndef GRAPHCSR_H
#define GRAPHCSR_H
#include <stdint.h>
#include "graphConfig.h"
#include "edgeList.h"
#include "vertex.h"
struct GraphCSR {
    uint32_t num_edges;
    uint32_t num_vertices;
    uint32_t avg_degree;
#if WEIGHTED
    float max_weight;
#endif
    struct Vertex *vertices;
    struct EdgeList *sorted_edges_array;
#if DIRECTED
    struct Vertex *inverse_vertices;
    struct EdgeList *inverse_sorted_edges_array;
#endif
};
#endif
