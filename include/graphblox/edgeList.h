/* Layout-identical struct EdgeList (01_host/include/structures/edgeList.h:12-23). */
#ifndef EDGELIST_H
#define EDGELIST_H
#include <stdint.h>
struct EdgeList {
    uint32_t num_edges;
    uint32_t num_vertices;
    uint32_t avg_degree;
    float max_weight;
    float *edges_array_weight;
    uint32_t *edges_array_src;
    uint32_t *edges_array_dest;
    uint32_t *mask_array;
    uint32_t *label_array;
    uint32_t *inverse_label_array;
};
#endif
