/* Layout-identical struct Vertex (01_host/include/structures/vertex.h:17-23). */
#ifndef VERTEX_H
#define VERTEX_H
#include <stdint.h>
struct Vertex {
    uint32_t num_vertices;
    uint32_t *out_degree;
    uint32_t *in_degree;
    uint32_t *edges_idx;
};
#endif
