/* cuda integration: same Stats struct and entry points as the reference's
 * 01_host/include/algorithms/openmp/pageRank.h:19-74, backed by gbx_pagerank_pull. */
#ifndef PAGERANK_H
#define PAGERANK_H
#ifdef __cplusplus
extern "C" {
#endif
#include <stdint.h>
#include "graphConfig.h"
#include "graphCSR.h"
#define Damp 0.85f
struct PageRankStats {
    float damp;
    float base_pr;
    uint32_t iterations;
    uint32_t num_vertices;
    uint32_t activeVertices;
    uint32_t *realRanks;
    float *pageRanks;
    double time_total;
    double error_total;
};
struct PageRankStats *newPageRankStatsGraphCSR(struct GraphCSR *graph);
void freePageRankStats(struct PageRankStats *stats);
struct PageRankStats *pageRankGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPullGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct PageRankStats *pageRankPushGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
#ifdef __cplusplus
}
#endif
#endif
