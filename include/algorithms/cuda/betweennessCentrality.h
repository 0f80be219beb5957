/* cuda integration: the reference's betweenness Stats and entry points
 * (01_host/include/algorithms/openmp/betweennessCentrality.h:16-60). Brandes
 * runs in gbx_betweenness on the GPU from roots drawn, as the reference
 * draws them, from arguments->mt19937var. */
#ifndef BETWEENNESSCENTRALITY_H
#define BETWEENNESSCENTRALITY_H

#ifdef __cplusplus
extern "C" {
#endif

#include <stdint.h>
#include "graphConfig.h"
#include "graphCSR.h"

struct Predecessor {
    uint32_t *nodes;
    uint32_t degree;
};

struct BetweennessCentralityStats {
    struct Predecessor *stack;
    uint32_t *distances;
    uint32_t *realRanks;
    int *parents;
    int *sigma;
    float *dependency;
    float *betweennessCentrality;
    struct Predecessor *predecessors;
    uint32_t iteration;
    uint32_t processed_nodes;
    uint32_t num_vertices;
    double time_total;
};

struct BetweennessCentralityStats *newBetweennessCentralityStatsGraphCSR(struct GraphCSR *graph);
void freeBetweennessCentralityStats(struct BetweennessCentralityStats *stats);
void clearBetweennessCentralityStats(struct BetweennessCentralityStats *stats);
void printRanksBetweennessCentralityStats(struct BetweennessCentralityStats *stats);
uint32_t generateRandomRootBetweennessCentrality(mt19937state *mt19937var, struct GraphCSR *graph);

struct BetweennessCentralityStats *betweennessCentralityGraphCSR(struct Arguments *arguments, struct GraphCSR *graph);
struct BetweennessCentralityStats *betweennessCentralityBrandesGraphCSR(struct Arguments *arguments,
                                                                       struct GraphCSR *graph);

#ifdef __cplusplus
}
#endif

#endif
