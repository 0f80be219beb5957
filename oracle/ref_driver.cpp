// Dump driver for the reference OpenMP host, built from the reference's own
// sources by oracle/build_ref.sh. Test infrastructure only: it is the
// "oracle/_ref" reference run that pins the C restatement (oracle/gbx_oracle.c)
// and generates the golden vectors under tests/golden/.
//
// It fills a reference `struct Arguments` the way the reference CLI does
// (01_host/src/main/GraphBlox.c:313-375: argumentsNew, then the flags, then
// `-k` forces sort=1), builds the graph with generateGraphDataStructure
// (01_host/src/utils_graph/graphRun.c:279), calls ONE algorithm entry point of
// the openmp integration directly, and writes the CSR arrays and the stats
// arrays as raw little-endian files into an output directory:
//
//   csr_V.txt ... scalars as "key value" lines (scalars.txt)
//   out_degree.u32, edges_idx.u32, dest.u32, src.u32, weight.f32,
//   label.u32, inverse_label.u32 (+ inv_* for the inverse CSR when DIRECTED)
//   bfs_distances.u32, bfs_parents.i32, pr_ranks.f32, sssp_distances.u32,
//   cc_components.u32, spmv_y.f32, spmv_x.f32
//
// Usage: gbx_ref_<variant> FILE OUTDIR [flags]
//   -a ALG  (0 bfs, 1 pr, 2 sssp, 5 spmv, 6 cc, 8 tc, -1 csr only)
//   -p PP   pushpull variant        -s symmetric      -k dedup (+sort 1)
//   -w      weighted .wbin input    -o SORT           -l LMODE
//   -r ROOT -i ITERS -e EPS -b DELTA -n THREADS
//   -W      also write the reference's binary CSR file (graph.csr)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <string>
#include <omp.h>

extern "C" {
#include "graphConfig.h"
#include "graphCSR.h"
#include "graphRun.h"
#include "BFS.h"
#include "pageRank.h"
#include "SSSP.h"
#include "connectedComponents.h"
#include "triangleCount.h"
#include "bellmanFord.h"
#include "DFS.h"
#include "betweennessCentrality.h"
#include "SPMV.h"
}

static void dump(const std::string &dir, const char *name, const void *p, size_t bytes) {
    std::string path = dir + "/" + name;
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(2); }
    if (bytes && std::fwrite(p, 1, bytes, f) != bytes) { std::perror("fwrite"); std::exit(2); }
    std::fclose(f);
}

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s FILE OUTDIR [flags]\n", argv[0]);
        return 2;
    }
    struct Arguments *a = argumentsNew();
    a->fnameb = strdup(argv[1]);
    std::string out = argv[2];
    int alg = -1;
    int threads = omp_get_max_threads();
    bool write_csr = false;
    for (int i = 3; i < argc; ++i) {
        std::string f = argv[i];
        auto next = [&](void) -> const char * {
            if (i + 1 >= argc) { std::fprintf(stderr, "missing value for %s\n", f.c_str()); std::exit(2); }
            return argv[++i];
        };
        if (f == "-a") alg = std::atoi(next());
        else if (f == "-p") a->pushpull = (uint32_t)std::atoi(next());
        else if (f == "-s") a->symmetric = 1;
        else if (f == "-k") a->dflag = 1;
        else if (f == "-w") a->weighted = 1;
        else if (f == "-o") a->sort = (uint32_t)std::atoi(next());
        else if (f == "-l") a->lmode = (uint32_t)std::atoi(next());
        else if (f == "-r") a->source = (uint32_t)std::strtoul(next(), nullptr, 10);
        else if (f == "-i") a->iterations = (uint32_t)std::atoi(next());
        else if (f == "-e") a->epsilon = std::atof(next());
        else if (f == "-b") a->delta = (uint32_t)std::atoi(next());
        else if (f == "-n") threads = std::atoi(next());
        else if (f == "-W") write_csr = true;
        else if (f == "-M") a->mmode = (uint32_t)std::atoi(next());
        else if (f == "-C") a->cache_size = (uint32_t)std::strtoul(next(), nullptr, 10);
        else { std::fprintf(stderr, "unknown flag %s\n", f.c_str()); return 2; }
    }
    a->pre_numThreads = threads;
    a->algo_numThreads = threads;
    a->ker_numThreads = threads;
    a->algorithm = (uint32_t)(alg < 0 ? 0 : alg);
    if (a->dflag) a->sort = 1;  // GraphBlox.c:355-356

    struct GraphCSR *g = (struct GraphCSR *)generateGraphDataStructure(a);
    omp_set_num_threads(threads);

    // the reference's binary CSR file (writeToBinFileGraphCSR, graphCSR.c:458-529):
    // OUTDIR/graph.csr
    if (write_csr) writeToBinFileGraphCSR((out + "/graph").c_str(), g);

    FILE *sc = std::fopen((out + "/scalars.txt").c_str(), "w");
    if (!sc) { std::perror("scalars"); return 2; }
    const uint32_t V = g->num_vertices, E = g->num_edges;
    std::fprintf(sc, "num_vertices %u\nnum_edges %u\navg_degree %u\n", V, E, g->avg_degree);
    std::fprintf(sc, "directed %d\nweighted %d\n", DIRECTED, WEIGHTED);
    dump(out, "out_degree.u32", g->vertices->out_degree, V * 4ull);
    dump(out, "edges_idx.u32", g->vertices->edges_idx, V * 4ull);
    dump(out, "dest.u32", g->sorted_edges_array->edges_array_dest, E * 4ull);
    dump(out, "src.u32", g->sorted_edges_array->edges_array_src, E * 4ull);
    dump(out, "label.u32", g->sorted_edges_array->label_array, V * 4ull);
    dump(out, "inverse_label.u32", g->sorted_edges_array->inverse_label_array, V * 4ull);
    // hot/warm/lukewarm/cold hints of mask mode (maskGraphProcess, reorder.c:1164-1475)
    if (a->mmode && g->sorted_edges_array->mask_array)
        dump(out, "mask.u32", g->sorted_edges_array->mask_array, V * 4ull);
#if WEIGHTED
    dump(out, "weight.f32", g->sorted_edges_array->edges_array_weight, E * 4ull);
#endif
#if DIRECTED
    dump(out, "inv_out_degree.u32", g->inverse_vertices->out_degree, V * 4ull);
    dump(out, "inv_edges_idx.u32", g->inverse_vertices->edges_idx, V * 4ull);
    dump(out, "inv_dest.u32", g->inverse_sorted_edges_array->edges_array_dest, E * 4ull);
#if WEIGHTED
    dump(out, "inv_weight.f32", g->inverse_sorted_edges_array->edges_array_weight, E * 4ull);
#endif
#endif

    switch (alg) {
    case 0: {
        struct BFSStats *s = breadthFirstSearchGraphCSR(a, g);
        std::fprintf(sc, "source %u\nprocessed_nodes %u\niteration %u\ntime_total %.9f\n",
                     a->source, s->processed_nodes, s->iteration, s->time_total);
        dump(out, "bfs_distances.u32", s->distances, V * 4ull);
        dump(out, "bfs_parents.i32", s->parents, V * 4ull);
        freeBFSStats(s);
    } break;
    case 1: {
        struct PageRankStats *s = pageRankGraphCSR(a, g);
        std::fprintf(sc, "iterations %u\nerror_total %.17g\ntime_total %.9f\n",
                     s->iterations, s->error_total, s->time_total);
        dump(out, "pr_ranks.f32", s->pageRanks, V * 4ull);
        freePageRankStats(s);
    } break;
    case 2: {
        struct SSSPStats *s = SSSPGraphCSR(a, g);
        std::fprintf(sc, "source %u\nprocessed_nodes %u\ntime_total %.9f\n",
                     a->source, s->processed_nodes, s->time_total);
        dump(out, "sssp_distances.u32", s->distances, V * 4ull);
        freeSSSPStats(s);
    } break;
    case 3: {
        struct BellmanFordStats *s = bellmanFordGraphCSR(a, g);
        std::fprintf(sc, "source %u\nprocessed_nodes %u\ntime_total %.9f\n",
                     a->source, s->processed_nodes, s->time_total);
        dump(out, "bf_distances.u32", s->distances, V * 4ull);
        dump(out, "bf_parents.u32", s->parents, V * 4ull);
        freeBellmanFordStats(s);
    } break;
    case 4: {
        struct DFSStats *s = depthFirstSearchGraphCSR(a, g);
        std::fprintf(sc, "source %u\nprocessed_nodes %u\ntime_total %.9f\n",
                     a->source, s->processed_nodes, s->time_total);
        dump(out, "dfs_distances.u32", s->distances, V * 4ull);
        dump(out, "dfs_parents.i32", s->parents, V * 4ull);
        freeDFSStats(s);
    } break;
    case 7: {
        // the roots Brandes will draw, from a copy of the generator state
        mt19937state rng = a->mt19937var;
        uint32_t *roots = (uint32_t *)std::malloc((a->iterations + 1) * 4ull);
        for (uint32_t i = 0; i < a->iterations; ++i)
            roots[i] = generateRandomRootBetweennessCentrality(&rng, g);
        dump(out, "bc_roots.u32", roots, a->iterations * 4ull);
        std::free(roots);
        struct BetweennessCentralityStats *s = betweennessCentralityGraphCSR(a, g);
        std::fprintf(sc, "iteration %u\nprocessed_nodes %u\ntime_total %.9f\n",
                     s->iteration, s->processed_nodes, s->time_total);
        dump(out, "bc_centrality.f32", s->betweennessCentrality, V * 4ull);
        dump(out, "bc_distances.u32", s->distances, V * 4ull);
        dump(out, "bc_sigma.i32", s->sigma, V * 4ull);
        dump(out, "bc_dependency.f32", s->dependency, V * 4ull);
        freeBetweennessCentralityStats(s);
    } break;
    case 5: {
        struct SPMVStats *s = SPMVGraphCSR(a, g);
        std::fprintf(sc, "iterations %u\ntime_total %.9f\n", s->iterations, s->time_total);
        dump(out, "spmv_y.f32", s->vector_output, V * 4ull);
        dump(out, "spmv_x.f32", s->vector_input, V * 4ull);
        freeSPMVStats(s);
    } break;
    case 6: {
        struct CCStats *s = connectedComponentsGraphCSR(a, g);
        std::fprintf(sc, "iterations %u\ntime_total %.9f\n", s->iterations, s->time_total);
        dump(out, "cc_components.u32", s->components, V * 4ull);
        freeCCStats(s);
    } break;
    case 8: {
        struct TCStats *s = triangleCountGraphCSR(a, g);
        std::fprintf(sc, "total_counts %llu\ntime_total %.9f\n",
                     (unsigned long long)s->total_counts, s->time_total);
        freeTCStats(s);
    } break;
    default:
        break;
    }
    std::fclose(sc);
    return 0;
}
