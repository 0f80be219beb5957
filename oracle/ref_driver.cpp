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
//   -a ALG  (0 bfs, 1 pr, 2 sssp, 5 spmv, 6 cc, 8 tc, -1 csr only,
//            100 CSR segments: see dump_segments)
//   -p PP   pushpull variant        -s symmetric      -k dedup (+sort 1)
//   -w      weighted .wbin input    -o SORT           -l LMODE
//   -r ROOT -i ITERS -e EPS -b DELTA -n THREADS
//   -W      also write the reference's binary CSR file (graph.csr)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <string>
#include <vector>
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
#include "csrSegments.h"
#include "edgeList.h"
#include "sortRun.h"
#include "reorder.h"
#include "myMalloc.h"
}

static void dump(const std::string &dir, const char *name, const void *p, size_t bytes) {
    std::string path = dir + "/" + name;
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(2); }
    if (bytes && std::fwrite(p, 1, bytes, f) != bytes) { std::perror("fwrite"); std::exit(2); }
    std::fclose(f);
}

// CSR segments, the reference's own functions in the order csrSegmentsNew
// (csrSegments.c:157-240) calls them, on the edge list that
// graphCSRSegmentsPreProcessingStep (graphCSRSegments.c:134-194) prepares.
// The last step of csrSegmentsNew, csrSegmentsCreationPreprocessing, builds a
// GraphCSR per segment from an edge list whose num_vertices is the segment's
// largest id (csrSegmentsSegmentVertexSizePreprocessing), one short of the
// arrays that id needs; here each segment's edge list gets largest id + 1
// vertices (identity labels) before the same per-segment preprocessing
// (argumentsNew defaults with lmode 1, as csrSegmentsCreationPreprocessing
// sets them), so the dump is well defined. Dumped (concatenated over
// segments): seg_* partition arrays, segcsr_* per-segment CSR arrays.
static int dump_segments(struct Arguments *a, const std::string &out) {
    struct EdgeList *el = readEdgeListsbin(a->fnameb, 0, a->symmetric, a->weighted);
    el = sortRunAlgorithms(el, a->sort);
    if (a->dflag) el = removeDulpicatesSelfLoopEdges(el);
    if (a->lmode) {
        el = reorderGraphProcess(el, a);
        el = sortRunAlgorithms(el, a->sort);
    }
    struct CSRSegments *cs = (struct CSRSegments *)std::calloc(1, sizeof(struct CSRSegments));
    cs->num_edges = el->num_edges;
    cs->num_vertices = el->num_vertices;
    cs->num_segments = csrSegmentsCalculateSegments(el, a->cache_size);
    const uint32_t S = cs->num_segments, V = cs->num_vertices, E = cs->num_edges;
    cs->segments = (struct Segment *)std::calloc(S, sizeof(struct Segment));
    cs->activeSegments = (uint32_t *)std::calloc(S, 4);
    cs->out_degree = (uint32_t *)std::calloc(V + 1, 4);
    cs->in_degree = (uint32_t *)std::calloc(V + 1, 4);
    cs->vertex_segment_index = (uint32_t *)std::calloc(V + 1, 4);
    graphCSRSegmentsProcessInOutDegrees(cs, el);
    csrSegmentsSegmentEdgeListSizePreprocessing(cs, el);
    csrSegmentsSegmentsMemoryAllocations(cs);
    csrSegmentsSegmentEdgePopulation(cs, el);
    csrSegmentsSegmentVertexSizePreprocessing(cs);
    FILE *sc = std::fopen((out + "/scalars.txt").c_str(), "w");
    if (!sc) { std::perror("scalars"); return 2; }
    std::fprintf(sc, "num_vertices %u\nnum_edges %u\nnum_segments %u\n", V, E, S);
    std::fclose(sc);
    dump(out, "seg_out_degree.u32", cs->out_degree, V * 4ull);
    dump(out, "seg_in_degree.u32", cs->in_degree, V * 4ull);
    dump(out, "seg_vertex_index.u32", cs->vertex_segment_index, V * 4ull);
    std::string ne, nv, ssrc, sdst, sw, cdeg, cidx, cdst, clab, cilab, cnv;
    std::vector<uint32_t> seg_ne(S), seg_nv(S), csr_nv;
    std::vector<uint32_t> all_src, all_dst, c_deg, c_idx, c_dst, c_lab, c_ilab;
    std::vector<float> all_w;
    for (uint32_t j = 0; j < S; ++j) {
        struct Segment &sg = cs->segments[j];
        seg_ne[j] = sg.num_edges;
        seg_nv[j] = sg.num_vertices;
        if (!sg.num_edges) continue;
        struct EdgeList *se = sg.edgeList;
        all_src.insert(all_src.end(), se->edges_array_src, se->edges_array_src + se->num_edges);
        all_dst.insert(all_dst.end(), se->edges_array_dest, se->edges_array_dest + se->num_edges);
        all_w.insert(all_w.end(), se->edges_array_weight, se->edges_array_weight + se->num_edges);
        // one more vertex than the largest id, identity labels
        const uint32_t nvs = se->num_vertices + 1;
        se->num_vertices = nvs;
        se->mask_array = (uint32_t *)std::calloc(nvs, 4);
        se->label_array = (uint32_t *)std::malloc(nvs * 4ull);
        se->inverse_label_array = (uint32_t *)std::malloc(nvs * 4ull);
        for (uint32_t i = 0; i < nvs; ++i) se->label_array[i] = se->inverse_label_array[i] = i;
        se->avg_degree = se->num_edges / nvs;
        struct Arguments *al = argumentsNew();
        al->lmode = 1;
        al->pre_numThreads = a->pre_numThreads;
        struct GraphCSR *gs = graphCSRPreProcessingStepFromEdgelist(al, se);
        csr_nv.push_back(gs->num_vertices);
        c_deg.insert(c_deg.end(), gs->vertices->out_degree, gs->vertices->out_degree + gs->num_vertices);
        c_idx.insert(c_idx.end(), gs->vertices->edges_idx, gs->vertices->edges_idx + gs->num_vertices);
        c_dst.insert(c_dst.end(), gs->sorted_edges_array->edges_array_dest,
                     gs->sorted_edges_array->edges_array_dest + gs->num_edges);
        c_lab.insert(c_lab.end(), gs->sorted_edges_array->label_array,
                     gs->sorted_edges_array->label_array + gs->num_vertices);
        c_ilab.insert(c_ilab.end(), gs->sorted_edges_array->inverse_label_array,
                      gs->sorted_edges_array->inverse_label_array + gs->num_vertices);
    }
    dump(out, "seg_num_edges.u32", seg_ne.data(), S * 4ull);
    dump(out, "seg_num_vertices.u32", seg_nv.data(), S * 4ull);
    dump(out, "seg_src.u32", all_src.data(), all_src.size() * 4ull);
    dump(out, "seg_dst.u32", all_dst.data(), all_dst.size() * 4ull);
    if (a->weighted) dump(out, "seg_weight.f32", all_w.data(), all_w.size() * 4ull);
    dump(out, "segcsr_num_vertices.u32", csr_nv.data(), csr_nv.size() * 4ull);
    dump(out, "segcsr_out_degree.u32", c_deg.data(), c_deg.size() * 4ull);
    dump(out, "segcsr_edges_idx.u32", c_idx.data(), c_idx.size() * 4ull);
    dump(out, "segcsr_dest.u32", c_dst.data(), c_dst.size() * 4ull);
    dump(out, "segcsr_label.u32", c_lab.data(), c_lab.size() * 4ull);
    dump(out, "segcsr_inverse_label.u32", c_ilab.data(), c_ilab.size() * 4ull);
    return 0;
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
    if (alg == 100) {
        omp_set_num_threads(threads);
        return dump_segments(a, out);
    }

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
