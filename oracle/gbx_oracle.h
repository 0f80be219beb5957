/*
 * gbx_oracle.h -- CPU restatement of the GraphBlox OpenMP host algorithms.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE. Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load liboracle.so, and only as the checker
 * or as the timed CPU baseline; nothing in graphblox_gb300/ links it.
 *
 * Parity is pinned two ways (tests/test_oracle_*.py):
 *   - against the reference host itself, compiled from its sources by
 *     oracle/build_ref.sh into oracle/_ref/ and run on identical inputs;
 *   - against the golden vectors committed under tests/golden/ (the
 *     reference's 03_data/TEST CSR dumps and outputs of oracle/_ref).
 *
 * Conventions follow the reference's GraphCSR (01_host/include/structures/
 * graphCSR.h:14-31): per-vertex edges_idx[] and out_degree[] over a
 * (src,dst)-sorted uint32 dest[] array, optional float weights. A "pull"
 * CSR is the inverse CSR when the graph is directed, or the forward CSR
 * itself for the reference's DIRECTED 0 build (valid on symmetric graphs).
 * All functions take num_threads (<=0 means the OpenMP default).
 */
#ifndef GBX_ORACLE_H
#define GBX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- edge list -> CSR ------------------------------------------------- */
/* Stable sort of (src,dst[,w]) by source (sort_mode 0/2) or by
 * (source,destination) (sort_mode 1/3), like radixsort.c:231-339 /
 * countsort.c:28-270. Sorts in place. */
void orc_sort_edges(uint32_t num_edges, uint32_t *src, uint32_t *dst, float *w,
                    int sort_mode, int num_threads);
/* removeDulpicatesSelfLoopEdges (edgeList.c:255-321) on a (src,dst)-sorted
 * list: drops self loops and adjacent duplicates, keeps the first weight
 * truncated through uint32 as the reference does. Returns the new count. */
uint32_t orc_dedup_edges(uint32_t num_edges, uint32_t *src, uint32_t *dst, float *w);
/* mapVerticesWithInOutDegree_base (vertex.c:204-328): out_degree[v] and
 * edges_idx[v] (first position of v, 0 when v has no edges). */
void orc_map_vertices(uint32_t num_vertices, uint32_t num_edges, const uint32_t *src,
                      uint32_t *out_degree, uint32_t *edges_idx);

/* ---- degree reordering (reorder.c:275-380, :1483-1552, :1618-1637) ----- */
/* lmode 1 out-degree, 2 in-degree, 3 in+out. Writes labels[old]=new and
 * inverse_labels[new]=old (identity label arrays on entry, as after
 * readEdgeListsbin). Relabels src/dst in place. */
void orc_degree_reorder(uint32_t num_vertices, uint32_t num_edges, uint32_t *src, uint32_t *dst,
                        int lmode, uint32_t *labels, uint32_t *inverse_labels, int num_threads);

/* ---- mask mode (maskGraphProcess, reorder.c:1164-1475) ------------------ */
void orc_mask_graph(uint32_t num_vertices, uint32_t num_edges, uint32_t *src, uint32_t *dst,
                    int mmode, uint32_t cache_size, uint32_t *mask);

/* ---- BFS (BFS.c:42-78, :335-613) -------------------------------------- */
/* Direction-optimising BFS (alpha 15, beta 18). distances: level, 0 for
 * the source and for unreached vertices; parents: -out_degree (or -1) for
 * unreached, the source for itself, a BFS parent otherwise. */
void orc_bfs(uint32_t num_vertices, uint32_t num_edges,
             const uint32_t *out_degree, const uint32_t *edges_idx, const uint32_t *dest,
             const uint32_t *pull_degree, const uint32_t *pull_idx, const uint32_t *pull_src,
             uint32_t source, uint32_t *distances, int32_t *parents,
             uint32_t *processed_nodes, uint32_t *iterations, int num_threads);

/* ---- PageRank pull (pageRank.c:47-75, :245-368) ----------------------- */
/* FP32 recurrence in the reference's operation order (per-vertex sum in
 * edge order), so the result is bit-identical to the reference's. */
void orc_pagerank_pull(uint32_t num_vertices, const uint32_t *out_degree,
                       const uint32_t *pull_degree, const uint32_t *pull_idx, const uint32_t *pull_src,
                       uint32_t max_iterations, double epsilon, float *ranks,
                       uint32_t *iterations, double *error_total, int num_threads);
/* Same recurrence entirely in FP64 (the 1e-6 relative-L1 yardstick). */
void orc_pagerank_pull_f64(uint32_t num_vertices, const uint32_t *out_degree,
                           const uint32_t *pull_degree, const uint32_t *pull_idx, const uint32_t *pull_src,
                           uint32_t max_iterations, double epsilon, double *ranks,
                           uint32_t *iterations, int num_threads);

/* ---- SSSP (SSSP.c:76-105, :514-653) ----------------------------------- */
/* Shortest distances with the reference's relaxation arithmetic
 * newDistance = (uint32_t)((float)d + w) (SSSP.c:204,262); weights NULL
 * means weight 1 (WEIGHTED 0). Unreached = UINT_MAX/2. Deterministic
 * (bucketed label-correcting with delta). */
void orc_sssp(uint32_t num_vertices, const uint32_t *out_degree, const uint32_t *edges_idx,
              const uint32_t *dest, const float *weights, uint32_t source, uint32_t delta,
              uint32_t *distances, uint32_t *processed_nodes, int num_threads);

/* ---- connected components (connectedComponents.c:177-629) ------------- */
/* variant 0 Shiloach-Vishkin, 1 Afforest, 2 label propagation. All give
 * components[v] = smallest vertex id of v's component. For directed
 * graphs pass the inverse CSR too (pull_* may be NULL). */
void orc_cc(uint32_t num_vertices, const uint32_t *out_degree, const uint32_t *edges_idx,
            const uint32_t *dest, const uint32_t *pull_degree, const uint32_t *pull_idx,
            const uint32_t *pull_src, int variant, uint32_t *components,
            uint32_t *iterations, int num_threads);

/* ---- triangle count (triangleCount.c:254-334) ------------------------- */
/* Pull semantics on a (src,dst)-sorted CSR: sum over edges u->v with
 * v <= u, over w in N(v) with w <= v, of [w in N(u)]. */
uint64_t orc_triangle_count(uint32_t num_vertices, const uint32_t *out_degree,
                            const uint32_t *edges_idx, const uint32_t *dest, int num_threads);

/* ---- SpMV pull (SPMV.c:117-215) --------------------------------------- */
/* y[v] += sum_j w_j * x[src_j] over the pull CSR, repeated `iterations`
 * times (y is never reset, as in the reference). weights NULL means the
 * reference's constant 0.0001f. */
void orc_spmv_pull(uint32_t num_vertices, const uint32_t *pull_degree, const uint32_t *pull_idx,
                   const uint32_t *pull_src, const float *weights, float default_weight,
                   const float *x, float *y, uint32_t iterations, int num_threads);
void orc_spmv_pull_f64(uint32_t num_vertices, const uint32_t *pull_degree, const uint32_t *pull_idx,
                       const uint32_t *pull_src, const float *weights, float default_weight,
                       const float *x, double *y, uint32_t iterations, int num_threads);

/* ---- random roots (mt19937.c, betweennessCentrality.c:172-189) -------- */
void orc_random_roots(uint32_t seed, uint32_t n, uint32_t num_vertices, const uint32_t *out_degree,
                      uint32_t avg_degree, uint32_t *roots);

/* ---- betweenness centrality (betweennessCentrality.c:230-466) ---------- */
void orc_betweenness(uint32_t num_vertices, const uint32_t *pull_degree, const uint32_t *pull_idx,
                     const uint32_t *pull_src, uint32_t num_roots, const uint32_t *roots, float *bc,
                     uint32_t *distances, int32_t *sigma, float *dependency, uint32_t *processed_nodes);

/* ---- depth-first search (DFS.c:156-205) -------------------------------- */
void orc_dfs(uint32_t num_vertices, const uint32_t *out_degree, const uint32_t *edges_idx,
             const uint32_t *dest, uint32_t source, uint32_t *distances, int32_t *parents,
             uint32_t *processed_nodes);

/* ---- synthetic inputs (no reference counterpart) ----------------------
 * The same counter-based streams as the library's generators (every edge or
 * value drawn from a stream keyed by (seed, index)), so the CPU side builds
 * the benchmark's inputs without the GPU library: RMAT edges with quadrant
 * probabilities a, b, c (d = 1-a-b-c), and values of `kind` 0 (integers in
 * [lo, hi]), 1 (uniform (0, 1]), 2 (uniform [-1, 1)), 3 (lognormal(0, 1)). */
int orc_generate_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c, uint64_t seed,
                      uint32_t *src, uint32_t *dst);
int orc_generate_values(uint64_t count, int kind, uint32_t lo, uint32_t hi, uint64_t seed, float *out);

/* Triangles whose largest vertex u lies in [lo, hi) (the pull count of
 * orc_triangle_count restricted to those pivots): the counts of a partition
 * of [0, V) sum to the whole count. */
uint64_t orc_triangle_count_range(uint32_t num_vertices, const uint32_t *out_degree,
                                  const uint32_t *edges_idx, const uint32_t *dest, uint32_t lo,
                                  uint32_t hi, int num_threads);

/* ---- CSR segments (csrSegments.c:157-578) --------------------------------
 * csrSegmentsCalculateSegments and the partition csrSegmentsNew computes
 * before its per-segment preprocessing: degrees, the segment of every
 * destination, per-segment edge counts and largest ids, and the edges
 * grouped by the segment of their destination in input order (the order
 * the reference's population loop gives with one thread). */
uint32_t orc_csr_segments_count(uint32_t num_vertices, uint32_t cache_size);
void orc_csr_segments(uint32_t num_edges, const uint32_t *src, const uint32_t *dst, const float *w,
                      uint32_t num_vertices, uint32_t num_segments, uint32_t *out_degree, uint32_t *in_degree,
                      uint32_t *vertex_segment_index, uint32_t *segment_num_edges, uint32_t *segment_max_id,
                      uint32_t *seg_src, uint32_t *seg_dst, float *seg_w);

#ifdef __cplusplus
}
#endif
#endif
