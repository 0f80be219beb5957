/*
 * gbx.h -- C ABI of libgbx.so, the GB300 (sm_103a) backend for GraphBlox's
 * vertex-centric CSR kernels.
 *
 * Two layers sit on this ABI:
 *   - the drop-in "cuda" integration (the C files in
 *     graphblox_gb300/integration/, headers in include/algorithms/cuda/),
 *     which exports the same symbols
 *     and Stats structs as the reference's 01_host/include/algorithms/openmp
 *     headers so that 01_host/src/utils_graph/graphRun.c links unchanged;
 *   - the Python host mirror (graphblox_gb300/), which binds it with ctypes.
 *
 * Conventions
 *   - Plain pointers and sizes only. Every array argument may be host memory
 *     (pageable or pinned) or device memory of the current device; the
 *     library detects which and copies as needed.
 *   - Every function returns an int status: GBX_OK (0) or a negative
 *     GBX_ERR_* code. gbx_last_error() gives a message for the calling thread.
 *   - `stream` is a cudaStream_t (NULL = the legacy default stream). Entry
 *     points that return results into host memory synchronize that stream
 *     before returning; results into device memory are stream-ordered.
 *   - Vertex ids are uint32 (the reference's limit is 2^30, EXTRACT_VALUE in
 *     01_host/include/preprocess/reorder.h:23). Edge counts are uint32 in the
 *     reference-compatible entry points, as in struct GraphCSR.
 *   - No entry point falls back to the CPU: without a usable GPU every
 *     compute call fails with GBX_ERR_NO_DEVICE.
 *
 * Reference interfaces replaced (paths within the GraphBlox project):
 *   gbx_graph_create_csr      -> the device copy of struct GraphCSR
 *                                (01_host/include/structures/graphCSR.h:14-31)
 *   gbx_bfs                   -> breadthFirstSearchGraphCSR (01_host/src/algorithms/openmp/BFS.c:103-127)
 *   gbx_pagerank_pull         -> pageRankPullGraphCSR (01_host/src/algorithms/openmp/pageRank.c:245-368)
 *   gbx_sssp                  -> SSSPGraphCSR (01_host/src/algorithms/openmp/SSSP.c:489-653)
 *   gbx_cc                    -> connectedComponentsGraphCSR (01_host/src/algorithms/openmp/connectedComponents.c:268-629)
 *   gbx_tc                    -> triangleCountGraphCSR (01_host/src/algorithms/openmp/triangleCount.c:158-334)
 *   gbx_spmv                  -> SPMVGraphCSR (01_host/src/algorithms/openmp/SPMV.c:89-215)
 *   gbx_csr_build             -> graphCSRPreProcessingStep's sort/dedup/map
 *                                (01_host/src/structures/graphCSR.c:243-327,
 *                                 radixsort.c:231-339, edgeList.c:255-321, vertex.c:204-328)
 *   gbx_degree_reorder        -> reorderGraphProcess (01_host/src/preprocess/reorder.c:1556-1614): degree
 *                                (:275-380), DBG (:387-572), HUBSort (:762-982), HUBCluster (:984-1170),
 *                                Corder (:574-624), degrees (:1483-1552), relabel (:1618-1637)
 *   gbx_relabel               -> relabelEdgeListFromFile's relabelling (01_host/src/preprocess/reorder.c:1662-1714)
 *   gbx_bellman_ford          -> bellmanFordGraphCSR (01_host/src/algorithms/openmp/bellmanFord.c:419-738)
 *   gbx_dfs                   -> depthFirstSearchGraphCSR (01_host/src/algorithms/openmp/DFS.c:156-205)
 *   gbx_betweenness           -> betweennessCentralityGraphCSR (01_host/src/algorithms/openmp/betweennessCentrality.c:230-466)
 *   gbx_mask_graph            -> maskGraphProcess (01_host/src/preprocess/reorder.c:1164-1475) and
 *                                maskEdgeList (:1639-1657), the -M mask mode
 * Extension entry points (batched, multi-source, personalised PageRank and
 * its adjoint, generators) have no reference counterpart.
 */
#ifndef GBX_H
#define GBX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ---------------------------------------------------------- */
#define GBX_OK 0
#define GBX_ERR_INVALID (-1)     /* bad argument (NULL, size, source out of range) */
#define GBX_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define GBX_ERR_NOMEM (-3)       /* device allocation failed */
#define GBX_ERR_ITER_CAP (-4)    /* an iteration cap was reached before convergence */
#define GBX_ERR_NO_DEVICE (-5)   /* no usable CUDA device */
#define GBX_ERR_UNSUPPORTED (-6) /* graph layout not supported by this entry point */
#define GBX_ERR_DEVICE_TIMEOUT (-7) /* a bounded device-side wait gave up */

const char *gbx_status_string(int status);
/* Message for the last failing call on this host thread ("" if none). */
const char *gbx_last_error(void);
/* Library version as "major.minor.patch". */
const char *gbx_version(void);
/* Select the device for subsequent calls on this thread (cudaSetDevice). */
int gbx_set_device(int device);
/* Number of kernels this process has launched through the library. */
uint64_t gbx_kernel_launches(void);

/* ---- device-resident graph ------------------------------------------- */
typedef struct gbx_graph gbx_graph;

/* Copy a CSR in the reference's layout to the device.
 *   edges_idx[v], out_degree[v]: first edge position and degree of v (the
 *     reference's struct Vertex, vertex.h:17-23; edges_idx is 0 for
 *     degree-0 vertices). The edges of v are the run dest[edges_idx[v] ..
 *     +out_degree[v]). Runs in vertex order (the reference's CSR build) are
 *     copied as they are; runs in any other order (the inverse CSR of a
 *     masked edge list, sorted on the masked ids) are gathered into vertex
 *     order on the device, keeping the order inside each run. A run that
 *     ends past num_edges is GBX_ERR_INVALID.
 *   dest[E], weight[E] (weight may be NULL).
 *   in_*: the inverse CSR (in-edges; the reference's DIRECTED 1 build), or
 *     all NULL. Pull-direction kernels use it when present, else they pull
 *     over the forward CSR (the reference's DIRECTED 0 behaviour).
 * The top two bits of ids (the reference's mask bits) are cleared. */
int gbx_graph_create_csr(gbx_graph **out, uint32_t num_vertices, uint32_t num_edges,
                         const uint32_t *edges_idx, const uint32_t *out_degree,
                         const uint32_t *dest, const float *weight,
                         const uint32_t *in_edges_idx, const uint32_t *in_degree,
                         const uint32_t *in_src, const float *in_weight, void *stream);
/* Same, from standard CSR offsets (num_vertices+1 entries). */
int gbx_graph_create_offsets(gbx_graph **out, uint32_t num_vertices, uint32_t num_edges,
                             const uint32_t *offsets, const uint32_t *dest, const float *weight,
                             const uint32_t *in_offsets, const uint32_t *in_src,
                             const float *in_weight, void *stream);
int gbx_graph_destroy(gbx_graph *g);
int gbx_graph_info(const gbx_graph *g, uint32_t *num_vertices, uint32_t *num_edges,
                   int *has_inverse, int *has_weights);
/* Device pointers of the resident arrays (for zero-copy use by callers). */
int gbx_graph_device_arrays(const gbx_graph *g, const uint32_t **offsets, const uint32_t **dest,
                            const float **weight, const uint32_t **in_offsets,
                            const uint32_t **in_src, const float **in_weight);

/* ---- tuning (no reference counterpart) ---------------------------------- */
/* Per-graph knobs: "bfs_alpha" (switch to bottom-up when the frontier's edges
 * exceed unexplored edges / alpha; the reference fixes 15), "bfs_beta" (stay
 * bottom-up while the frontier exceeds V / beta; 18), "sssp_delta" (bucket
 * width, 0 = default), "pull_heavy_min" (in-degree above which PR/SpMV cut a
 * row into CTA-sized chunks; 4096). SSSP distances never change; PR and SpMV
 * sums may change their FP32 summation order only. BFS results do not depend
 * on alpha/beta when the graph has an inverse CSR or is symmetric; without an
 * inverse CSR the reference pulls over out-edges, and on an asymmetric graph
 * its levels then follow the direction schedule (gbx_autotune does not touch
 * alpha/beta on such graphs). */
int gbx_graph_set_tuning(gbx_graph *g, const char *key, double value);
int gbx_graph_get_tuning(const gbx_graph *g, const char *key, double *value);
/* Time candidate settings on num_samples sources of this graph (CUDA
 * events) and keep the fastest: flags bit 0 BFS direction threshold (graphs
 * with an inverse CSR only), bit 1 SSSP bucket width, bit 2 the pull engine's
 * heavy-row threshold (timed on PageRank iterations). */
int gbx_autotune(gbx_graph *g, uint32_t flags, uint32_t num_samples, void *stream);

/* ---- BFS --------------------------------------------------------------- */
typedef struct gbx_bfs_result {
    uint32_t processed_nodes; /* vertices reached, source included (BFSStats.processed_nodes) */
    uint32_t iteration;       /* steps counted like BFSStats.iteration */
    uint32_t depth;           /* largest level */
    uint32_t top_down_steps;
    uint32_t bottom_up_steps;
    uint32_t reserved;
    uint64_t edges_traversed; /* sum of out-degrees of reached vertices (GTEPS numerator) */
} gbx_bfs_result;

/* Direction-optimising BFS (alpha 15, beta 18 as in BFS.c:374-375).
 * distances[v] = level (0 for the source and for unreached vertices, as the
 * reference reports), parents[v] = BFS parent, the source for itself, and
 * -out_degree[v] (or -1) for unreached vertices. parents may be NULL.
 * mode: 0 pull-only (bottom-up), 1 push-only (top-down), 2 direction-optimising. */
int gbx_bfs(gbx_graph *g, uint32_t source, int mode, uint32_t *distances, int32_t *parents,
            gbx_bfs_result *result, void *stream);

/* The BFS trials of the reference's benchmark loop (runGraphAlgorithms,
 * graphRun.c:463-595: one breadthFirstSearchGraphCSR per trial, each from a
 * new root): one gbx_bfs traversal per source, enqueued back to back on
 * `stream` with a single host synchronisation after the last. sources and
 * results are host arrays of num_sources entries; results[i] is what gbx_bfs
 * returns for sources[i]. distances / parents: NULL, or device or host
 * arrays; with out_stride 0 every trial writes the same V entries (the last
 * trial's levels and parents remain), with out_stride >= V trial i writes
 * entries [i * out_stride, i * out_stride + V). A host array is filled
 * through two device staging buffers: trial i's copy to the host overlaps
 * trial i+1's traversal (pinned host memory makes the copies asynchronous). */
int gbx_bfs_trials(gbx_graph *g, const uint32_t *sources, uint32_t num_sources, int mode,
                   uint32_t *distances, int32_t *parents, uint64_t out_stride, gbx_bfs_result *results,
                   void *stream);

/* ---- PageRank ----------------------------------------------------------- */
typedef struct gbx_pr_result {
    uint32_t iterations;  /* counted like PageRankStats.iterations */
    uint32_t active_last; /* vertices that still moved by >= epsilon */
    double error_total;   /* mean |delta| of the last iteration (FP64 reduction) */
} gbx_pr_result;

/* One top-down BFS step over a caller-held frontier: the reference's
 * topDownStepGraphCSR (BFS.c:498-546). For every frontier vertex v and edge
 * v -> u with parents[u] < 0 (unvisited: -out_degree or -1), u is claimed
 * by a compare-and-swap of that value to v (the winner among frontier
 * vertices is a race, as in the reference), distances[u] = distances[v] + 1,
 * u is appended to next (at most next_capacity entries; more is
 * GBX_ERR_INVALID) and mf grows by -parents_old[u]. parents and distances
 * (num_vertices each) are read and updated in place; *next_len gets the
 * next frontier's size. */
int gbx_bfs_top_down_step(gbx_graph *g, const uint32_t *frontier, uint32_t frontier_len, int32_t *parents,
                          uint32_t *distances, uint32_t *next, uint32_t next_capacity, uint32_t *next_len,
                          uint32_t *mf, void *stream);

/* One bottom-up BFS step: the reference's bottomUpStepGraphCSR
 * (BFS.c:562-613). Every vertex v with parents[v] < 0 takes as parent the
 * first pull in-neighbour u (inverse CSR when the graph has one) that is set
 * in bitmap_curr, with distances[v] = distances[u] + 1, and is OR-ed into
 * bitmap_next. Bitmaps hold (num_vertices + 31) / 32 words, bit v in word
 * v / 32 at position v % 32 (the reference's struct Bitmap bitarray).
 * *nf gets the number of vertices found. */
int gbx_bfs_bottom_up_step(gbx_graph *g, const uint32_t *bitmap_curr, uint32_t *bitmap_next, int32_t *parents,
                           uint32_t *distances, uint32_t *nf, void *stream);

/* Pull PageRank with the reference's recurrence (damping 0.85f, ranks start
 * at 1-d, dangling mass dropped, stop when no vertex moves by >= epsilon,
 * final ranks divided by N). epsilon = 0 runs exactly max_iterations. FP32
 * ranks; high-degree pull sums use compensated (Kahan) accumulation;
 * the convergence residual is reduced in FP64. */
int gbx_pagerank_pull(gbx_graph *g, uint32_t max_iterations, double epsilon, float *ranks,
                      gbx_pr_result *result, void *stream);

/* The pull PageRank recurrence of gbx_pagerank_pull evaluated in FP64 for
 * exactly `iterations` iterations (no early exit), final ranks divided by
 * N: the double-precision yardstick FP32 ranks are reported against on
 * graphs too large for a CPU restatement (pageRank.c:245-368). No
 * counterpart in the reference. ranks: num_vertices doubles. */
int gbx_pagerank_pull_fp64(gbx_graph *g, uint32_t iterations, double *ranks, void *stream);

/* Pull PageRank that allocates no memory. No counterpart in the reference.
 * For callers that cannot call cudaMalloc: hosts whose own allocator took all
 * device memory at start-up, and real-time hosts that must not grow the CUDA
 * heap while they run. The working memory is a fixed file-scope device array
 * (about 64 MiB per GPU that loads the library, held until exit), so
 * num_vertices <= 4,194,304 and max_iterations <= 1024; larger sizes fail
 * with GBX_ERR_INVALID. pull_offsets (num_vertices+1), pull_src, out_degree
 * and ranks must be device memory. The first call on a device looks up the
 * array's address. All calls share the
 * array: calls that overlap on the GPU race, so serialise them. A non-NULL
 * result is copied to the host and the stream synchronised before return.
 * Same recurrence and result as gbx_pagerank_pull. */
int gbx_pagerank_pull_noalloc(uint32_t num_vertices, const uint32_t *pull_offsets,
                              const uint32_t *pull_src, const uint32_t *out_degree,
                              uint32_t max_iterations, double epsilon, float *ranks,
                              gbx_pr_result *result, void *stream);

/* Multi-source BFS: num_sources (1..256) BFS runs on one graph in one
 * level-synchronous sweep over per-vertex source bitmasks. No counterpart in
 * the reference as a batch; per source the results equal gbx_bfs from that
 * source (BFS.c:103-127). distances is vertex-major, num_vertices *
 * num_sources entries: distances[v * num_sources + i] = level of v from
 * sources[i] (0 for the source itself and for unreached vertices). results
 * (may be NULL) has one entry per source; top_down_steps / bottom_up_steps
 * count the shared push / pull levels. Sources may repeat. */
int gbx_bfs_multisource(gbx_graph *g, uint32_t num_sources, const uint32_t *sources,
                        uint32_t *distances, gbx_bfs_result *results, void *stream);

/* ---- batches of graphs -----------------------------------------------------
 * No counterpart in the reference as a batch: every graph of a batch gets
 * the results gbx_bfs (mode 2) / gbx_pagerank_pull give it alone, i.e. the
 * reference's breadthFirstSearchGraphCSR (BFS.c:103-127) and
 * pageRankPullGraphCSR (pageRank.c:245-368) per graph, from one persistent
 * launch over a device work queue of whole graphs.
 * Packed back-to-back CSR of num_graphs graphs: graph g owns packed vertices
 * vertex_base[g] .. vertex_base[g+1]-1 (vertex_base[0] = 0, every graph has
 * at least one vertex); offsets (total V + 1) are global edge positions
 * (offsets[0] = 0); dest holds graph-local ids. in_offsets / in_src give the
 * in-edge CSR in the same packing (NULL: the forward CSR is its own
 * transpose, as for symmetric graphs). Inputs may be host or device memory;
 * they are copied and checked (GBX_ERR_INVALID for a decreasing offset or a
 * local id at or above its graph's vertex count). */
typedef struct gbx_batch gbx_batch;
int gbx_batch_create(gbx_batch **out, uint32_t num_graphs, const uint32_t *vertex_base,
                     const uint32_t *offsets, const uint32_t *dest, const uint32_t *in_offsets,
                     const uint32_t *in_src, void *stream);
int gbx_batch_destroy(gbx_batch *b);
int gbx_batch_info(const gbx_batch *b, uint32_t *num_graphs, uint32_t *num_vertices,
                   uint32_t *num_edges);
/* BFS of every graph from its graph-local sources[g]. distances and parents
 * (may be NULL) are packed like the vertices; results (may be NULL) has one
 * entry per graph. */
int gbx_bfs_batched(gbx_batch *b, const uint32_t *sources, uint32_t *distances, int32_t *parents,
                    gbx_bfs_result *results, void *stream);
/* Pull PageRank of every graph (ranks packed like the vertices, each graph's
 * ranks divided by its own vertex count); results (may be NULL) per graph. */
int gbx_pr_batched(gbx_batch *b, uint32_t max_iterations, double epsilon, float *ranks,
                   gbx_pr_result *results, void *stream);

/* ---- personalised PageRank and its adjoint -------------------------------
 * No counterpart in the reference (its PageRank, pageRank.c:245-368, is the
 * un-personalised pull recurrence). K teleport vectors at once:
 *   P[v,u] = w_e / s_u for forward edge e = (u -> v), s_u = sum of u's
 *            out-weights (a source with s_u = 0 drops its mass)
 *   R = (1-d) T + d P R          forward fixed point
 *   L = sum W .* R               loss (FP64 dot)
 *   Lam = W + d P^T Lam          adjoint fixed point at the converged R
 *   dL/dT = (1-d) Lam,  dL/dw_e = (d <Lam[v],R[u]> - sum_{e' of u} d <Lam[v'],R[u]> P_e') / s_u
 * T, R, W, Lam and dL/dT are [V][K] row-major FP32 blocks (K = 32, 64, 128
 * or 256); weights and dL/dw are in forward-CSR edge order. Both solves stop
 * when, over all columns, the largest L1 change of an iteration divided by
 * the L1 norm of the column's source term (T forward, W adjoint; norm 1 for
 * a zero column) is below tol, reduced in FP64. For teleport columns that
 * sum to 1 this is the plain L1 residual. GBX_ERR_ITER_CAP when
 * max_iterations is reached first (the outputs then hold the last iterate).
 * Arrays may be host or device memory; the first call on a graph builds and
 * caches its in-edge order. */
typedef struct gbx_ppr_result {
    uint32_t iterations;          /* forward sweeps */
    uint32_t adjoint_iterations;  /* adjoint sweeps */
    double residual;              /* forward: last relative max-column L1 change */
    double adjoint_residual;      /* adjoint: last relative max-column L1 change */
    double loss;                  /* adjoint: sum W .* R in FP64 */
} gbx_ppr_result;

int gbx_ppr_forward(gbx_graph *g, uint32_t K, const float *weights, const float *teleport,
                    double damping, double tol, uint32_t max_iterations, float *ranks,
                    gbx_ppr_result *result, void *stream);
/* grad_weights (E) and grad_teleport (V*K) may each be NULL to skip them. */
int gbx_ppr_adjoint(gbx_graph *g, uint32_t K, const float *weights, const float *ranks,
                    const float *loss_weights, double damping, double tol,
                    uint32_t max_iterations, float *grad_weights, float *grad_teleport,
                    gbx_ppr_result *result, void *stream);

/* ---- SSSP --------------------------------------------------------------- */
typedef struct gbx_sssp_result {
    uint32_t reached;        /* vertices with a finite distance */
    uint32_t rounds;         /* relaxation rounds */
    uint64_t edges_relaxed;  /* total edge relaxations performed */
    uint64_t edges_traversed;/* sum of out-degrees of reached vertices */
} gbx_sssp_result;

/* Single-source shortest paths with the reference's arithmetic
 * newDistance = (uint32)((float)d + w) (SSSP.c:204,262), weight 1 when the
 * graph has no weights. distances[v] = UINT32_MAX/2 when unreached.
 * delta: bucket width of the near/far schedule (0 = autotuned). */
int gbx_sssp(gbx_graph *g, uint32_t source, uint32_t delta, uint32_t *distances,
             gbx_sssp_result *result, void *stream);

/* Bellman-Ford: the reference's distances (its pull and push variants and
 * SSSP all reach the same fixpoint of (uint32)((float)d + w)), computed by
 * the SSSP engine; parents[v] = the smallest u with an edge u->v on a
 * shortest path (the reference keeps the last racing writer), the source
 * its own parent, UINT32_MAX when unreached. parents may be NULL. The
 * result counts the SSSP engine's work, not the reference's active-vertex
 * sum, which depends on its relaxation order. */
int gbx_bellman_ford(gbx_graph *g, uint32_t source, uint32_t *distances, uint32_t *parents,
                     gbx_sssp_result *result, void *stream);

/* ---- depth-first search ---------------------------------------------------- */
/* The reference's stack traversal over the forward CSR: pop v, push every
 * out-neighbour whose parent is still -1 (parent v, distance d[v] + 1), in
 * row order; the source is its own parent. Unreached vertices keep
 * distance 0 and parent -1; *processed_nodes = vertices popped. Each pop
 * depends on the previous ones, so one warp runs it (latency-bound). */
int gbx_dfs(gbx_graph *g, uint32_t source, uint32_t *distances, int32_t *parents,
            uint32_t *processed_nodes, void *stream);

/* ---- betweenness centrality ------------------------------------------------ */
typedef struct gbx_bc_result {
    uint32_t iteration;        /* roots processed */
    uint32_t processed_nodes;  /* last root: predecessor entries (DAG edges) */
    uint32_t levels;           /* last root: BFS levels */
} gbx_bc_result;

/* Brandes from each of roots[0..num_roots) in turn (the reference draws them
 * from its generator: out-degree above the average), ADDING each root's
 * dependency / 2 into centrality[V] (zero it for a fresh run, as the
 * reference's new stats are). Levels come from the pull CSR (inverse when
 * present), sigma is int32 (wrapping), and the dependency fold follows the
 * reference's order and rounding exactly, so centrality is bit-identical to
 * the reference's. distances (UINT32_MAX unreached), sigma and dependency
 * of the last root are written when not NULL. */
int gbx_betweenness(gbx_graph *g, uint32_t num_roots, const uint32_t *roots, float *centrality,
                    uint32_t *distances, int32_t *sigma, float *dependency, gbx_bc_result *result,
                    void *stream);
/* The n roots the reference's Brandes draws from a generator seeded with
 * seed (the reference seeds 27491095 and draws its trial roots from the same
 * stream, so a run that drew those first continues from a later state):
 * MT19937 values, kept when below num_vertices with an out-degree above
 * num_edges / num_vertices. Host computation; roots is host memory.
 * GBX_ERR_INVALID when no vertex qualifies. */
int gbx_reference_roots(gbx_graph *g, uint32_t seed, uint32_t n, uint32_t *roots);

/* ---- CSR segments ------------------------------------------------------
 * The reference's cache-blocked graph form (csrSegmentsNew,
 * csrSegments.c:157-578; graphCSRSegmentsNew, graphCSRSegments.c:100-131).
 * gbx_csr_segments_count is csrSegmentsCalculateSegments (:538-553):
 * ceil(8 num_vertices / cache_size), at least 4. gbx_csr_segments builds the
 * partition on the GPU: the vertex range cut as getSegmentID (:555-570)
 * cuts it, every edge in the segment of its destination. Outputs:
 * out_degree / in_degree (num_vertices, over all edges),
 * vertex_segment_index (num_vertices: the segment of every destination, 0
 * for vertices that are no destination), segment_num_edges and
 * segment_max_id (num_segments: edge count and largest id among the
 * segment's edge ends, the reference's per-segment num_vertices), and
 * seg_src / seg_dst / seg_weight (num_edges: the edges grouped by segment,
 * input order inside a segment; seg_weight may be NULL). Any array may be
 * host or device memory; edge ends outside [0, num_vertices) fail with
 * GBX_ERR_INVALID. */
uint32_t gbx_csr_segments_count(uint32_t num_vertices, uint32_t cache_size);
int gbx_csr_segments(uint32_t num_edges, const uint32_t *src, const uint32_t *dst, const float *weight,
                     uint32_t num_vertices, uint32_t num_segments, uint32_t *out_degree, uint32_t *in_degree,
                     uint32_t *vertex_segment_index, uint32_t *segment_num_edges, uint32_t *segment_max_id,
                     uint32_t *seg_src, uint32_t *seg_dst, float *seg_weight, void *stream);

/* One draw of the Mersenne Twister MT19937 (Matsumoto and Nishimura, 1998)
 * from a state laid out like the reference's mt19937state (624 unsigned long
 * words and the index; mt19937.h:58-62), which it advances in place: the
 * value the reference's generateRandInt (mt19937.c) returns from that state.
 * gbx_reference_roots and the drop-in betweenness draw with it. */
uint32_t gbx_mt19937_next(unsigned long *mt, int *mti);

/* ---- connected components ---------------------------------------------- */
/* components[v] = smallest vertex id in v's component. variant 0 SV-style
 * hooking sweeps, 1 Afforest (default), 2 label propagation. All variants
 * give identical labels. iterations may be NULL. */
int gbx_cc(gbx_graph *g, int variant, uint32_t *components, uint32_t *iterations, void *stream);

/* ---- triangle count ----------------------------------------------------- */
/* Count with the reference's pull semantics on a (src,dst)-sorted CSR:
 * sum over edges u->v with v <= u, over w in N(v) with w <= v, of
 * [w in N(u)]; on a symmetric, self-loop-free, deduplicated graph this is
 * the number of triangles. Run after gbx_degree_reorder it is the
 * degree-ordered DAG count. */
int gbx_tc(gbx_graph *g, uint64_t *total, void *stream);

/* ---- SpMV ----------------------------------------------------------------- */
/* y[v] += sum over pull edges (u->v) of w_uv * x[u], `iterations` times.
 * values: per-edge values in pull-CSR order; NULL uses the graph's weights
 * in that order, or default_value when the graph has none. */
int gbx_spmv(gbx_graph *g, const float *values, float default_value, const float *x, float *y,
             uint32_t iterations, void *stream);

/* ---- preprocessing -------------------------------------------------------- */
/* CSR build on the device from an edge list (the GraphCSR preprocessing
 * step): optional symmetrisation (appends every edge reversed), stable sort
 * by source (sort_mode 0) or by (source,destination) (sort_mode 1), then
 * optional removal of self loops and adjacent duplicates (dedup; requires
 * sort_mode 1, keeps the first weight truncated through uint32 as the
 * reference does). num_vertices = max id + 1 over the input. Ids may carry
 * the mask bits of gbx_mask_graph (top two bits): the vertex is the id
 * without them and the sort key the whole id, as in the reference's radix
 * sort, so the runs of such a CSR are not in vertex order.
 * Outputs (caller-allocated; capacity = 2*num_edges when symmetric):
 * out_degree[V], edges_idx[V], src_out[E'], dst_out[E'], w_out[E'] (may be
 * NULL), *num_edges_out = E'. */
int gbx_csr_build(uint32_t num_edges, const uint32_t *src, const uint32_t *dst, const float *w,
                  int symmetric, int dedup, int sort_mode, uint32_t num_vertices,
                  uint32_t *out_degree, uint32_t *edges_idx, uint32_t *src_out, uint32_t *dst_out,
                  float *w_out, uint32_t *num_edges_out, void *stream);

/* Reordering by the reference's lmode (its -l flag). Degrees: in-degree for
 * lmode 2, 5, 7, 9, in + out for 3, out-degree otherwise (12 and 13 both
 * count out-degrees, as the reference's degree routine does).
 *   1, 2, 3      stable ascending sort of (degree, id), new label of the i-th
 *                = N-1-i (highest degree first, larger id first on ties)
 *   4, 5, 12, 13 DBG (12/13: Corder, which runs the DBG routine in the
 *                reference): 11 buckets, thresholds t0 = avg <= 1 ? 1 :
 *                avg/2 (avg = E/V, integer), doubling, last UINT32_MAX;
 *                labels bucket by bucket from the highest, ids ascending
 *   6, 7         HUBSort: vertices above t0 sorted by degree as in mode 1,
 *                then the others in id order
 *   8, 9         HUBCluster: vertices above avg, then the others, both in
 *                id order
 * lmode 10 (random) is GBX_ERR_UNSUPPORTED: the reference draws per-thread
 * random keys, so its order depends on its thread count. lmode 11 (labels
 * from a file) is gbx_relabel. Composes labels[] and inverse_labels[] in
 * place (identity on a fresh graph) and relabels src/dst in place. The
 * caller re-sorts with gbx_csr_build, as the reference re-runs
 * sortRunAlgorithms. */
int gbx_degree_reorder(uint32_t num_vertices, uint32_t num_edges, uint32_t *src, uint32_t *dst,
                       int lmode, uint32_t *labels, uint32_t *inverse_labels, void *stream);
/* Relabel with explicit new labels (new_labels[v] = label of v; the
 * reference's lmode 11 reads them from a text file, one per line):
 * GBX_ERR_INVALID unless new_labels is a permutation of [0, num_vertices).
 * Relabels src/dst and composes labels[] / inverse_labels[] like
 * gbx_degree_reorder. */
int gbx_relabel(uint32_t num_vertices, uint32_t num_edges, uint32_t *src, uint32_t *dst,
                const uint32_t *new_labels, uint32_t *labels, uint32_t *inverse_labels, void *stream);
/* Mask mode (the reference's -M, run after the last sort): hot/cold hints
 * 0xC0000000 HOT, 0x80000000 WARM, 0x40000000 LUKEWARM, 0 COLD per vertex
 * into mask_array[V]. Degrees: in-degree for mmode 2, 4, in + out for 5, 6,
 * out-degree for 1, 3. Vertices in DBG order (11 buckets, t0 = avg <= 1 ?
 * 1 : avg/2, highest bucket first, ids ascending) fill the regions in turn;
 * with cs = cache_size / 4 (the reference's -C, default 32768) the regions
 * are V/4 HOT, V/4 WARM, V/4 LUKEWARM when V - cs < 2 cs, else cs*8, cs*32,
 * cs*128 (uint32 products); the rest are COLD. This is the reference's
 * assignment run by one thread (with several, its threads take the regions
 * concurrently and the hints depend on the schedule). mmode 1, 2 also OR the
 * hints into src/dst in place (every kernel of this library clears them);
 * 3-6 leave the edges unchanged. Ids must be below num_vertices on entry. */
int gbx_mask_graph(uint32_t num_vertices, uint32_t num_edges, uint32_t *src, uint32_t *dst,
                   int mmode, uint32_t cache_size, uint32_t *mask_array, void *stream);

/* ---- synthetic inputs (no reference counterpart) ------------------------ */
/* R-MAT edge list: 2^scale vertices, num_edges edges, quadrant
 * probabilities a, b, c (d = 1-a-b-c), counter-based RNG keyed by seed, so
 * the same seed gives the same edges on any host or thread count. Host
 * pointers only. */
int gbx_generate_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c,
                      uint64_t seed, uint32_t *src, uint32_t *dst);
/* Per-edge value streams keyed by (seed, edge index):
 * kind 0: integer weights uniform in [lo, hi] stored as float;
 * kind 1: uniform in (0, 1]; kind 2: uniform in [-1, 1]; kind 3: lognormal(0,1). */
int gbx_generate_values(uint64_t count, int kind, uint32_t lo, uint32_t hi, uint64_t seed, float *out);
/* Chung-Lu edge list generated on the GPU: vertex i has weight
 * (i + i0)^(-1/(exponent-1)) (i0 puts the largest expected degree near
 * sqrt(num_edges)); each edge's source is drawn by weight, its destination
 * with probability local_fraction uniformly inside the source's block of
 * `window` consecutive ids, otherwise by weight. Out-degrees follow a power
 * law with the given exponent and mean num_edges / num_vertices.
 * Counter-based streams keyed by (seed, edge index). src/dst may be host or
 * device memory (num_edges entries each, num_edges < 2^32). */
int gbx_generate_chung_lu(uint32_t num_vertices, uint64_t num_edges, double exponent, uint32_t window,
                          double local_fraction, uint64_t seed, uint32_t *src, uint32_t *dst,
                          void *stream);

#ifdef __cplusplus
}
#endif
#endif
