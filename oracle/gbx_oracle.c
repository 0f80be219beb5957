/*
 * gbx_oracle.c -- CPU restatement of the GraphBlox OpenMP host algorithms.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE: the checker for the CUDA path and
 * the timed CPU baseline ("port"). Built with -ffp-contract=off so that the
 * FP32 results do not depend on whether the host ISA has FMA (the reference
 * itself is compiled for x86-64, which has none in its base ISA).
 *
 * Each function cites the reference function whose behaviour it restates;
 * the declarations in gbx_oracle.h document the conventions.
 */
#include "gbx_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define ORC_INF (UINT_MAX / 2u)

static void set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) abort();
    return p;
}

/* ------------------------------------------------------------------------ */
/* edge list -> CSR                                                         */
/* ------------------------------------------------------------------------ */

/* One stable counting-sort pass keyed by key[] (values < nkeys). */
static void counting_pass(uint32_t n, const uint32_t *key, uint32_t nkeys,
                          const uint32_t *perm_in, uint32_t *perm_out) {
    uint32_t *cnt = (uint32_t *)calloc((size_t)nkeys + 1, sizeof(uint32_t));
    if (!cnt) abort();
    for (uint32_t i = 0; i < n; ++i) cnt[key[perm_in[i]] + 1]++;
    for (uint32_t k = 0; k < nkeys; ++k) cnt[k + 1] += cnt[k];
    for (uint32_t i = 0; i < n; ++i) perm_out[cnt[key[perm_in[i]]]++] = perm_in[i];
    free(cnt);
}

/* One stable LSD radix pass over (key, index) pairs: digit = key bits
 * [shift, shift + 11). Each thread counts and scatters a contiguous chunk,
 * and the chunks' offsets are laid out thread after thread within a digit,
 * so equal digits keep their input order. */
#define ORC_RADIX_BITS 11
#define ORC_RADIX (1u << ORC_RADIX_BITS)
static void radix_pass(uint32_t n, int shift, const uint64_t *kin, const uint32_t *iin, uint64_t *kout,
                       uint32_t *iout) {
    const int T = omp_get_max_threads();
    uint32_t *hist = (uint32_t *)calloc((size_t)T * ORC_RADIX, 4);
    if (!hist) abort();
    const uint32_t chunk = (uint32_t)(((uint64_t)n + T - 1) / T);
    #pragma omp parallel num_threads(T)
    {
        const int t = omp_get_thread_num();
        const uint32_t lo = (uint32_t)((uint64_t)t * chunk < n ? (uint64_t)t * chunk : n);
        const uint32_t hi = (uint32_t)((uint64_t)lo + chunk < n ? (uint64_t)lo + chunk : n);
        uint32_t *h = hist + (size_t)t * ORC_RADIX;
        for (uint32_t i = lo; i < hi; ++i) h[(kin[i] >> shift) & (ORC_RADIX - 1)]++;
        #pragma omp barrier
        #pragma omp single
        {
            uint32_t run = 0;
            for (uint32_t d = 0; d < ORC_RADIX; ++d)
                for (int u = 0; u < T; ++u) {
                    const uint32_t c = hist[(size_t)u * ORC_RADIX + d];
                    hist[(size_t)u * ORC_RADIX + d] = run;
                    run += c;
                }
        }
        for (uint32_t i = lo; i < hi; ++i) {
            const uint32_t pos = h[(kin[i] >> shift) & (ORC_RADIX - 1)]++;
            kout[pos] = kin[i];
            iout[pos] = iin[i];
        }
    }
    free(hist);
}

/* radixSortEdgesBySource / ...BySourceAndDestination (radixsort.c:231-339):
 * a stable sort by source (sort_mode 0/2) or by (source, destination)
 * (sort_mode 1/3) on the full 32-bit ids, as LSD radix passes over the
 * composite key (source << 32 | destination); edges with equal keys keep
 * their input order. */
void orc_sort_edges(uint32_t num_edges, uint32_t *src, uint32_t *dst, float *w,
                    int sort_mode, int num_threads) {
    set_threads(num_threads);
    if (num_edges == 0) return;
    const uint32_t n = num_edges;
    const int by_dst = sort_mode == 1 || sort_mode == 3;
    uint32_t maxs = 0, maxd = 0;
    #pragma omp parallel for reduction(max : maxs, maxd)
    for (uint32_t i = 0; i < n; ++i) {
        if (src[i] > maxs) maxs = src[i];
        if (dst[i] > maxd) maxd = dst[i];
    }
    uint64_t *k0 = (uint64_t *)xmalloc((size_t)n * 8), *k1 = (uint64_t *)xmalloc((size_t)n * 8);
    uint32_t *i0 = (uint32_t *)xmalloc((size_t)n * 4), *i1 = (uint32_t *)xmalloc((size_t)n * 4);
    #pragma omp parallel for
    for (uint32_t i = 0; i < n; ++i) {
        k0[i] = ((uint64_t)src[i] << 32) | (by_dst ? dst[i] : 0u);
        i0[i] = i;
    }
    int bits_d = 0, bits_s = 0;
    while (by_dst && bits_d < 32 && (maxd >> bits_d)) bits_d++;
    while (bits_s < 32 && (maxs >> bits_s)) bits_s++;
    for (int sh = 0; sh < bits_d; sh += ORC_RADIX_BITS) {
        radix_pass(n, sh, k0, i0, k1, i1);
        uint64_t *tk = k0; k0 = k1; k1 = tk;
        uint32_t *ti = i0; i0 = i1; i1 = ti;
    }
    for (int sh = 0; sh < bits_s; sh += ORC_RADIX_BITS) {
        radix_pass(n, 32 + sh, k0, i0, k1, i1);
        uint64_t *tk = k0; k0 = k1; k1 = tk;
        uint32_t *ti = i0; i0 = i1; i1 = ti;
    }
    /* apply the permutation i0 */
    uint32_t *t = (uint32_t *)k1;
    #pragma omp parallel for
    for (uint32_t i = 0; i < n; ++i) t[i] = dst[i0[i]];
    memcpy(dst, t, (size_t)n * 4);
    #pragma omp parallel for
    for (uint32_t i = 0; i < n; ++i) src[i] = (uint32_t)(k0[i] >> 32);
    if (w) {
        float *tw = (float *)k1;
        #pragma omp parallel for
        for (uint32_t i = 0; i < n; ++i) tw[i] = w[i0[i]];
        memcpy(w, tw, (size_t)n * 4);
    }
    free(k0);
    free(k1);
    free(i0);
    free(i1);
}

/* removeDulpicatesSelfLoopEdges (edgeList.c:255-321). The reference keeps
 * the weight in a uint32_t temporary, so kept weights are truncated to
 * integers; the leading run of self loops is skipped before the first kept
 * edge. An input made only of self loops yields zero edges here (the
 * reference reads past the end of its arrays in that case). */
uint32_t orc_dedup_edges(uint32_t num_edges, uint32_t *src, uint32_t *dst, float *w) {
    uint32_t i = 0, j = 0;
    while (i < num_edges && src[i] == dst[i]) ++i;
    if (i == num_edges) return 0;
    src[0] = src[i];
    dst[0] = dst[i];
    if (w) w[0] = (float)(uint32_t)w[i];
    j = 1;
    for (++i; i < num_edges; ++i) {
        if (src[i] == dst[i]) continue;
        if (src[j - 1] != src[i] || dst[j - 1] != dst[i]) {
            src[j] = src[i];
            dst[j] = dst[i];
            if (w) w[j] = (float)(uint32_t)w[i];
            ++j;
        }
    }
    return j;
}

void orc_map_vertices(uint32_t num_vertices, uint32_t num_edges, const uint32_t *src,
                      uint32_t *out_degree, uint32_t *edges_idx) {
    memset(out_degree, 0, (size_t)num_vertices * 4);
    memset(edges_idx, 0, (size_t)num_vertices * 4);
    for (uint32_t i = 0; i < num_edges; ++i) {
        uint32_t v = src[i] & 0x3FFFFFFFu; /* VERTEX_CACHE_MASK_U32, reorder.h */
        out_degree[v]++;
        if (i == 0 || src[i] != src[i - 1]) edges_idx[v] = i;
    }
}

/* ------------------------------------------------------------------------ */
/* degree reordering                                                        */
/* ------------------------------------------------------------------------ */

/* reorderGraphProcess (reorder.c:1556-1614) for the deterministic modes.
 *
 * Degrees (reorderGraphGenerateInOutDegrees, reorder.c:1483-1552): lmodes
 * 2, 5, 7, 9 count in-degrees, 3 in + out, every other mode (1, 4, 6, 8 and,
 * through the switch's default, 12 and 13) out-degrees.
 *
 * lmode 1-3 (reorderGraphListDegree, :296-380): stable ascending sort of
 * (degree, id); the i-th smallest gets label N-1-i, so the largest degree
 * gets label 0 and, within a degree, the larger old id the smaller label.
 *
 * Bucketed modes: thresholds t0 = avg <= 1 ? 1 : avg/2 (avg = E/V, uint32;
 * HUBCluster takes t0 = avg itself, :1001), t_i = 2 t_{i-1}, last =
 * UINT32_MAX; v goes to the first bucket with degree <= t_i. lmode 4, 5 (DBG, :387-572) and 12, 13 (Corder, whose
 * process function calls the DBG list routine, :574-624) use 11 buckets,
 * lmode 8, 9 (HUBCluster, :984-1170) two: labels are given bucket by bucket
 * from the highest, in ascending id order inside a bucket. lmode 6, 7
 * (HUBSort, :762-982), two buckets: the hot bucket's vertices (ascending
 * ids) are stably sorted by degree and labelled in reverse (hot size - 1 -
 * position), the cold ones follow in id order.
 *
 * Then label composition (:368-373) and relabelEdgeList (:1618-1637).
 * lmode 10 (random) draws from per-thread generators and depends on the
 * thread count, so it is not restated. */
static uint32_t reorder_buckets(int lmode) {
    switch (lmode) {
    case 4: case 5: case 12: case 13: return 11;
    case 6: case 7: case 8: case 9: return 2;
    default: return 0;
    }
}

void orc_degree_reorder(uint32_t num_vertices, uint32_t num_edges, uint32_t *src, uint32_t *dst,
                        int lmode, uint32_t *labels, uint32_t *inverse_labels, int num_threads) {
    set_threads(num_threads);
    uint32_t n = num_vertices;
    uint32_t *deg = (uint32_t *)calloc((size_t)n + 1, 4);
    if (!deg) abort();
    const int in = lmode == 2 || lmode == 5 || lmode == 7 || lmode == 9;
    for (uint32_t i = 0; i < num_edges; ++i) {
        if (in) deg[dst[i]]++;
        else if (lmode == 3) { deg[dst[i]]++; deg[src[i]]++; }
        else deg[src[i]]++;
    }
    uint32_t *newlab = (uint32_t *)xmalloc((size_t)n * 4 + 4);
    const uint32_t nb = reorder_buckets(lmode);
    if (nb == 0) {
        uint32_t maxdeg = 0;
        for (uint32_t v = 0; v < n; ++v) if (deg[v] > maxdeg) maxdeg = deg[v];
        uint32_t *ids = (uint32_t *)calloc((size_t)n + 1, 4);
        uint32_t *sorted = (uint32_t *)xmalloc((size_t)n * 4 + 4);
        if (!ids) abort();
        for (uint32_t v = 0; v < n; ++v) ids[v] = v;
        counting_pass(n, deg, maxdeg + 1, ids, sorted);
        for (uint32_t i = 0; i < n; ++i) newlab[sorted[i]] = n - 1 - i;
        free(sorted);
        free(ids);
    } else {
        uint32_t th[11];
        const uint32_t avg = n ? num_edges / n : 0;
        th[0] = (lmode == 8 || lmode == 9) ? avg : (avg <= 1 ? 1u : avg / 2);
        for (uint32_t i = 1; i + 1 < nb; ++i) th[i] = th[i - 1] * 2u;
        th[nb - 1] = 0xFFFFFFFFu;
        uint8_t *bk = (uint8_t *)xmalloc((size_t)n + 1);
        uint32_t size[11] = {0};
        for (uint32_t v = 0; v < n; ++v) {
            uint32_t i = 0;
            while (deg[v] > th[i]) ++i;
            bk[v] = (uint8_t)i;
            size[i]++;
        }
        if (lmode == 6 || lmode == 7) {
            const uint32_t hot = size[1];
            uint32_t *hid = (uint32_t *)xmalloc((size_t)hot * 4 + 4);
            uint32_t *hs = (uint32_t *)xmalloc((size_t)hot * 4 + 4);
            uint32_t h = 0, c = 0, maxdeg = 0;
            for (uint32_t v = 0; v < n; ++v) {
                if (bk[v] == 1) {
                    hid[h++] = v;
                    if (deg[v] > maxdeg) maxdeg = deg[v];
                } else {
                    newlab[v] = hot + c++;
                }
            }
            counting_pass(hot, deg, maxdeg + 1, hid, hs);
            for (uint32_t i = 0; i < hot; ++i) newlab[hs[i]] = hot - 1 - i;
            free(hs);
            free(hid);
        } else {
            uint32_t start[11];
            uint32_t acc = 0;
            for (int j = (int)nb - 1; j >= 0; --j) { start[j] = acc; acc += size[j]; }
            for (uint32_t v = 0; v < n; ++v) newlab[v] = start[bk[v]]++;
        }
        free(bk);
    }
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)num_edges; ++i) {
        src[i] = newlab[src[i]];
        dst[i] = newlab[dst[i]];
    }
    for (uint32_t v = 0; v < n; ++v) {
        labels[v] = newlab[labels[v]];
        inverse_labels[labels[v]] = v;
    }
    free(newlab);
    free(deg);
}

/* maskGraphProcess (reorder.c:1164-1475) run by one thread.
 *
 * Degrees (maskGraphProcessGenerateInOutDegrees, :1260-1306): mmode 2, 4
 * count in-degrees, 5, 6 in + out, every other mode out-degrees. Buckets as
 * DBG: 11 thresholds t0 = avg <= 1 ? 1 : avg/2 (avg = E/V, uint32),
 * doubling, last UINT32_MAX. Regions (:1329-1345), cs = cache_size / 4:
 * V/4 HOT, V/4 WARM, V/4 LUKEWARM when V - cs < 2 cs, else cs*8 HOT, cs*32
 * WARM, cs*128 LUKEWARM (uint32 products); the rest COLD. Vertices take the
 * regions in order, buckets from the highest and ascending ids inside a
 * bucket (:1408-1436). With more than one thread the reference's regions
 * are taken by the threads concurrently, so which vertex gets which hint
 * then depends on the schedule; the one-thread order is the one restated.
 * mmode 1, 2 then OR the hints into the edge list's ids (maskEdgeList,
 * :1639-1657); every mode returns the hints per vertex. */
void orc_mask_graph(uint32_t num_vertices, uint32_t num_edges, uint32_t *src, uint32_t *dst,
                    int mmode, uint32_t cache_size, uint32_t *mask) {
    const uint32_t n = num_vertices;
    uint32_t *deg = (uint32_t *)calloc((size_t)n + 1, 4);
    if (!deg) abort();
    for (uint32_t i = 0; i < num_edges; ++i) {
        if (mmode == 2 || mmode == 4) deg[dst[i]]++;
        else if (mmode == 5 || mmode == 6) { deg[dst[i]]++; deg[src[i]]++; }
        else deg[src[i]]++;
    }
    uint32_t th[11];
    const uint32_t avg = n ? num_edges / n : 0;
    th[0] = avg <= 1 ? 1u : avg / 2;
    for (int i = 1; i < 10; ++i) th[i] = th[i - 1] * 2u;
    th[10] = 0xFFFFFFFFu;
    uint8_t *bk = (uint8_t *)xmalloc((size_t)n + 1);
    for (uint32_t v = 0; v < n; ++v) {
        uint32_t i = 0;
        while (deg[v] > th[i]) ++i;
        bk[v] = (uint8_t)i;
    }
    const uint32_t cs = cache_size >> 2;
    uint32_t region[3];
    if ((int64_t)n - (int64_t)cs < 2 * (int64_t)cs) {
        region[0] = region[1] = region[2] = n / 4;
    } else {
        region[0] = cs * 8u;
        region[1] = region[0] * 4u;
        region[2] = region[1] * 4u;
    }
    static const uint32_t hint[4] = {0xC0000000u, 0x80000000u, 0x40000000u, 0u};
    for (int j = 10; j >= 0; --j) {
        for (uint32_t v = 0; v < n; ++v) {
            if (bk[v] != j) continue;
            int r = 0;
            while (r < 3 && region[r] == 0) ++r;
            if (r < 3) region[r]--;
            mask[v] = hint[r];
        }
    }
    if (mmode == 1 || mmode == 2) {
        for (uint32_t i = 0; i < num_edges; ++i) {
            src[i] |= mask[src[i]];
            dst[i] |= mask[dst[i]];
        }
    }
    free(bk);
    free(deg);
}

/* ------------------------------------------------------------------------ */
/* BFS                                                                      */
/* ------------------------------------------------------------------------ */

/* Frontier of the top-down step: newly discovered vertices are claimed
 * with a compare-and-swap on parents[] (BFS.c:518-540) and collected in
 * per-thread buffers that are concatenated (the reference's local queues
 * flushed to the shared queue, arrayQueue.c:257-270). Returns mf, the sum
 * of -parent_old over claimed vertices (out-degree, or 1 for degree 0). */
static uint32_t bfs_top_down(const uint32_t *out_degree, const uint32_t *edges_idx,
                             const uint32_t *dest, uint32_t *distances, int32_t *parents,
                             const uint32_t *queue, uint32_t qlen, uint32_t *next,
                             uint32_t *next_len, uint32_t *scratch, uint32_t n) {
    uint32_t mf = 0;
    uint32_t total = 0;
    int nt = omp_get_max_threads();
    uint32_t *counts = (uint32_t *)calloc((size_t)nt + 1, 4);
    if (!counts) abort();
    #pragma omp parallel reduction(+ : mf)
    {
        int t = omp_get_thread_num();
        int T = omp_get_num_threads();
        /* each thread owns a slice of scratch of size n/T+1 worst case is
         * not guaranteed, so threads write to a private heap buffer */
        uint32_t cap = 1024, len = 0;
        uint32_t *local = (uint32_t *)xmalloc((size_t)cap * 4);
        #pragma omp for schedule(dynamic, 64)
        for (uint32_t i = 0; i < qlen; ++i) {
            uint32_t v = queue[i];
            uint32_t b = edges_idx[v], e = b + out_degree[v];
            for (uint32_t j = b; j < e; ++j) {
                uint32_t u = dest[j] & 0x3FFFFFFFu;
                int32_t pu = __atomic_load_n(&parents[u], __ATOMIC_RELAXED);
                if (pu < 0) {
                    if (__atomic_compare_exchange_n(&parents[u], &pu, (int32_t)v, 0,
                                                    __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                        distances[u] = distances[v] + 1;
                        mf += (uint32_t)(-pu);
                        if (len == cap) {
                            cap *= 2;
                            local = (uint32_t *)realloc(local, (size_t)cap * 4);
                            if (!local) abort();
                        }
                        local[len++] = u;
                    }
                }
            }
        }
        counts[t + 1] = len;
        #pragma omp barrier
        #pragma omp single
        {
            for (int k = 0; k < T; ++k) counts[k + 1] += counts[k];
            total = counts[T];
        }
        memcpy(next + counts[t], local, (size_t)len * 4);
        free(local);
    }
    (void)scratch;
    (void)n;
    free(counts);
    *next_len = total;
    return mf;
}

/* bottomUpStepGraphCSR (BFS.c:562-613): every unvisited vertex scans its
 * pull neighbours for one in the current frontier bitmap. */
static uint32_t bfs_bottom_up(uint32_t n, const uint32_t *pull_degree, const uint32_t *pull_idx,
                              const uint32_t *pull_src, uint32_t *distances, int32_t *parents,
                              const uint8_t *curr, uint8_t *next) {
    uint32_t nf = 0;
    #pragma omp parallel for schedule(dynamic, 1024) reduction(+ : nf)
    for (uint32_t v = 0; v < n; ++v) {
        if (parents[v] < 0) {
            uint32_t b = pull_idx[v], e = b + pull_degree[v];
            for (uint32_t j = b; j < e; ++j) {
                uint32_t u = pull_src[j] & 0x3FFFFFFFu;
                if (curr[u]) {
                    parents[v] = (int32_t)u;
                    distances[v] = distances[u] + 1;
                    next[v] = 1;
                    nf++;
                    break;
                }
            }
        }
    }
    return nf;
}

/* breadthFirstSearchDirectionOptimizedGraphCSR (BFS.c:335-485), with the
 * stats initialisation of newBFSStatsGraphCSR (BFS.c:42-78). */
void orc_bfs(uint32_t num_vertices, uint32_t num_edges,
             const uint32_t *out_degree, const uint32_t *edges_idx, const uint32_t *dest,
             const uint32_t *pull_degree, const uint32_t *pull_idx, const uint32_t *pull_src,
             uint32_t source, uint32_t *distances, int32_t *parents,
             uint32_t *processed_nodes, uint32_t *iterations, int num_threads) {
    set_threads(num_threads);
    uint32_t n = num_vertices;
    #pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < n; ++v) {
        distances[v] = 0;
        parents[v] = out_degree[v] ? -(int32_t)out_degree[v] : -1;
    }
    *processed_nodes = 0;
    *iterations = 0;
    if (source >= n) return;
    uint32_t *queue = (uint32_t *)xmalloc((size_t)n * 4 + 4);
    uint32_t *next = (uint32_t *)xmalloc((size_t)n * 4 + 4);
    uint8_t *bcur = (uint8_t *)calloc((size_t)n + 1, 1);
    uint8_t *bnext = (uint8_t *)calloc((size_t)n + 1, 1);
    if (!bcur || !bnext) abort();
    uint32_t qlen = 1;
    queue[0] = source;
    parents[source] = (int32_t)source;
    uint32_t processed = 1, iter = 1;
    uint32_t mu = num_edges, mf = out_degree[source];
    const uint32_t alpha = 15, beta = 18;
    while (qlen) {
        if (mf > mu / alpha) {
            memset(bcur, 0, n);
            for (uint32_t i = 0; i < qlen; ++i) bcur[queue[i]] = 1;
            uint32_t nf = qlen, nf_prev;
            do {
                nf_prev = nf;
                nf = bfs_bottom_up(n, pull_degree, pull_idx, pull_src, distances, parents, bcur, bnext);
                uint8_t *t = bcur; bcur = bnext; bnext = t;
                memset(bnext, 0, n);
                processed += nf;
                iter++;
            } while (nf > nf_prev || nf > n / beta);
            qlen = 0;
            for (uint32_t v = 0; v < n; ++v)
                if (bcur[v]) queue[qlen++] = v;
            mf = 1;
        } else {
            mu -= mf;
            uint32_t nlen = 0;
            mf = bfs_top_down(out_degree, edges_idx, dest, distances, parents, queue, qlen, next,
                              &nlen, NULL, n);
            uint32_t *t = queue; queue = next; next = t;
            qlen = nlen;
            processed += qlen;
            iter++;
        }
    }
    *processed_nodes = processed;
    *iterations = iter;
    free(queue);
    free(next);
    free(bcur);
    free(bnext);
}

/* ------------------------------------------------------------------------ */
/* PageRank                                                                 */
/* ------------------------------------------------------------------------ */

/* pageRankPullGraphCSR (pageRank.c:245-368) with the stats defaults of
 * newPageRankStatsGraphCSR (pageRank.c:47-75): damp 0.85f, ranks start at
 * base_pr = 1-damp, contributions r/outdeg (0 for dangling vertices), stop
 * when no vertex moved by >= epsilon, finally r /= N. */
void orc_pagerank_pull(uint32_t num_vertices, const uint32_t *out_degree,
                       const uint32_t *pull_degree, const uint32_t *pull_idx, const uint32_t *pull_src,
                       uint32_t max_iterations, double epsilon, float *ranks,
                       uint32_t *iterations, double *error_total, int num_threads) {
    set_threads(num_threads);
    const uint32_t n = num_vertices;
    const float damp = 0.85f;
    const float base_pr = 1.0f - damp;
    float *contrib = (float *)xmalloc((size_t)n * 4 + 4);
    float *sums = (float *)xmalloc((size_t)n * 4 + 4);
    for (uint32_t v = 0; v < n; ++v) ranks[v] = base_pr;
    double err = 0.0;
    uint32_t it;
    for (it = 0; it < max_iterations; ++it) {
        err = 0.0;
        uint32_t active = 0;
        #pragma omp parallel for schedule(static)
        for (uint32_t v = 0; v < n; ++v)
            contrib[v] = out_degree[v] ? ranks[v] / (float)out_degree[v] : 0.0f;
        #pragma omp parallel for schedule(dynamic, 1024)
        for (uint32_t v = 0; v < n; ++v) {
            float s = 0.0f;
            uint32_t b = pull_idx[v], e = b + pull_degree[v];
            for (uint32_t j = b; j < e; ++j) s += contrib[pull_src[j] & 0x3FFFFFFFu];
            sums[v] = s;
        }
        #pragma omp parallel for schedule(static) reduction(+ : err, active)
        for (uint32_t v = 0; v < n; ++v) {
            float prev = ranks[v];
            float next = base_pr + damp * sums[v];
            ranks[v] = next;
            double e = fabs((double)(next - prev));
            err += e / n;
            if (e >= epsilon) active++;
        }
        if (active == 0) break;
    }
    for (uint32_t v = 0; v < n; ++v) ranks[v] = ranks[v] / (float)n;
    *iterations = it;
    *error_total = err;
    free(contrib);
    free(sums);
}

void orc_pagerank_pull_f64(uint32_t num_vertices, const uint32_t *out_degree,
                           const uint32_t *pull_degree, const uint32_t *pull_idx, const uint32_t *pull_src,
                           uint32_t max_iterations, double epsilon, double *ranks,
                           uint32_t *iterations, int num_threads) {
    set_threads(num_threads);
    const uint32_t n = num_vertices;
    /* the FP32 constants, held exactly in FP64, so that the comparison
     * measures arithmetic rounding only */
    const double damp = (double)0.85f;
    const double base_pr = (double)(1.0f - 0.85f);
    double *contrib = (double *)xmalloc((size_t)n * 8 + 8);
    double *sums = (double *)xmalloc((size_t)n * 8 + 8);
    for (uint32_t v = 0; v < n; ++v) ranks[v] = base_pr;
    uint32_t it;
    for (it = 0; it < max_iterations; ++it) {
        uint32_t active = 0;
        #pragma omp parallel for schedule(static)
        for (uint32_t v = 0; v < n; ++v)
            contrib[v] = out_degree[v] ? ranks[v] / (double)out_degree[v] : 0.0;
        #pragma omp parallel for schedule(dynamic, 1024)
        for (uint32_t v = 0; v < n; ++v) {
            double s = 0.0;
            uint32_t b = pull_idx[v], e = b + pull_degree[v];
            for (uint32_t j = b; j < e; ++j) s += contrib[pull_src[j] & 0x3FFFFFFFu];
            sums[v] = s;
        }
        #pragma omp parallel for schedule(static) reduction(+ : active)
        for (uint32_t v = 0; v < n; ++v) {
            double next = base_pr + damp * sums[v];
            if (fabs(next - ranks[v]) >= epsilon) active++;
            ranks[v] = next;
        }
        if (active == 0) break;
    }
    for (uint32_t v = 0; v < n; ++v) ranks[v] = ranks[v] / (double)n;
    *iterations = it;
    free(contrib);
    free(sums);
}

/* ------------------------------------------------------------------------ */
/* SSSP                                                                     */
/* ------------------------------------------------------------------------ */

static inline uint32_t sssp_add(uint32_t d, float w) {
    /* SSSP.c:204,262: uint32 + float evaluated in float, stored to uint32 */
    return (uint32_t)((float)d + w);
}

static inline int atomic_min_u32(uint32_t *p, uint32_t v) {
    uint32_t old = __atomic_load_n(p, __ATOMIC_ACQUIRE);
    while (old > v) {
        if (__atomic_compare_exchange_n(p, &old, v, 1, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE))
            return 1;
    }
    return 0;
}

/* SSSPDataDrivenPushGraphCSR (SSSP.c:514-653): each vertex sits in at most
 * one bucket (buckets_map[v] = dist/delta); bucket `cur` is drained
 * repeatedly by full sweeps over V until it stays empty. The relaxation
 * takes the minimum with an atomic, and a vertex whose distance drops is
 * re-filed under min(old bucket, new bucket), so a drop that races with
 * the vertex being drained is never lost; the fixed point is the unique
 * shortest-distance vector under the reference's arithmetic. Empty buckets
 * are skipped by jumping to the smallest occupied one. */
void orc_sssp(uint32_t num_vertices, const uint32_t *out_degree, const uint32_t *edges_idx,
              const uint32_t *dest, const float *weights, uint32_t source, uint32_t delta,
              uint32_t *distances, uint32_t *processed_nodes, int num_threads) {
    set_threads(num_threads);
    const uint32_t n = num_vertices;
    if (delta == 0) delta = 1;
    uint32_t *bucket = (uint32_t *)xmalloc((size_t)n * 4 + 4);
    #pragma omp parallel for schedule(static)
    for (uint32_t v = 0; v < n; ++v) {
        distances[v] = ORC_INF;
        bucket[v] = ORC_INF;
    }
    uint32_t processed = 0;
    if (source < n) {
        distances[source] = 0;
        bucket[source] = 0;
        uint32_t cur = 0;
        for (;;) {
            int changed = 1;
            while (changed) {
                changed = 0;
                #pragma omp parallel for schedule(dynamic, 1024) reduction(| : changed) reduction(+ : processed)
                for (uint32_t v = 0; v < n; ++v) {
                    if (__atomic_load_n(&bucket[v], __ATOMIC_RELAXED) != cur) continue;
                    uint32_t expect = cur;
                    if (!__atomic_compare_exchange_n(&bucket[v], &expect, ORC_INF, 0,
                                                     __ATOMIC_ACQ_REL, __ATOMIC_RELAXED))
                        continue;
                    processed++;
                    uint32_t d = __atomic_load_n(&distances[v], __ATOMIC_ACQUIRE);
                    uint32_t b = edges_idx[v], e = b + out_degree[v];
                    for (uint32_t j = b; j < e; ++j) {
                        uint32_t u = dest[j] & 0x3FFFFFFFu;
                        float w = weights ? weights[j] : 1.0f;
                        uint32_t nd = sssp_add(d, w);
                        if (atomic_min_u32(&distances[u], nd)) {
                            uint32_t nb = nd / delta;
                            atomic_min_u32(&bucket[u], nb);
                            if (nb == cur) changed = 1;
                        }
                    }
                }
            }
            uint32_t nextb = ORC_INF;
            #pragma omp parallel for schedule(static) reduction(min : nextb)
            for (uint32_t v = 0; v < n; ++v)
                if (bucket[v] < nextb) nextb = bucket[v];
            if (nextb == ORC_INF) break;
            cur = nextb;
        }
    }
    if (processed_nodes) *processed_nodes = processed;
    free(bucket);
}

/* ------------------------------------------------------------------------ */
/* connected components                                                     */
/* ------------------------------------------------------------------------ */

/* linkNodes (connectedComponents.c:177-196): hook the higher root under
 * the lower one with a compare-and-swap, re-reading on failure. */
static void cc_link(uint32_t u, uint32_t v, uint32_t *comp) {
    uint32_t p1 = __atomic_load_n(&comp[u], __ATOMIC_RELAXED);
    uint32_t p2 = __atomic_load_n(&comp[v], __ATOMIC_RELAXED);
    while (p1 != p2) {
        uint32_t high = p1 > p2 ? p1 : p2;
        uint32_t low = p1 + (p2 - high);
        uint32_t phigh = __atomic_load_n(&comp[high], __ATOMIC_RELAXED);
        if (phigh == low) break;
        if (phigh == high) {
            uint32_t expect = high;
            if (__atomic_compare_exchange_n(&comp[high], &expect, low, 0, __ATOMIC_RELAXED,
                                            __ATOMIC_RELAXED))
                break;
        }
        p1 = __atomic_load_n(&comp[__atomic_load_n(&comp[high], __ATOMIC_RELAXED)], __ATOMIC_RELAXED);
        p2 = __atomic_load_n(&comp[low], __ATOMIC_RELAXED);
    }
}

/* compressNodes (connectedComponents.c:199-210) */
static void cc_compress(uint32_t n, uint32_t *comp) {
    #pragma omp parallel for schedule(dynamic, 2048)
    for (uint32_t v = 0; v < n; ++v) {
        while (comp[v] != comp[comp[v]]) comp[v] = comp[comp[v]];
    }
}

void orc_cc(uint32_t num_vertices, const uint32_t *out_degree, const uint32_t *edges_idx,
            const uint32_t *dest, const uint32_t *pull_degree, const uint32_t *pull_idx,
            const uint32_t *pull_src, int variant, uint32_t *components,
            uint32_t *iterations, int num_threads) {
    set_threads(num_threads);
    const uint32_t n = num_vertices;
    uint32_t *comp = components;
    for (uint32_t v = 0; v < n; ++v) comp[v] = v;
    uint32_t iters = 0;
    if (variant == 0) {
        /* Shiloach-Vishkin (connectedComponents.c:293-377) */
        int change = 1;
        while (change) {
            change = 0;
            iters++;
            #pragma omp parallel for schedule(dynamic, 512) reduction(| : change)
            for (uint32_t v = 0; v < n; ++v) {
                uint32_t b = edges_idx[v], e = b + out_degree[v];
                for (uint32_t j = b; j < e; ++j) {
                    uint32_t u = dest[j] & 0x3FFFFFFFu;
                    uint32_t cs = __atomic_load_n(&comp[v], __ATOMIC_RELAXED);
                    uint32_t cd = __atomic_load_n(&comp[u], __ATOMIC_RELAXED);
                    if (cs == cd) continue;
                    uint32_t high = cs > cd ? cs : cd, low = cs + (cd - high);
                    if (__atomic_load_n(&comp[high], __ATOMIC_RELAXED) == high) {
                        /* the reference's plain store races benignly; a CAS keeps
                         * hooks on roots only */
                        uint32_t expect = high;
                        __atomic_compare_exchange_n(&comp[high], &expect, low, 0, __ATOMIC_RELAXED,
                                                    __ATOMIC_RELAXED);
                        change = 1;
                    }
                }
                if (pull_degree) {
                    uint32_t pb = pull_idx[v], pe = pb + pull_degree[v];
                    for (uint32_t j = pb; j < pe; ++j) {
                        uint32_t u = pull_src[j] & 0x3FFFFFFFu;
                        uint32_t cs = __atomic_load_n(&comp[v], __ATOMIC_RELAXED);
                        uint32_t cd = __atomic_load_n(&comp[u], __ATOMIC_RELAXED);
                        if (cs == cd) continue;
                        uint32_t high = cs > cd ? cs : cd, low = cs + (cd - high);
                        if (__atomic_load_n(&comp[high], __ATOMIC_RELAXED) == high) {
                            uint32_t expect = high;
                            __atomic_compare_exchange_n(&comp[high], &expect, low, 0,
                                                        __ATOMIC_RELAXED, __ATOMIC_RELAXED);
                            change = 1;
                        }
                    }
                }
            }
            cc_compress(n, comp);
        }
    } else if (variant == 2) {
        /* weakly connected label propagation (connectedComponents.c:537-629) */
        int change = 1;
        while (change) {
            change = 0;
            iters++;
            #pragma omp parallel for schedule(dynamic, 512) reduction(| : change)
            for (uint32_t v = 0; v < n; ++v) {
                uint32_t b = edges_idx[v], e = b + out_degree[v];
                for (uint32_t j = b; j < e; ++j) {
                    uint32_t u = dest[j] & 0x3FFFFFFFu;
                    if (atomic_min_u32(&comp[u], __atomic_load_n(&comp[v], __ATOMIC_RELAXED))) change = 1;
                    if (atomic_min_u32(&comp[v], __atomic_load_n(&comp[u], __ATOMIC_RELAXED))) change = 1;
                }
            }
        }
    } else {
        /* Afforest (connectedComponents.c:379-535): two neighbour rounds,
         * sample the most frequent component, final link skipping it. */
        const uint32_t rounds = 2;
        for (uint32_t r = 0; r < rounds; ++r) {
            #pragma omp parallel for schedule(dynamic, 2048)
            for (uint32_t u = 0; u < n; ++u) {
                if (r < out_degree[u]) cc_link(u, dest[edges_idx[u] + r] & 0x3FFFFFFFu, comp);
            }
            cc_compress(n, comp);
        }
        /* most frequent component among 1024 sampled vertices (first max in
         * key order, as the Judy scan does); which one is chosen does not
         * change the final labels */
        uint32_t skip = 0;
        if (n > 0) {
            uint32_t ns = n < 1024 ? n / 2 : 1024;
            uint32_t *samp = (uint32_t *)xmalloc((size_t)ns * 4 + 4);
            uint64_t x = 0x9E3779B97F4A7C15ull;
            for (uint32_t i = 0; i < ns; ++i) {
                x ^= x >> 12; x ^= x << 25; x ^= x >> 27;
                samp[i] = comp[(uint32_t)((x * 2685821657736338717ull) >> 32) % n];
            }
            /* insertion-free mode: sort then scan */
            for (uint32_t i = 1; i < ns; ++i) {
                uint32_t key = samp[i];
                int64_t k = (int64_t)i - 1;
                while (k >= 0 && samp[k] > key) { samp[k + 1] = samp[k]; --k; }
                samp[k + 1] = key;
            }
            uint32_t best = 0, bestc = 0;
            for (uint32_t i = 0; i < ns;) {
                uint32_t k = i;
                while (k < ns && samp[k] == samp[i]) ++k;
                if (k - i > bestc) { bestc = k - i; best = samp[i]; }
                i = k;
            }
            skip = best;
            free(samp);
        }
        #pragma omp parallel for schedule(dynamic, 2048)
        for (uint32_t u = 0; u < n; ++u) {
            if (comp[u] == skip) continue;
            uint32_t b = edges_idx[u], e = b + out_degree[u];
            for (uint32_t j = b + rounds; j < e; ++j) cc_link(u, dest[j] & 0x3FFFFFFFu, comp);
            if (pull_degree) {
                uint32_t pb = pull_idx[u], pe = pb + pull_degree[u];
                for (uint32_t j = pb; j < pe; ++j) cc_link(u, pull_src[j] & 0x3FFFFFFFu, comp);
            }
        }
        cc_compress(n, comp);
        iters = rounds;
    }
    if (iterations) *iterations = iters;
}

/* ------------------------------------------------------------------------ */
/* triangle count                                                           */
/* ------------------------------------------------------------------------ */

/* triangleCountPullGraphCSR (triangleCount.c:254-334). The innermost scan
 * of N(u) for the first element >= w is a membership test on a sorted
 * list, done here with a binary search; the count is the same. */
uint64_t orc_triangle_count_range(uint32_t num_vertices, const uint32_t *out_degree,
                                  const uint32_t *edges_idx, const uint32_t *dest, uint32_t lo,
                                  uint32_t hi, int num_threads) {
    set_threads(num_threads);
    uint64_t count = 0;
    if (hi > num_vertices) hi = num_vertices;
    #pragma omp parallel for schedule(dynamic, 128) reduction(+ : count)
    for (uint32_t u = lo; u < hi; ++u) {
        const uint32_t *nu = dest + edges_idx[u];
        uint32_t du = out_degree[u];
        for (uint32_t a = 0; a < du; ++a) {
            uint32_t v = nu[a] & 0x3FFFFFFFu;
            if (v > u) break;
            const uint32_t *nv = dest + edges_idx[v];
            uint32_t dv = out_degree[v];
            for (uint32_t c = 0; c < dv; ++c) {
                uint32_t w = nv[c] & 0x3FFFFFFFu;
                if (w > v) break;
                /* first element of N(u) that is >= w */
                uint32_t l = 0, h = du;
                while (l < h) {
                    uint32_t mid = (l + h) >> 1;
                    if ((nu[mid] & 0x3FFFFFFFu) < w) l = mid + 1; else h = mid;
                }
                if (l < du && (nu[l] & 0x3FFFFFFFu) == w) count++;
            }
        }
    }
    return count;
}

uint64_t orc_triangle_count(uint32_t num_vertices, const uint32_t *out_degree,
                            const uint32_t *edges_idx, const uint32_t *dest, int num_threads) {
    return orc_triangle_count_range(num_vertices, out_degree, edges_idx, dest, 0, num_vertices, num_threads);
}

/* ------------------------------------------------------------------------ */
/* SpMV                                                                     */
/* ------------------------------------------------------------------------ */

void orc_spmv_pull(uint32_t num_vertices, const uint32_t *pull_degree, const uint32_t *pull_idx,
                   const uint32_t *pull_src, const float *weights, float default_weight,
                   const float *x, float *y, uint32_t iterations, int num_threads) {
    set_threads(num_threads);
    for (uint32_t it = 0; it < iterations; ++it) {
        #pragma omp parallel for schedule(dynamic, 1024)
        for (uint32_t v = 0; v < num_vertices; ++v) {
            uint32_t b = pull_idx[v], e = b + pull_degree[v];
            float acc = y[v];
            for (uint32_t j = b; j < e; ++j) {
                float w = weights ? weights[j] : default_weight;
                acc += w * x[pull_src[j] & 0x3FFFFFFFu];
            }
            y[v] = acc;
        }
    }
}

void orc_spmv_pull_f64(uint32_t num_vertices, const uint32_t *pull_degree, const uint32_t *pull_idx,
                       const uint32_t *pull_src, const float *weights, float default_weight,
                       const float *x, double *y, uint32_t iterations, int num_threads) {
    set_threads(num_threads);
    for (uint32_t it = 0; it < iterations; ++it) {
        #pragma omp parallel for schedule(dynamic, 1024)
        for (uint32_t v = 0; v < num_vertices; ++v) {
            uint32_t b = pull_idx[v], e = b + pull_degree[v];
            double acc = y[v];
            for (uint32_t j = b; j < e; ++j) {
                double w = weights ? (double)weights[j] : (double)default_weight;
                acc += w * (double)x[pull_src[j] & 0x3FFFFFFFu];
            }
            y[v] = acc;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* random roots (mt19937.c, betweennessCentrality.c:172-189)                */
/* ------------------------------------------------------------------------ */

/* The Mersenne Twister MT19937 (Matsumoto and Nishimura, 1998) with the
 * seeding of its first release (Knuth's LCG x <- 69069 x + 1, two draws
 * per state word, the upper 16 bits of each), which is the generator the
 * reference seeds with 27491095 (graphConfig.c:84). */
typedef struct { uint32_t mt[624]; int mti; } orc_mt;

static void orc_mt_seed(orc_mt *m, uint32_t seed) {
    for (int i = 0; i < 624; ++i) {
        m->mt[i] = seed & 0xffff0000u;
        seed = 69069u * seed + 1u;
        m->mt[i] |= (seed & 0xffff0000u) >> 16;
        seed = 69069u * seed + 1u;
    }
    m->mti = 624;
}

static uint32_t orc_mt_next(orc_mt *m) {
    if (m->mti >= 624) {
        for (int k = 0; k < 624; ++k) {
            const uint32_t y = (m->mt[k] & 0x80000000u) | (m->mt[(k + 1) % 624] & 0x7fffffffu);
            m->mt[k] = m->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        m->mti = 0;
    }
    uint32_t y = m->mt[m->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* generateRandomRootBetweennessCentrality, n times from one seeded state:
 * draw until the value is a vertex whose out-degree exceeds avg_degree. */
void orc_random_roots(uint32_t seed, uint32_t n, uint32_t num_vertices, const uint32_t *out_degree,
                      uint32_t avg_degree, uint32_t *roots) {
    orc_mt m;
    orc_mt_seed(&m, seed);
    for (uint32_t i = 0; i < n; ++i) {
        for (;;) {
            const uint32_t r = orc_mt_next(&m);
            if (r < num_vertices && out_degree[r] > avg_degree) { roots[i] = r; break; }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* betweenness centrality (betweennessCentrality.c:230-466)                 */
/* ------------------------------------------------------------------------ */

/* Brandes from each root in turn, accumulating into bc[] (which the caller
 * zeroes, as newBetweennessCentralityStatsGraphCSR does). Per root: a
 * level-synchronous pull BFS over the pull CSR (the inverse CSR in a
 * DIRECTED build, the forward one otherwise): an unreached v whose pull
 * row holds frontier vertices gets level + 1, sigma[v] = the sum of their
 * sigma (int) and the list of those entries as its predecessors, in row
 * order (:289-347). The stack holds the levels in order, ids ascending
 * inside a level (copyBitmapToStack, :205-217). Then, for the stack from
 * the top down to (not including) the root, each predecessor v of w takes
 * dependency[v] += (sigma[v] * 1.0 / sigma[w]) * (1 + dependency[w]) --
 * a double product of the double ratio and the float 1 + dependency[w],
 * added in double and stored as float -- when sigma[w] != 0, and
 * bc[w] += dependency[w] / 2 for w != root (:432-455). Returns, for the
 * last root, its distances (UINT32_MAX unreached), sigma, dependency and
 * processed_nodes = the number of predecessor entries. */
void orc_betweenness(uint32_t num_vertices, const uint32_t *pull_degree, const uint32_t *pull_idx,
                     const uint32_t *pull_src, uint32_t num_roots, const uint32_t *roots, float *bc,
                     uint32_t *distances, int32_t *sigma, float *dependency, uint32_t *processed_nodes) {
    const uint32_t n = num_vertices;
    uint64_t E = 0;
    for (uint32_t v = 0; v < n; ++v) E += pull_degree[v];
    uint32_t *pred_off = (uint32_t *)xmalloc(((size_t)n + 1) * 4);
    uint32_t *pred_cnt = (uint32_t *)xmalloc((size_t)n * 4 + 4);
    uint32_t *preds = (uint32_t *)xmalloc((size_t)E * 4 + 4);
    uint32_t *stack = (uint32_t *)xmalloc((size_t)n * 4 + 4);
    uint8_t *frontier = (uint8_t *)xmalloc((size_t)n + 1);
    uint8_t *next = (uint8_t *)xmalloc((size_t)n + 1);
    pred_off[0] = 0;
    for (uint32_t v = 0; v < n; ++v) pred_off[v + 1] = pred_off[v] + pull_degree[v];
    for (uint32_t r = 0; r < num_roots; ++r) {
        const uint32_t s = roots[r];
        uint32_t processed = 0, top = 0;
        for (uint32_t v = 0; v < n; ++v) {
            distances[v] = 0xFFFFFFFFu;
            dependency[v] = 0.0f;
            sigma[v] = 0;
            pred_cnt[v] = 0;
            frontier[v] = 0;
        }
        distances[s] = 0;
        sigma[s] = 1;
        frontier[s] = 1;
        stack[top++] = s;
        uint32_t nf = 1;
        while (nf) {
            nf = 0;
            memset(next, 0, n);
            for (uint32_t v = 0; v < n; ++v) {
                if (distances[v] != 0xFFFFFFFFu) continue;
                for (uint32_t j = pull_idx[v]; j < pull_idx[v] + pull_degree[v]; ++j) {
                    const uint32_t u = pull_src[j] & 0x3FFFFFFFu;
                    if (!frontier[u]) continue;
                    distances[v] = distances[u] + 1;
                    sigma[v] = (int32_t)((uint32_t)sigma[v] + (uint32_t)sigma[u]);
                    preds[pred_off[v] + pred_cnt[v]++] = u;
                    next[v] = 1;
                    ++nf;
                }
            }
            /* the loop above reads distances[] of frontier vertices only and
             * writes those of unreached ones, so its order does not matter */
            for (uint32_t v = 0; v < n; ++v) if (next[v]) stack[top++] = v;
            processed += nf;
            uint8_t *t = frontier; frontier = next; next = t;
        }
        for (uint32_t t = top - 1; t > 0; --t) {
            const uint32_t w = stack[t];
            for (uint32_t k = 0; k < pred_cnt[w]; ++k) {
                const uint32_t v = preds[pred_off[w] + k];
                if (sigma[w] != 0) {
                    const double ratio = (double)sigma[v] * 1.0 / (double)sigma[w];
                    const float one_plus = 1.0f + dependency[w];
                    dependency[v] = (float)((double)dependency[v] + ratio * (double)one_plus);
                }
            }
            if (w != s) bc[w] += dependency[w] / 2;
        }
        *processed_nodes = processed;
    }
    free(next);
    free(frontier);
    free(stack);
    free(preds);
    free(pred_cnt);
    free(pred_off);
}

/* ------------------------------------------------------------------------ */
/* depth-first search (DFS.c:156-205)                                       */
/* ------------------------------------------------------------------------ */

/* One LIFO stack, a vertex marked when pushed: pop v, then for v's
 * out-edges in CSR order push every u whose parent is still negative, with
 * parent v and distance distance[v] + 1. distances start 0, parents -1,
 * the root is its own parent; processed_nodes counts pops. */
void orc_dfs(uint32_t num_vertices, const uint32_t *out_degree, const uint32_t *edges_idx,
             const uint32_t *dest, uint32_t source, uint32_t *distances, int32_t *parents,
             uint32_t *processed_nodes) {
    const uint32_t n = num_vertices;
    uint32_t *stack = (uint32_t *)xmalloc((size_t)n * 4 + 4);
    for (uint32_t v = 0; v < n; ++v) { distances[v] = 0; parents[v] = -1; }
    uint32_t top = 0, processed = 0;
    stack[top++] = source;
    parents[source] = (int32_t)source;
    while (top) {
        const uint32_t v = stack[--top];
        ++processed;
        for (uint32_t j = edges_idx[v]; j < edges_idx[v] + out_degree[v]; ++j) {
            const uint32_t u = dest[j] & 0x3FFFFFFFu;
            if (parents[u] < 0) {
                parents[u] = (int32_t)v;
                distances[u] = distances[v] + 1;
                stack[top++] = u;
            }
        }
    }
    *processed_nodes = processed;
    free(stack);
}

/* ------------------------------------------------------------------------ */
/* synthetic inputs (no reference counterpart)                              */
/* ------------------------------------------------------------------------ */

/* splitmix64's finaliser (Steele, Lea and Flood, 2014) */
static inline uint64_t orc_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* the start of the stream of draw `index` under `seed` */
static inline uint64_t orc_stream(uint64_t seed, uint64_t index) {
    return orc_mix64(seed * 0xD1B54A32D192ED03ull + 0x9E3779B97F4A7C15ull) ^ (index * 0x9E3779B97F4A7C15ull);
}

int orc_generate_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c, uint64_t seed,
                      uint32_t *src, uint32_t *dst) {
    if (!src || !dst || scale == 0 || scale > 30 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return -1;
    /* quadrant cut points on a 32-bit uniform */
    const double two32 = 4294967296.0;
    const uint64_t cut_a = (uint64_t)(a * two32), cut_ab = (uint64_t)((a + b) * two32);
    const uint64_t cut_abc = (uint64_t)((a + b + c) * two32);
    #pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)num_edges; ++e) {
        uint64_t state = orc_stream(seed, (uint64_t)e), word = 0;
        uint32_t s = 0, d = 0;
        for (uint32_t level = 0; level < scale; ++level) {
            /* one 64-bit draw serves two levels: low half, then high half */
            if (!(level & 1u)) {
                state += 0x9E3779B97F4A7C15ull;
                word = orc_mix64(state);
            }
            const uint64_t r = (level & 1u) ? (word >> 32) : (word & 0xFFFFFFFFull);
            const uint32_t right = r >= cut_abc || (r >= cut_a && r < cut_ab);  /* quadrants b, d */
            const uint32_t down = r >= cut_ab;                                 /* quadrants c, d */
            s = (s << 1) | down;
            d = (d << 1) | right;
        }
        src[e] = s;
        dst[e] = d;
    }
    return 0;
}

int orc_generate_values(uint64_t count, int kind, uint32_t lo, uint32_t hi, uint64_t seed, float *out) {
    if (!out || kind < 0 || kind > 3 || (kind == 0 && hi < lo)) return -1;
    const uint64_t span = (uint64_t)hi - lo + 1;
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; ++i) {
        const uint64_t h = orc_mix64(orc_stream(seed, (uint64_t)i) + 0x632BE59BD9B4E019ull);
        float v;
        if (kind == 0) {
            v = (float)(lo + (uint32_t)(h % span));
        } else if (kind == 1) {
            v = (float)((double)((h >> 40) + 1) / 16777216.0);
        } else if (kind == 2) {
            v = (float)((double)(h >> 40) / 8388608.0 - 1.0);
        } else {
            /* Box-Muller on two 26-bit uniforms in (0, 1) */
            const double u1 = ((double)(h >> 38) + 0.5) / 67108864.0;
            const double u2 = ((double)((h >> 12) & 0x3FFFFFFull) + 0.5) / 67108864.0;
            v = (float)exp(sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
        }
        out[i] = v;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* CSR segments                                                             */
/* ------------------------------------------------------------------------ */

uint32_t orc_csr_segments_count(uint32_t num_vertices, uint32_t cache_size) {
    /* csrSegmentsCalculateSegments (csrSegments.c:538-553) */
    uint32_t n = cache_size ? ((num_vertices * 8u) + cache_size - 1) / cache_size : 4u;
    return n < 4 ? 4 : n;
}

/* getSegmentID (csrSegments.c:555-570) */
static uint32_t orc_segment_id(uint32_t V, uint32_t S, uint32_t id) {
    uint32_t size = V / S;
    if (V % S == 0) return id / size;
    size += 1;
    uint32_t split = (V % S) * size;
    return id < split ? id / size : (id - split) / (size - 1) + (V % S);
}

void orc_csr_segments(uint32_t num_edges, const uint32_t *src, const uint32_t *dst, const float *w,
                      uint32_t num_vertices, uint32_t num_segments, uint32_t *out_degree, uint32_t *in_degree,
                      uint32_t *vertex_segment_index, uint32_t *segment_num_edges, uint32_t *segment_max_id,
                      uint32_t *seg_src, uint32_t *seg_dst, float *seg_w) {
    const uint32_t V = num_vertices, S = num_segments;
    memset(out_degree, 0, (size_t)V * 4);
    memset(in_degree, 0, (size_t)V * 4);
    memset(vertex_segment_index, 0, (size_t)V * 4);
    memset(segment_num_edges, 0, (size_t)S * 4);
    memset(segment_max_id, 0, (size_t)S * 4);
    /* graphCSRSegmentsProcessInOutDegrees, csrSegmentsSegmentEdgeListSizePreprocessing */
    for (uint32_t i = 0; i < num_edges; ++i) {
        out_degree[src[i]]++;
        in_degree[dst[i]]++;
        uint32_t seg = orc_segment_id(V, S, dst[i]);
        segment_num_edges[seg]++;
        vertex_segment_index[dst[i]] = seg;
    }
    /* csrSegmentsSegmentEdgePopulation (one thread: input order), and the
     * largest id of csrSegmentsSegmentVertexSizePreprocessing */
    uint32_t *pos = (uint32_t *)xmalloc((size_t)S * 4 + 4);
    uint32_t run = 0;
    for (uint32_t j = 0; j < S; ++j) {
        pos[j] = run;
        run += segment_num_edges[j];
    }
    for (uint32_t i = 0; i < num_edges; ++i) {
        uint32_t seg = orc_segment_id(V, S, dst[i]);
        uint32_t k = pos[seg]++;
        seg_src[k] = src[i];
        seg_dst[k] = dst[i];
        if (w && seg_w) seg_w[k] = w[i];
        uint32_t m = src[i] > dst[i] ? src[i] : dst[i];
        if (m > segment_max_id[seg]) segment_max_id[seg] = m;
    }
    free(pos);
}
