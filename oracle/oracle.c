/*
 * oracle.c - CPU oracle for DFQ-BFS parity tests.  TEST INFRASTRUCTURE ONLY:
 * tests/, the smoke check and bench.py's CPU-baseline leg call it as the
 * checker; no product code path links or calls it.
 *
 * It restates the reference's own CPU path of
 *   design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu   ("DFQ" below)
 * which every reference program uses to check its kernel:
 *   oracle_bfs            DFQ:216-253  serial frontier BFS: F walked from the
 *                                      back (:232), X[] visited (:220-221),
 *                                      C[nid] = C[id] + 1 (:244), F = F_next (:250)
 *   oracle_compare        DFQ:290-299  near_nodes / near_errors / dist over the
 *                                      CPU-reached vertices, plus the check the
 *                                      reference leaves out (unreached == -1 on
 *                                      both sides)
 * and adds what the reference has no counterpart for:
 *   oracle_validate_tree  parent array is a BFS tree of the given levels
 *   oracle_reached_edges  E_R = sum of out-degrees of reached vertices (the
 *                         traversed-edge count of the GTEPS metric; it equals the
 *                         reference profiler's per-edge visit() total,
 *                         design/global-q/atomic-sa(-)/sup-sep(-)/upper-bound/profile/workload.cuh:12-14)
 *
 * Graph layout: CSR offsets[n+1] / cols[e]; the reference's Node{start,length}
 * is start = offsets[v], length = offsets[v+1] - offsets[v].
 * Levels are int32 with -1 = unreached (the reference's short cost[] with -1).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Returns the number of reached vertices (including src), or -1 on bad input /
 * allocation failure.  levels[n] is written for every vertex. */
int64_t oracle_bfs(int32_t n, const int32_t* offsets, const int32_t* cols, int32_t src, int32_t* levels) {
    if (n <= 0 || src < 0 || src >= n || !offsets || !levels) return -1;
    unsigned char* X = (unsigned char*)calloc((size_t)n, 1);
    int32_t* F = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* Fn = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    if (!X || !F || !Fn) { free(X); free(F); free(Fn); return -1; }
    for (int32_t i = 0; i < n; ++i) levels[i] = -1;
    /* C[] of the reference starts at 0 everywhere and is only read where X is
       set; with -1 for unreached vertices the output is the level array */
    levels[src] = 0;
    X[src] = 1;
    int64_t fsize = 1, reached = 1;
    F[0] = src;
    while (fsize > 0) {
        int64_t nsize = 0;
        for (int64_t i = fsize - 1; i >= 0; --i) { /* DFQ:232, back to front */
            const int32_t id = F[i];
            const int32_t start = offsets[id], end = offsets[id + 1];
            for (int32_t j = start; j < end; ++j) {
                const int32_t nid = cols[j];
                if (!X[nid]) {
                    X[nid] = 1;
                    levels[nid] = levels[id] + 1;
                    Fn[nsize++] = nid;
                }
            }
        }
        reached += nsize;
        int32_t* t = F; F = Fn; Fn = t;
        fsize = nsize;
    }
    free(X); free(F); free(Fn);
    return reached;
}

/* The reference's end-of-run check (DFQ:290-296), applied to a candidate level
 * array `got` against oracle levels `want`:
 *   out[0] = near_nodes  (vertices the oracle reached)
 *   out[1] = near_errors (reached by the oracle, got differs)
 *   out[2] = dist        (max level among matching reached vertices)
 *   out[3] = extra       (unreached by the oracle but got != -1: the check the
 *                         reference omits)
 * Returns out[1] + out[3] (0 = bit-exact). */
int64_t oracle_compare(int32_t n, const int32_t* want, const int32_t* got, int64_t* out) {
    int64_t near = 0, err = 0, dist = 0, extra = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (want[i] >= 0) {
            ++near;
            if (got[i] != want[i]) ++err;
            else if (got[i] > dist) dist = got[i];
        } else if (got[i] != -1) {
            ++extra;
        }
    }
    if (out) { out[0] = near; out[1] = err; out[2] = dist; out[3] = extra; }
    return err + extra;
}

/* BFS-tree validation of parents against levels.  Conditions:
 *   parents[src] == src and levels[src] == 0;
 *   levels[v] == -1  <=>  parents[v] == -1;
 *   otherwise p = parents[v] is in range, levels[p] == levels[v] - 1, and the
 *   edge p -> v exists in the CSR.
 * The edge check is one pass over the CSR (every edge u -> v with
 * parents[v] == u marks v), so the cost is O(n + e) whatever the degrees.
 * Returns 0 if valid, else 1 + the first offending vertex (so a caller can
 * report it), or -1 if the scratch allocation fails. */
int64_t oracle_validate_tree(int32_t n, const int32_t* offsets, const int32_t* cols, int32_t src,
                             const int32_t* levels, const int32_t* parents) {
    if (src < 0 || src >= n) return 1;
    if (parents[src] != src || levels[src] != 0) return 1 + (int64_t)src;
    unsigned char* has_edge = (unsigned char*)calloc((size_t)n, 1);
    if (!has_edge) return -1;
    for (int32_t u = 0; u < n; ++u)
        for (int32_t j = offsets[u]; j < offsets[u + 1]; ++j) {
            const int32_t v = cols[j];
            if (parents[v] == u) has_edge[v] = 1;
        }
    int64_t bad = 0;
    for (int32_t v = 0; v < n && !bad; ++v) {
        if (v == src) continue;
        const int32_t p = parents[v];
        if (levels[v] < 0) {
            if (p != -1) bad = 1 + (int64_t)v;
            continue;
        }
        if (p < 0 || p >= n || levels[p] != levels[v] - 1 || !has_edge[v]) bad = 1 + (int64_t)v;
    }
    free(has_edge);
    return bad;
}

/* E_R: sum of out-degrees over vertices with levels >= 0. */
int64_t oracle_reached_edges(int32_t n, const int32_t* offsets, const int32_t* levels) {
    int64_t s = 0;
    for (int32_t v = 0; v < n; ++v)
        if (levels[v] >= 0) s += offsets[v + 1] - offsets[v];
    return s;
}

/* Reached count, depth and per-level frontier sizes (hist[0..maxlev], hist may
 * be null).  Returns the depth (max level), -1 if nothing is reached. */
int32_t oracle_level_histogram(int32_t n, const int32_t* levels, int64_t* hist, int32_t maxlev) {
    int32_t depth = -1;
    if (hist) memset(hist, 0, sizeof(int64_t) * ((size_t)maxlev + 1));
    for (int32_t v = 0; v < n; ++v) {
        const int32_t l = levels[v];
        if (l < 0) continue;
        if (l > depth) depth = l;
        if (hist && l <= maxlev) hist[l]++;
    }
    return depth;
}
