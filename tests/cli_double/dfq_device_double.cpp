// Test double of libdfq's device entry points (dfq_opts_default,
// dfq_graph_create / destroy, dfq_bfs, dfq_autotune), so that the bfs
// program's host logic - argument handling, input formats, the stdout block,
// the '$' loop, --frontier-profile - can be tested on a machine without a
// GPU.  TEST INFRASTRUCTURE ONLY: linked into a test copy of the program,
// never into libdfq.  Its BFS is a plain serial queue BFS; the tests check
// the program's output against the oracle.
#include "dfq.h"

#include <cstring>
#include <new>
#include <vector>

struct dfq_graph {
    int32_t n = 0;
    std::vector<int32_t> off, cols;
    dfq_opts opts{};
};

extern "C" {

void dfq_opts_default(dfq_opts* o) {
    std::memset(o, 0, sizeof *o);
    o->block_threads = 512;
    o->medium_min_degree = 64;
    o->large_min_degree = 256;
    o->local_queue_cap = 256;
    o->local_edge_budget = 8192;
    o->piece_edges = 256;
    o->probe_first = 2;
    o->use_tma = 1;
    o->timeout_ms = 5000;
}

int dfq_graph_create(const int32_t* offsets, const int32_t* cols, int32_t n, int64_t e, const dfq_opts* opts,
                     dfq_graph** out) {
    if (!out || !offsets || n < 1 || e < 0 || (e > 0 && !cols)) return DFQ_EINVAL;
    dfq_graph* g = new (std::nothrow) dfq_graph;
    if (!g) return DFQ_ENOMEM;
    g->n = n;
    g->off.assign(offsets, offsets + n + 1);
    g->cols.assign(cols, cols + e);
    if (opts) g->opts = *opts;
    else dfq_opts_default(&g->opts);
    *out = g;
    return DFQ_OK;
}

int dfq_graph_destroy(dfq_graph* g) {
    if (!g) return DFQ_EINVAL;
    delete g;
    return DFQ_OK;
}

int dfq_bfs(dfq_graph* g, int32_t src, int32_t* levels, int32_t* parents, dfq_stats* st) {
    if (!g || !levels || src < 0 || src >= g->n) return DFQ_EINVAL;
    for (int32_t v = 0; v < g->n; ++v) levels[v] = -1;
    if (parents)
        for (int32_t v = 0; v < g->n; ++v) parents[v] = -1;
    std::vector<int32_t> q{src};
    levels[src] = 0;
    if (parents) parents[src] = src;
    int64_t edges = 0;
    int32_t depth = 0;
    for (size_t h = 0; h < q.size(); ++h) {
        const int32_t u = q[h];
        edges += g->off[u + 1] - g->off[u];
        for (int32_t k = g->off[u]; k < g->off[u + 1]; ++k) {
            const int32_t v = g->cols[k];
            if (levels[v] >= 0) continue;
            levels[v] = levels[u] + 1;
            if (parents) parents[v] = u;
            if (levels[v] > depth) depth = levels[v];
            q.push_back(v);
        }
    }
    if (st) {
        std::memset(st, 0, sizeof *st);
        st->kernel_ms = 0.125f;
        st->depth = depth;
        st->levels = depth + 1;
        st->reached = (int64_t)q.size();
        st->edges = edges;
    }
    return DFQ_OK;
}

int dfq_autotune(dfq_graph* g, const int32_t* sources, int32_t nsrc, dfq_opts* best) {
    if (!g || !sources || nsrc < 1 || !best) return DFQ_EINVAL;
    *best = g->opts;
    return DFQ_OK;
}

}  // extern "C"
