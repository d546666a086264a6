// Autotuner for the per-graph kernel options.  No reference counterpart: the
// reference fixes bin thresholds, tile sizes and queue capacities with
// #defines per program (bfs.cu:16-36) and compared hand-picked settings
// offline (com-orkut_8-64-1024-16384-all and its siblings).  Here the options
// are searched per graph by coordinate descent, timing real launches.
#include "common.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

using namespace dfq;

namespace {

// Median over sources of the device time of one BFS (ms); < 0 on failure.
double time_opts(dfq_graph* g, const dfq_opts& o, const int32_t* src, int nsrc, int32_t* levels_dev,
                 cudaEvent_t a, cudaEvent_t b) {
    if (dfq_graph_set_opts(g, &o) != DFQ_OK) return -1;
    cudaStream_t s = (cudaStream_t)dfq_graph_stream(g);
    std::vector<double> t;
    for (int i = 0; i < nsrc; ++i) {
        if (dfq_bfs_launch(g, src[i], levels_dev, nullptr) != DFQ_OK) return -1;  // warm
        cudaEventRecord(a, s);
        if (dfq_bfs_launch(g, src[i], levels_dev, nullptr) != DFQ_OK) return -1;
        cudaEventRecord(b, s);
        if (dfq_graph_sync(g) != DFQ_OK) return -1;
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        t.push_back(ms);
    }
    std::sort(t.begin(), t.end());
    return t[t.size() / 2];
}

}  // namespace

extern "C" int dfq_autotune(dfq_graph* g, const int32_t* sources, int32_t nsrc, dfq_opts* best) {
    clear_error();
    if (!g || !sources || nsrc < 1 || !best) return fail(DFQ_EINVAL, "dfq_autotune: bad arguments");
    dfq_opts cur;
    dfq_graph_get_opts(g, &cur);
    const dfq_opts start = cur;
    const int32_t n = dfq_graph_num_vertices(g);
    int32_t* levels = nullptr;
    if (cudaMalloc((void**)&levels, sizeof(int32_t) * (size_t)n) != cudaSuccess)
        return fail(DFQ_ENOMEM, "dfq_autotune: no device memory for a level array");
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int ns = std::min<int32_t>(nsrc, 8);
    double best_t = time_opts(g, cur, sources, ns, levels, a, b);
    int rc = DFQ_OK;
    if (best_t < 0) rc = DFQ_ECUDA;
    struct Axis { int32_t dfq_opts::*field; std::vector<int32_t> values; };
    const std::vector<Axis> axes = {
        {&dfq_opts::block_threads, {256, 512, 1024}},
        {&dfq_opts::large_min_degree, {256, 512, 1024, 2048, 4096, 16384}},
        {&dfq_opts::medium_min_degree, {8, 16, 32, 64, 128, 1 << 30}},
        {&dfq_opts::piece_edges, {128, 256, 512, 1024}},
        {&dfq_opts::local_queue_cap, {256, 512, 1024, 2048}},
        {&dfq_opts::local_edge_budget, {1024, 4096, 8192, 32768, 1 << 30}},
        {&dfq_opts::probe_first, {0, 1, 2}},
        {&dfq_opts::use_tma, {0, 1}},
        {&dfq_opts::blocks_per_sm, {0, 1, 2}},
        {&dfq_opts::l2_persist, {0, 1}},
    };
    for (int pass = 0; pass < 2 && rc == DFQ_OK; ++pass) {
        bool improved = false;
        for (const Axis& ax : axes) {
            for (int32_t v : ax.values) {
                if (cur.*ax.field == v) continue;
                dfq_opts t = cur;
                t.*ax.field = v;
                if (t.medium_min_degree > t.large_min_degree) t.medium_min_degree = t.large_min_degree;
                const double ms = time_opts(g, t, sources, ns, levels, a, b);
                if (ms > 0 && ms < best_t * 0.98) { best_t = ms; cur = t; improved = true; }
            }
        }
        if (!improved) break;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(levels);
    if (rc != DFQ_OK) {
        dfq_graph_set_opts(g, &start);
        return fail(rc, "dfq_autotune: baseline timing failed");
    }
    dfq_graph_set_opts(g, &cur);
    *best = cur;
    return DFQ_OK;
}
