// Host-side frontier profile: the idle-lane accounting of the reference's
// binned expansion (design/shared-q/atomic-sa/our-sep/upper-bound/
// bfs_ftr_prof.cu:98-144), computed exactly from a BFS's levels and the
// graph's degrees instead of by device atomics in the kernel.  The levels of
// this library's kernel equal the reference's, so the profile is the one the
// reference's profiler would print for the same graph and source.
#include "common.hpp"

#include <algorithm>
#include <cstring>
#include <vector>

using namespace dfq;

extern "C" {

int dfq_frontier_profile(const dfq_csr* g, const int32_t* levels, const int32_t tiles[4], int64_t threads,
                         int32_t max_levels, int64_t* idle, int64_t* count) {
    clear_error();
    if (!g || !levels || !tiles || max_levels < 0 || (g->n > 0 && !g->offsets))
        return fail(DFQ_EINVAL, "dfq_frontier_profile: bad arguments");
    if (threads < 1) return fail(DFQ_EINVAL, "dfq_frontier_profile: threads must be >= 1");
    for (int b = 0; b < 4; ++b) {
        const int32_t t = tiles[b];
        if (t < 1 || (t & (t - 1)) || (b > 0 && t <= tiles[b - 1]))
            return fail(DFQ_EINVAL, "dfq_frontier_profile: tiles must be increasing powers of two");
    }
    const int32_t n = g->n;
    int32_t depth = -1;
    for (int32_t v = 0; v < n; ++v) depth = std::max(depth, levels[v]);
    const int32_t L = std::min(depth + 1, max_levels);
    // per-range partial sums, combined in range order (results independent of threads)
    const int nt = std::max(1, std::min(host_threads(), (int)((int64_t)n / (1 << 16) + 1)));
    std::vector<std::vector<int64_t>> part_idle((size_t)nt, std::vector<int64_t>((size_t)L * 5, 0));
    std::vector<std::vector<int64_t>> part_cnt((size_t)nt, std::vector<int64_t>((size_t)L * 5, 0));
    run_threads(nt, [&](int i) {
        const int64_t lo = (int64_t)n * i / nt, hi = (int64_t)n * (i + 1) / nt;
        int64_t* pi = part_idle[(size_t)i].data();
        int64_t* pc = part_cnt[(size_t)i].data();
        for (int64_t v = lo; v < hi; ++v) {
            const int32_t lv = levels[v];
            if (lv < 0 || lv >= L) continue;
            const int64_t d = (int64_t)g->offsets[v + 1] - g->offsets[v];
            if (d <= 0) continue;
            int b = 0;
            while (b < 4 && d > tiles[b]) ++b;
            const int64_t waste = b < 4 ? tiles[b] - (d & (tiles[b] - 1)) : threads - (d % threads);
            pi[(size_t)lv * 5 + b] += waste;
            pc[(size_t)lv * 5 + b] += 1;
        }
    });
    if (idle) std::memset(idle, 0, sizeof(int64_t) * (size_t)max_levels * 5);
    if (count) std::memset(count, 0, sizeof(int64_t) * (size_t)max_levels * 5);
    for (int i = 0; i < nt; ++i)
        for (size_t k = 0; k < (size_t)L * 5; ++k) {
            if (idle) idle[k] += part_idle[(size_t)i][k];
            if (count) count[k] += part_cnt[(size_t)i][k];
        }
    return L;
}

}  // extern "C"
