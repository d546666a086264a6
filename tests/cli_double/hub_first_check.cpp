// Host check of dfq::hub_first_csr (the renumbering pools apply to wide
// skewed graphs).  TEST INFRASTRUCTURE ONLY.  Prints "ok" or the first
// property that fails:
//   order is a permutation and rank its inverse; in-degrees never increase
//   along order (ties by input id); new row i holds the renamed neighbours of
//   input row order[i] with its smallest new id first; auto mode renumbers the
//   R-MAT graph but not the grid; mode 1 never renumbers; the result does not
//   depend on the number of host threads.
#include "common.hpp"

#include <algorithm>
#include <cstdio>
#include <vector>

using namespace dfq;

static int check(const dfq_csr& in, int mode, int want_renumbered, const char* name) {
    dfq_csr out{};
    std::vector<int32_t> rank, order;
    const int r = hub_first_csr(in, mode, &out, &rank, &order);
    if (r != want_renumbered) { printf("%s: renumbered=%d, expected %d\n", name, r, want_renumbered); return 1; }
    if (r == 0) return 0;
    const int32_t n = in.n;
    std::vector<int32_t> indeg(n, 0);
    for (int64_t k = 0; k < in.e; ++k) indeg[in.cols[k]]++;
    std::vector<char> seen(n, 0);
    for (int32_t i = 0; i < n; ++i) {
        const int32_t o = order[i];
        if (o < 0 || o >= n || seen[o]) { printf("%s: order is not a permutation at %d\n", name, i); return 1; }
        seen[o] = 1;
        if (rank[o] != i) { printf("%s: rank is not the inverse of order at %d\n", name, i); return 1; }
        if (i > 0) {
            const int32_t p = order[i - 1];
            if (indeg[p] < indeg[o] || (indeg[p] == indeg[o] && p > o)) {
                printf("%s: order not by descending in-degree (ties by id) at %d\n", name, i);
                return 1;
            }
        }
        const int32_t d = in.offsets[o + 1] - in.offsets[o];
        if (out.offsets[i + 1] - out.offsets[i] != d) { printf("%s: degree of new row %d\n", name, i); return 1; }
        std::vector<int32_t> a(in.cols + in.offsets[o], in.cols + in.offsets[o + 1]);
        for (int32_t& c : a) c = rank[c];
        std::vector<int32_t> b(out.cols + out.offsets[i], out.cols + out.offsets[i + 1]);
        if (d > 0 && b[0] != *std::min_element(a.begin(), a.end())) {
            printf("%s: row %d does not start with its hub\n", name, i);
            return 1;
        }
        std::sort(a.begin(), a.end());
        std::sort(b.begin(), b.end());
        if (a != b) { printf("%s: row %d is not the renamed input row\n", name, i); return 1; }
    }
    // the same result with one host thread
    const int prev = dfq_host_threads();
    dfq_set_host_threads(1);
    dfq_csr out1{};
    std::vector<int32_t> rank1, order1;
    hub_first_csr(in, mode, &out1, &rank1, &order1);
    dfq_set_host_threads(prev);
    const bool same = order1 == order && std::equal(out.cols, out.cols + in.e, out1.cols);
    dfq_csr_free(&out1);
    dfq_csr_free(&out);
    if (!same) { printf("%s: result depends on the host thread count\n", name); return 1; }
    return 0;
}

int main() {
    dfq_csr rmat{}, grid{};
    if (dfq_gen_rmat(16, 16, 0.57, 0.19, 0.19, 7, DFQ_CSR_SYMMETRIZE | DFQ_CSR_DEDUP | DFQ_CSR_NO_SELF_LOOPS, &rmat) ||
        dfq_gen_grid(300, 0.01, 7, 1, &grid, nullptr)) {
        printf("generator failed: %s\n", dfq_last_error());
        return 1;
    }
    dfq_set_host_threads(8);
    int bad = check(rmat, 0, 1, "rmat16 auto") || check(rmat, 2, 1, "rmat16 always") ||
              check(rmat, 1, 0, "rmat16 keep") || check(grid, 0, 0, "grid auto") || check(grid, 2, 1, "grid always");
    dfq_csr_free(&rmat);
    dfq_csr_free(&grid);
    if (!bad) printf("ok\n");
    return bad;
}
