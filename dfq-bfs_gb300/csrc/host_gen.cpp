// Seeded synthetic graph generators.  The reference measures on SNAP datasets
// that are not in its repository (.MISSING_LARGE_BLOBS); these generators make
// inputs with the same shapes.  Every generator derives one random stream per
// fixed-size chunk of work from (seed, chunk index), so output is identical for
// any number of host threads.
#include "common.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

using namespace dfq;

namespace {

// Fisher-Yates permutation of [0, n).
std::vector<int32_t> permutation(int32_t n, uint64_t seed) {
    std::vector<int32_t> p(n);
    std::iota(p.begin(), p.end(), 0);
    Rng r(seed);
    for (int32_t i = n - 1; i > 0; --i) {
        int32_t j = (int32_t)r.below((uint64_t)i + 1);
        std::swap(p[i], p[j]);
    }
    return p;
}

struct UnionFind {
    std::vector<int32_t> p;
    explicit UnionFind(int32_t n) : p(n) { std::iota(p.begin(), p.end(), 0); }
    int32_t find(int32_t x) {
        while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
        return x;
    }
    void unite(int32_t a, int32_t b) {
        a = find(a); b = find(b);
        if (a == b) return;
        if (a < b) std::swap(a, b);
        p[a] = b;
    }
};

}  // namespace

extern "C" {

int dfq_gen_zipf_geometric(int32_t n, double mean_deg, double alpha, uint64_t seed, dfq_csr* out) {
    clear_error();
    if (!out || n < 2 || !(mean_deg >= 0) || !(alpha > 0))
        return fail(DFQ_EINVAL, "dfq_gen_zipf_geometric: need n >= 2, mean_deg >= 0, alpha > 0");
    memset(out, 0, sizeof *out);
    // destination ranks 1..n with weight k^-alpha, mapped through a permutation
    // so that the heaviest destinations are not the lowest ids
    std::vector<int32_t> perm = permutation(n, mix_seed(seed, 1));
    std::vector<double> cdf(n);
    double acc = 0;
    for (int32_t k = 0; k < n; ++k) { acc += std::pow((double)(k + 1), -alpha); cdf[k] = acc; }
    const double total = acc;
    // out-degree: failures before the first success of a Bernoulli(p) with
    // p = 1/(1+mean), so E[deg] = (1-p)/p = mean
    const double p = 1.0 / (1.0 + mean_deg);
    // r.next() >= p_thresh is a failure; p == 1 (mean 0) never fails
    const uint64_t p_thresh = p >= 1.0 ? ~0ULL : (uint64_t)std::ldexp(p, 64);
    const int64_t chunk = 4096;
    const int64_t nchunks = (n + chunk - 1) / chunk;
    std::vector<std::vector<int32_t>> rows(nchunks), degs(nchunks);
    parallel_for(nchunks, [&](int64_t lo, int64_t hi) {
        for (int64_t c = lo; c < hi; ++c) {
            Rng r(mix_seed(seed, 1000 + (uint64_t)c));
            int32_t u0 = (int32_t)(c * chunk), u1 = (int32_t)std::min<int64_t>(n, (c + 1) * chunk);
            auto& cols = rows[c];
            auto& dg = degs[c];
            std::vector<int32_t> picked;
            for (int32_t u = u0; u < u1; ++u) {
                int64_t d = 0;
                if (p_thresh != ~0ULL)
                    while (r.next() >= p_thresh) ++d;
                if (d > n - 1) d = n - 1;
                picked.clear();
                for (int64_t j = 0; j < d; ++j) {
                    int32_t v = -1;
                    for (int tries = 0;; ++tries) {
                        if (tries < 4096) {
                            double x = r.uniform() * total;
                            int32_t k = (int32_t)(std::upper_bound(cdf.begin(), cdf.end(), x) - cdf.begin());
                            if (k >= n) k = n - 1;
                            v = perm[k];
                        } else {  // pathological tail: uniform redraw keeps the loop finite
                            v = (int32_t)r.below((uint64_t)n);
                        }
                        if (v == u) continue;
                        if (std::find(picked.begin(), picked.end(), v) != picked.end()) continue;
                        break;
                    }
                    picked.push_back(v);
                }
                cols.insert(cols.end(), picked.begin(), picked.end());
                dg.push_back((int32_t)picked.size());
            }
        }
    }, 1);
    int64_t e = 0;
    for (auto& c : rows) e += (int64_t)c.size();
    out->n = n;
    out->e = e;
    out->source = 0;
    out->offsets = (int32_t*)malloc(sizeof(int32_t) * ((size_t)n + 1));
    out->cols = (int32_t*)malloc(sizeof(int32_t) * (size_t)(e > 0 ? e : 1));
    if (!out->offsets || !out->cols) { dfq_csr_free(out); return fail(DFQ_ENOMEM, "zipf: allocation failed"); }
    int64_t w = 0;
    int32_t u = 0;
    out->offsets[0] = 0;
    for (int64_t c = 0; c < nchunks; ++c) {
        memcpy(out->cols + w, rows[c].data(), sizeof(int32_t) * rows[c].size());
        w += (int64_t)rows[c].size();
        for (int32_t d : degs[c]) { out->offsets[u + 1] = out->offsets[u] + d; ++u; }
    }
    return DFQ_OK;
}

int dfq_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                 int32_t flags, dfq_csr* out) {
    clear_error();
    if (!out || scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1)
        return fail(DFQ_EINVAL, "dfq_gen_rmat: bad arguments");
    memset(out, 0, sizeof *out);
    const int32_t n = (int32_t)1 << scale;
    const int64_t m = (int64_t)edge_factor << scale;
    // quadrant thresholds on a 32-bit uniform: [0,A) -> a, [A,AB) -> b, [AB,ABC) -> c, else d
    const uint64_t A = (uint64_t)std::ldexp(a, 32), AB = (uint64_t)std::ldexp(a + b, 32),
                   ABC = (uint64_t)std::ldexp(a + b + c, 32);
    std::vector<int32_t> perm = permutation(n, mix_seed(seed, 2));
    std::vector<int32_t> src(m), dst(m);
    const int64_t chunk = 1 << 16;
    const int64_t nchunks = (m + chunk - 1) / chunk;
    parallel_for(nchunks, [&](int64_t lo, int64_t hi) {
        for (int64_t ch = lo; ch < hi; ++ch) {
            Rng r(mix_seed(seed, 1000000 + (uint64_t)ch));
            int64_t i0 = ch * chunk, i1 = std::min<int64_t>(m, (ch + 1) * chunk);
            for (int64_t i = i0; i < i1; ++i) {
                uint32_t u = 0, v = 0;
                uint64_t word = 0;
                for (int l = 0; l < scale; ++l) {
                    uint64_t x;
                    if (l & 1) x = word >> 32;
                    else { word = r.next(); x = word & 0xffffffffULL; }
                    uint32_t bu = x >= AB, bv = (x >= A && x < AB) || x >= ABC;
                    u = (u << 1) | bu;
                    v = (v << 1) | bv;
                }
                src[i] = perm[u];
                dst[i] = perm[v];
            }
        }
    }, 1);
    return dfq_csr_from_edges(src.data(), dst.data(), m, n, flags, out);
}

int dfq_gen_grid(int32_t side, double delete_frac, uint64_t seed, int32_t keep_lcc, dfq_csr* out,
                 int32_t** orig_ids) {
    clear_error();
    if (!out || side < 1 || side > 46340 || delete_frac < 0 || delete_frac > 1)
        return fail(DFQ_EINVAL, "dfq_gen_grid: bad arguments");
    memset(out, 0, sizeof *out);
    if (orig_ids) *orig_ids = nullptr;
    const int64_t nv = (int64_t)side * side;
    // undirected edge ids: horizontal (r,c)-(r,c+1) -> r*(side-1)+c,
    // vertical (r,c)-(r+1,c) -> side*(side-1) + r*side + c
    const int64_t nh = (int64_t)side * (side - 1);
    const uint64_t thr = (uint64_t)std::ldexp(delete_frac, 64);
    auto kept = [&](int64_t id) {
        if (delete_frac <= 0) return true;
        if (delete_frac >= 1) return false;
        uint64_t s = seed ^ 0x6a09e667f3bcc909ULL;
        uint64_t h = mix_seed(s, (uint64_t)id);
        return h >= thr;
    };
    auto right_ok = [&](int64_t r, int64_t c) { return c + 1 < side && kept(r * (side - 1) + c); };
    auto down_ok = [&](int64_t r, int64_t c) { return r + 1 < side && kept(nh + r * side + c); };
    std::vector<int32_t> keep(nv, 1);
    if (keep_lcc) {
        UnionFind uf((int32_t)nv);
        for (int64_t r = 0; r < side; ++r)
            for (int64_t c = 0; c < side; ++c) {
                int64_t v = r * side + c;
                if (right_ok(r, c)) uf.unite((int32_t)v, (int32_t)(v + 1));
                if (down_ok(r, c)) uf.unite((int32_t)v, (int32_t)(v + side));
            }
        std::vector<int32_t> cnt(nv, 0);
        for (int64_t v = 0; v < nv; ++v) cnt[uf.find((int32_t)v)]++;
        int32_t best = 0;
        for (int64_t v = 0; v < nv; ++v) if (cnt[v] > cnt[best]) best = (int32_t)v;
        for (int64_t v = 0; v < nv; ++v) keep[v] = uf.find((int32_t)v) == best;
    }
    std::vector<int32_t> newid(nv, -1);
    int32_t n = 0;
    for (int64_t v = 0; v < nv; ++v) if (keep[v]) newid[v] = n++;
    std::vector<int32_t> off((size_t)n + 1, 0);
    std::vector<int32_t> cols;
    cols.reserve((size_t)n * 4);
    for (int64_t r = 0; r < side; ++r)
        for (int64_t c = 0; c < side; ++c) {
            int64_t v = r * side + c;
            if (newid[v] < 0) continue;
            // neighbours in increasing id order: up, left, right, down
            if (r > 0 && down_ok(r - 1, c) && newid[v - side] >= 0) cols.push_back(newid[v - side]);
            if (c > 0 && right_ok(r, c - 1) && newid[v - 1] >= 0) cols.push_back(newid[v - 1]);
            if (right_ok(r, c) && newid[v + 1] >= 0) cols.push_back(newid[v + 1]);
            if (down_ok(r, c) && newid[v + side] >= 0) cols.push_back(newid[v + side]);
            off[newid[v] + 1] = (int32_t)cols.size();
        }
    out->n = n;
    out->e = (int64_t)cols.size();
    out->source = 0;
    out->offsets = (int32_t*)malloc(sizeof(int32_t) * ((size_t)n + 1));
    out->cols = (int32_t*)malloc(sizeof(int32_t) * (cols.empty() ? 1 : cols.size()));
    if (!out->offsets || !out->cols) { dfq_csr_free(out); return fail(DFQ_ENOMEM, "grid: allocation failed"); }
    memcpy(out->offsets, off.data(), sizeof(int32_t) * ((size_t)n + 1));
    if (!cols.empty()) memcpy(out->cols, cols.data(), sizeof(int32_t) * cols.size());
    if (orig_ids) {
        int32_t* o = (int32_t*)malloc(sizeof(int32_t) * (n ? n : 1));
        if (!o) { dfq_csr_free(out); return fail(DFQ_ENOMEM, "grid: allocation failed"); }
        for (int64_t v = 0; v < nv; ++v) if (newid[v] >= 0) o[newid[v]] = (int32_t)v;
        *orig_ids = o;
    }
    return DFQ_OK;
}

int dfq_pick_sources(const dfq_csr* g, int32_t k, uint64_t seed, int32_t* out) {
    clear_error();
    if (!g || !out || k < 0) return fail(DFQ_EINVAL, "dfq_pick_sources: bad arguments");
    std::vector<int32_t> cand;
    for (int32_t u = 0; u < g->n; ++u) if (g->offsets[u + 1] > g->offsets[u]) cand.push_back(u);
    if (cand.empty()) return fail(DFQ_EINVAL, "graph has no vertex with out-degree > 0");
    Rng r(mix_seed(seed, 3));
    if ((size_t)k <= cand.size()) {  // distinct: partial Fisher-Yates
        for (int32_t i = 0; i < k; ++i) {
            size_t j = i + (size_t)r.below(cand.size() - i);
            std::swap(cand[i], cand[j]);
            out[i] = cand[i];
        }
    } else {
        for (int32_t i = 0; i < k; ++i) out[i] = cand[r.below(cand.size())];
    }
    return DFQ_OK;
}

}  // extern "C"
