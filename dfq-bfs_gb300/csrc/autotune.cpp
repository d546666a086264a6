// Autotuner for the per-graph kernel options.  No reference counterpart: the
// reference fixes bin thresholds, tile sizes and queue capacities with
// #defines per program (bfs.cu:16-36) and compared hand-picked settings
// offline (com-orkut_8-64-1024-16384-all and its siblings).  Here the options
// are searched per graph by coordinate descent, timing real launches.
#include "common.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
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
        // not searched: l2_persist (the bitmap is L2-resident without it: on
        // GB300 neither time nor the L2 hit rate moved) and blocks_per_sm (one
        // block per SM measured 6-24 % slower on R-MAT and grids)
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

// ------------------------------------------------------------ cached results
namespace {

struct OptName {
    const char* name;
    int32_t dfq_opts::*field;
};
// every field of dfq_opts a tuned entry stores (the test hooks are not tuned)
const OptName kStored[] = {
    {"block_threads", &dfq_opts::block_threads},       {"blocks_per_sm", &dfq_opts::blocks_per_sm},
    {"medium_min_degree", &dfq_opts::medium_min_degree}, {"large_min_degree", &dfq_opts::large_min_degree},
    {"local_queue_cap", &dfq_opts::local_queue_cap},   {"local_edge_budget", &dfq_opts::local_edge_budget},
    {"piece_edges", &dfq_opts::piece_edges},           {"probe_first", &dfq_opts::probe_first},
    {"l2_persist", &dfq_opts::l2_persist},             {"use_tma", &dfq_opts::use_tma},
    {"timeout_ms", &dfq_opts::timeout_ms},             {"wide_min_edges", &dfq_opts::wide_min_edges},
    {"wide_min_degree", &dfq_opts::wide_min_degree},   {"hot_cache", &dfq_opts::hot_cache},
    {"vertex_order", &dfq_opts::vertex_order},         {"direction", &dfq_opts::direction},
};

struct CacheEntry {
    std::string gpu, cls;
    dfq_opts o{};
};

// The current device as "name|SMs|major.minor": tuned options carry over only
// between identical GPUs.
std::string gpu_key() {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
    char buf[320];
    snprintf(buf, sizeof buf, "%s|%d|%d.%d", prop.name, prop.multiProcessorCount, prop.major, prop.minor);
    return buf;
}

// Read a JSON string whose opening quote is s[i]; returns the index after it.
size_t read_string(const std::string& s, size_t i, std::string& out) {
    out.clear();
    if (i >= s.size() || s[i] != '"') return std::string::npos;
    for (++i; i < s.size() && s[i] != '"'; ++i) {
        if (s[i] == '\\' && i + 1 < s.size()) ++i;
        out.push_back(s[i]);
    }
    return i < s.size() ? i + 1 : std::string::npos;
}

size_t skip_sep(const std::string& s, size_t i) {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\t' || s[i] == '\r' || s[i] == ':' || s[i] == ','))
        ++i;
    return i;
}

// Entries of a cache file written by write_cache (unknown keys are skipped; a
// missing or unreadable file is an empty cache).
std::vector<CacheEntry> read_cache(const char* path) {
    std::vector<CacheEntry> out;
    FILE* f = fopen(path, "rb");
    if (!f) return out;
    std::string s;
    char buf[4096];
    size_t k;
    while ((k = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, k);
    fclose(f);
    size_t i = 0;
    while ((i = s.find("{\"gpu\"", i)) != std::string::npos) {
        const size_t opts_at = s.find("\"opts\"", i);
        if (opts_at == std::string::npos) break;
        size_t end = s.find('}', opts_at);              // closes "opts"
        if (end != std::string::npos) end = s.find('}', end + 1);  // closes the entry
        if (end == std::string::npos) break;
        CacheEntry e;
        dfq_opts_default(&e.o);
        size_t j = i + 1;
        while (j < end) {
            j = skip_sep(s, j);
            if (j >= end) break;
            if (s[j] != '"') { ++j; continue; }
            std::string key;
            j = read_string(s, j, key);
            if (j == std::string::npos) break;
            j = skip_sep(s, j);
            if (key == "gpu" || key == "class") {
                std::string v;
                j = read_string(s, j, v);
                if (j == std::string::npos) break;
                (key == "gpu" ? e.gpu : e.cls) = v;
            } else {
                for (const OptName& f : kStored)
                    if (key == f.name) e.o.*(f.field) = (int32_t)strtol(s.c_str() + j, nullptr, 10);
            }
        }
        if (!e.gpu.empty() && !e.cls.empty()) out.push_back(e);
        i = end + 1;
    }
    return out;
}

int write_cache(const char* path, const std::vector<CacheEntry>& es) {
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "wb");
    if (!f) return fail(DFQ_EIO, "cannot write autotune cache '%s'", tmp.c_str());
    fprintf(f, "{\"version\": 1, \"entries\": [\n");
    for (size_t k = 0; k < es.size(); ++k) {
        const CacheEntry& e = es[k];
        fprintf(f, "  {\"gpu\": \"%s\", \"class\": \"%s\", \"opts\": {", e.gpu.c_str(), e.cls.c_str());
        for (size_t q = 0; q < sizeof kStored / sizeof kStored[0]; ++q)
            fprintf(f, "%s\"%s\": %d", q ? ", " : "", kStored[q].name, (int)(e.o.*(kStored[q].field)));
        fprintf(f, "}}%s\n", k + 1 < es.size() ? "," : "");
    }
    fprintf(f, "]}\n");
    if (fclose(f) != 0) return fail(DFQ_EIO, "cannot write autotune cache '%s'", tmp.c_str());
    if (rename(tmp.c_str(), path) != 0) return fail(DFQ_EIO, "cannot replace autotune cache '%s'", path);
    return DFQ_OK;
}

}  // namespace

extern "C" int dfq_graph_class(const dfq_graph* g, char* buf, int32_t len) {
    clear_error();
    if (!g || !buf || len < 1) return fail(DFQ_EINVAL, "dfq_graph_class: bad arguments");
    const int32_t n = std::max<int32_t>(dfq_graph_num_vertices(g), 1);
    const int64_t e = dfq_graph_num_edges(g);
    const int ln = (int)std::lround(std::log2((double)n));
    const int ld = (int)std::lround(std::log2(std::max(1.0, (double)e / n)));
    const int k = snprintf(buf, (size_t)len, "%s-n2^%d-d2^%d", dfq_graph_is_hub_first(g) == 1 ? "skewed" : "even", ln, ld);
    return k < len ? k : fail(DFQ_EINVAL, "dfq_graph_class: buffer of %d bytes is too small", len);
}

extern "C" int dfq_autotune_cached(dfq_graph* g, const int32_t* sources, int32_t nsrc, const char* cache_path,
                                   dfq_opts* best, int32_t* hit) {
    clear_error();
    if (!g || !sources || nsrc < 1 || !best || !cache_path)
        return fail(DFQ_EINVAL, "dfq_autotune_cached: bad arguments");
    char cls[128];
    int rc = dfq_graph_class(g, cls, sizeof cls);
    if (rc < 0) return rc;
    const std::string gpu = gpu_key();
    std::vector<CacheEntry> es = read_cache(cache_path);
    for (const CacheEntry& e : es)
        if (e.gpu == gpu && e.cls == cls) {
            dfq_opts cur;
            dfq_graph_get_opts(g, &cur);
            dfq_opts o = e.o;
            o.profile = cur.profile;
            o.stall_test_level = 0;
            o.direction = cur.direction;  // a property of how the graph was created
            if (dfq_graph_set_opts(g, &o) != DFQ_OK) break;  // an unusable entry: tune again
            *best = o;
            if (hit) *hit = 1;
            return DFQ_OK;
        }
    if (hit) *hit = 0;
    if ((rc = dfq_autotune(g, sources, nsrc, best)) != DFQ_OK) return rc;
    es.erase(std::remove_if(es.begin(), es.end(), [&](const CacheEntry& e) { return e.gpu == gpu && e.cls == cls; }),
             es.end());
    CacheEntry ne;
    ne.gpu = gpu;
    ne.cls = cls;
    ne.o = *best;
    es.push_back(ne);
    return write_cache(cache_path, es);
}
