// Host-side graph substrate of libdfq: CSR construction, the reference's .dat
// format, SNAP edge lists and a binary CSR cache.
//
// Reference behaviour kept:
//   * .dat input (design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu:187-199):
//     "N E SOURCE", then N pairs "start length" (Node AoS, :38-42), then E pairs
//     "dst <ignored>".  The source comes from the header (:188).
//   * SNAP edge list documented in README.md:19-32 ("# Nodes: N Edges: E",
//     "# FromNodeId ToNodeId", then "u v" lines).  The reference's converter to
//     .dat is not in its repository; here SNAP is read directly.
#include "common.hpp"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>

namespace dfq {

static thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}
void clear_error() { g_err.clear(); }

int host_threads() {
    static int t = [] {
        const char* env = getenv("DFQ_HOST_THREADS");
        int v = env ? atoi(env) : 0;
        if (v <= 0) v = (int)std::thread::hardware_concurrency();
        if (v <= 0) v = 1;
        if (v > 64) v = 64;
        return v;
    }();
    return t;
}

// ------------------------------------------------------------------ CSR build
static int alloc_csr(int32_t n, int64_t e, dfq_csr* out) {
    out->n = n;
    out->e = e;
    out->source = 0;
    out->offsets = (int32_t*)malloc(sizeof(int32_t) * ((size_t)n + 1));
    out->cols = (int32_t*)malloc(sizeof(int32_t) * (size_t)(e > 0 ? e : 1));
    if (!out->offsets || !out->cols) {
        free(out->offsets);
        free(out->cols);
        out->offsets = out->cols = nullptr;
        return fail(DFQ_ENOMEM, "host allocation of CSR (n=%d, e=%lld) failed", n, (long long)e);
    }
    return DFQ_OK;
}

// Sort and de-duplicate each row in place, then compact.  Rows are processed
// in parallel; the compaction prefix is computed serially in row order, so the
// output does not depend on the thread count.
static void dedup_rows(dfq_csr* g) {
    const int32_t n = g->n;
    std::vector<int32_t> newdeg(n);
    int32_t* off = g->offsets;
    int32_t* col = g->cols;
    parallel_for(n, [&](int64_t lo, int64_t hi) {
        for (int64_t u = lo; u < hi; ++u) {
            int32_t* b = col + off[u];
            int32_t* e = col + off[u + 1];
            std::sort(b, e);
            newdeg[u] = (int32_t)(std::unique(b, e) - b);
        }
    }, 1 << 12);
    int64_t w = 0;
    for (int32_t u = 0; u < n; ++u) {
        int32_t b = off[u];
        int32_t d = newdeg[u];
        off[u] = (int32_t)w;
        if (w != b) memmove(col + w, col + b, sizeof(int32_t) * d);
        w += d;
    }
    off[n] = (int32_t)w;
    g->e = w;
}

}  // namespace dfq

using namespace dfq;

extern "C" {

const char* dfq_last_error(void) { return g_err.c_str(); }

void dfq_free(void* p) { free(p); }

void dfq_csr_free(dfq_csr* g) {
    if (!g) return;
    free(g->offsets);
    free(g->cols);
    memset(g, 0, sizeof *g);
}

int dfq_csr_from_edges(const int32_t* src, const int32_t* dst, int64_t m, int32_t n,
                       int32_t flags, dfq_csr* out) {
    clear_error();
    if (!out || (m > 0 && (!src || !dst)) || n < 0 || m < 0)
        return fail(DFQ_EINVAL, "dfq_csr_from_edges: bad arguments");
    memset(out, 0, sizeof *out);
    const bool sym = flags & DFQ_CSR_SYMMETRIZE;
    const bool noself = flags & DFQ_CSR_NO_SELF_LOOPS;
    // validate ids
    std::atomic<int64_t> bad{-1};
    parallel_for(m, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i)
            if ((uint32_t)src[i] >= (uint32_t)n || (uint32_t)dst[i] >= (uint32_t)n) {
                int64_t exp = -1;
                bad.compare_exchange_strong(exp, i);
                return;
            }
    });
    if (bad.load() >= 0) {
        int64_t i = bad.load();
        return fail(DFQ_EFORMAT, "edge %lld (%d -> %d) has an id outside [0, %d)", (long long)i,
                    src[i], dst[i], n);
    }
    std::vector<int64_t> deg((size_t)n + 1, 0);
    for (int64_t i = 0; i < m; ++i) {
        if (noself && src[i] == dst[i]) continue;
        deg[src[i]]++;
        if (sym) deg[dst[i]]++;
    }
    int64_t total = 0;
    for (int32_t u = 0; u < n; ++u) { int64_t d = deg[u]; deg[u] = total; total += d; }
    deg[n] = total;
    if (total >= ((int64_t)1 << 31))
        return fail(DFQ_EINVAL, "graph has %lld directed edges; int32 offsets need < 2^31",
                    (long long)total);
    int rc = alloc_csr(n, total, out);
    if (rc) return rc;
    for (int32_t u = 0; u <= n; ++u) out->offsets[u] = (int32_t)deg[u];
    // stable fill: for each source, neighbours in input order (reverse edges
    // interleave at the position of the edge that produced them)
    for (int64_t i = 0; i < m; ++i) {
        int32_t u = src[i], v = dst[i];
        if (noself && u == v) continue;
        out->cols[deg[u]++] = v;
        if (sym) out->cols[deg[v]++] = u;
    }
    if (flags & DFQ_CSR_DEDUP) dedup_rows(out);
    return DFQ_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ text I/O
namespace {

struct Buf {
    char* p = nullptr;
    size_t n = 0;
    ~Buf() { free(p); }
};

int read_file(const char* path, Buf& b) {
    FILE* f = fopen(path, "rb");
    if (!f) return fail(DFQ_EIO, "cannot open '%s': %s", path, strerror(errno));
    if (fseek(f, 0, SEEK_END) != 0) { fclose(f); return fail(DFQ_EIO, "cannot seek '%s'", path); }
    long sz = ftell(f);
    if (sz < 0) { fclose(f); return fail(DFQ_EIO, "cannot size '%s'", path); }
    fseek(f, 0, SEEK_SET);
    b.p = (char*)malloc((size_t)sz + 1);
    if (!b.p) { fclose(f); return fail(DFQ_ENOMEM, "cannot buffer %ld bytes of '%s'", sz, path); }
    size_t got = fread(b.p, 1, (size_t)sz, f);
    fclose(f);
    if (got != (size_t)sz) return fail(DFQ_EIO, "short read on '%s'", path);
    b.p[sz] = 0;
    b.n = (size_t)sz;
    return DFQ_OK;
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

// Cursor over a NUL-terminated buffer that reads whitespace-separated integers.
struct Cursor {
    const char* p;
    const char* end;
    void skip_space() { while (p < end && is_space(*p)) ++p; }
    // 0 ok, 1 end of input, -1 not an integer / overflow
    int next_int(int64_t& v) {
        skip_space();
        if (p >= end) return 1;
        bool neg = false;
        if (*p == '-' || *p == '+') { neg = (*p == '-'); ++p; }
        if (p >= end || *p < '0' || *p > '9') return -1;
        int64_t x = 0;
        while (p < end && *p >= '0' && *p <= '9') {
            x = x * 10 + (*p - '0');
            if (x > ((int64_t)1 << 40)) return -1;
            ++p;
        }
        if (p < end && !is_space(*p)) return -1;
        v = neg ? -x : x;
        return 0;
    }
    void skip_line() { while (p < end && *p != '\n') ++p; if (p < end) ++p; }
};

int parse_dat(const Buf& b, const char* path, dfq_csr* out) {
    Cursor c{b.p, b.p + b.n};
    int64_t n, e, s;
    if (c.next_int(n) || c.next_int(e) || c.next_int(s))
        return fail(DFQ_EFORMAT, "%s: .dat header must be 'N E SOURCE'", path);
    if (n < 0 || n >= ((int64_t)1 << 31) || e < 0 || e >= ((int64_t)1 << 31))
        return fail(DFQ_EFORMAT, "%s: header N=%lld E=%lld out of range", path, (long long)n, (long long)e);
    std::vector<int32_t> start(n), len(n);
    bool plain = true;  // rows already laid out back to back from 0?
    int64_t run = 0;
    for (int64_t i = 0; i < n; ++i) {
        int64_t st, ln;
        if (c.next_int(st) || c.next_int(ln))
            return fail(DFQ_EFORMAT, "%s: node record %lld missing or malformed", path, (long long)i);
        if (st < 0 || ln < 0 || st + ln > e)
            return fail(DFQ_EFORMAT, "%s: node %lld has start=%lld length=%lld outside E=%lld", path,
                        (long long)i, (long long)st, (long long)ln, (long long)e);
        start[i] = (int32_t)st;
        len[i] = (int32_t)ln;
        if (st != run) plain = false;
        run = st + ln;
    }
    if (run != e) plain = false;
    std::vector<int32_t> edge(e > 0 ? e : 1);
    for (int64_t i = 0; i < e; ++i) {
        int64_t d, ignored;
        if (c.next_int(d) || c.next_int(ignored))
            return fail(DFQ_EFORMAT, "%s: edge record %lld missing or malformed", path, (long long)i);
        if (d < 0 || d >= n)
            return fail(DFQ_EFORMAT, "%s: edge %lld targets %lld outside [0,%lld)", path, (long long)i,
                        (long long)d, (long long)n);
        edge[i] = (int32_t)d;
    }
    if (s < 0 || s >= n) s = 0;  // the reference re-prompts instead (DFQ:204-214)
    int64_t total = 0;
    for (int64_t i = 0; i < n; ++i) total += len[i];
    int rc = alloc_csr((int32_t)n, total, out);
    if (rc) return rc;
    out->source = (int32_t)s;
    out->offsets[0] = 0;
    for (int64_t i = 0; i < n; ++i) out->offsets[i + 1] = out->offsets[i] + len[i];
    if (plain) {
        memcpy(out->cols, edge.data(), sizeof(int32_t) * total);
    } else {  // arbitrary (start, length) records: gather rows in vertex order
        for (int64_t i = 0; i < n; ++i)
            memcpy(out->cols + out->offsets[i], edge.data() + start[i], sizeof(int32_t) * len[i]);
    }
    return DFQ_OK;
}

// "# Nodes: N Edges: E" -> N, E (returns false if the line is not that header)
bool parse_nodes_header(const char* p, const char* end, int64_t& n, int64_t& e) {
    const char* q = p;
    auto find = [&](const char* key) -> const char* {
        size_t k = strlen(key);
        for (const char* r = q; r + k <= end && *r != '\n'; ++r)
            if (strncmp(r, key, k) == 0) return r + k;
        return nullptr;
    };
    const char* a = find("Nodes:");
    const char* b = find("Edges:");
    if (!a) return false;
    n = strtoll(a, nullptr, 10);
    e = b ? strtoll(b, nullptr, 10) : -1;
    return true;
}

int parse_snap(const Buf& b, const char* path, int32_t flags, dfq_csr* out) {
    Cursor c{b.p, b.p + b.n};
    int64_t hdr_n = -1, hdr_e = -1;
    std::vector<int32_t> src, dst;
    int64_t maxid = -1;
    int64_t line = 0;
    while (true) {
        c.skip_space();
        if (c.p >= c.end) break;
        if (*c.p == '#') {
            int64_t nn, ee;
            if (hdr_n < 0 && parse_nodes_header(c.p, c.end, nn, ee)) {
                hdr_n = nn;
                hdr_e = ee;
                if (hdr_e > 0 && hdr_e < ((int64_t)1 << 31)) { src.reserve(hdr_e); dst.reserve(hdr_e); }
            }
            c.skip_line();
            continue;
        }
        int64_t u, v;
        ++line;
        if (c.next_int(u) || c.next_int(v))
            return fail(DFQ_EFORMAT, "%s: edge line %lld is not 'FromNodeId ToNodeId'", path, (long long)line);
        if (u < 0 || v < 0 || u >= ((int64_t)1 << 31) - 1 || v >= ((int64_t)1 << 31) - 1)
            return fail(DFQ_EFORMAT, "%s: edge line %lld has id out of int32 range", path, (long long)line);
        // anything after the two ids on the line (weights, timestamps) is ignored
        while (c.p < c.end && *c.p != '\n') ++c.p;
        src.push_back((int32_t)u);
        dst.push_back((int32_t)v);
        if (u > maxid) maxid = u;
        if (v > maxid) maxid = v;
    }
    int64_t n = hdr_n > 0 ? hdr_n : 0;
    if (maxid + 1 > n) n = maxid + 1;  // SNAP ids may exceed the header's count
    if (n >= ((int64_t)1 << 31)) return fail(DFQ_EFORMAT, "%s: too many vertices", path);
    return dfq_csr_from_edges(src.data(), dst.data(), (int64_t)src.size(), (int32_t)n, flags, out);
}

int read_bin(const Buf& b, const char* path, dfq_csr* out) {
    const size_t hdr = 8 + 4 + 4 + 8;
    if (b.n < hdr || memcmp(b.p, "DFQCSR01", 8) != 0)
        return fail(DFQ_EFORMAT, "%s: not a DFQCSR01 file", path);
    int32_t n, s;
    int64_t e;
    memcpy(&n, b.p + 8, 4);
    memcpy(&s, b.p + 12, 4);
    memcpy(&e, b.p + 16, 8);
    if (n < 0 || e < 0 || b.n != hdr + 4 * ((size_t)n + 1) + 4 * (size_t)e)
        return fail(DFQ_EFORMAT, "%s: DFQCSR01 size does not match its header", path);
    int rc = alloc_csr(n, e, out);
    if (rc) return rc;
    out->source = s;
    memcpy(out->offsets, b.p + hdr, 4 * ((size_t)n + 1));
    memcpy(out->cols, b.p + hdr + 4 * ((size_t)n + 1), 4 * (size_t)e);
    // validate
    if (out->offsets[0] != 0 || out->offsets[n] != e) { dfq_csr_free(out); return fail(DFQ_EFORMAT, "%s: bad offsets", path); }
    for (int32_t u = 0; u < n; ++u)
        if (out->offsets[u + 1] < out->offsets[u]) { dfq_csr_free(out); return fail(DFQ_EFORMAT, "%s: offsets decrease at %d", path, u); }
    for (int64_t i = 0; i < e; ++i)
        if ((uint32_t)out->cols[i] >= (uint32_t)n) { dfq_csr_free(out); return fail(DFQ_EFORMAT, "%s: column %lld out of range", path, (long long)i); }
    return DFQ_OK;
}

// Fast integer formatting into a growing buffer.
struct Out {
    std::vector<char> v;
    void put(const char* s) { v.insert(v.end(), s, s + strlen(s)); }
    void put_int(int64_t x) {
        char t[24];
        int k = 0;
        bool neg = x < 0;
        uint64_t u = neg ? (uint64_t)(-x) : (uint64_t)x;
        do { t[k++] = (char)('0' + u % 10); u /= 10; } while (u);
        if (neg) v.push_back('-');
        while (k) v.push_back(t[--k]);
    }
    void ch(char c) { v.push_back(c); }
};

int write_all(const char* path, const void* p, size_t n) {
    FILE* f = fopen(path, "wb");
    if (!f) return fail(DFQ_EIO, "cannot create '%s': %s", path, strerror(errno));
    size_t w = fwrite(p, 1, n, f);
    int cl = fclose(f);
    if (w != n || cl != 0) return fail(DFQ_EIO, "short write on '%s'", path);
    return DFQ_OK;
}

}  // namespace

extern "C" {

int dfq_csr_load(const char* path, int32_t format, int32_t flags, dfq_csr* out) {
    clear_error();
    if (!path || !out) return fail(DFQ_EINVAL, "dfq_csr_load: null argument");
    memset(out, 0, sizeof *out);
    Buf b;
    int rc = read_file(path, b);
    if (rc) return rc;
    if (format == DFQ_FMT_AUTO) {
        size_t i = 0;
        while (i < b.n && is_space(b.p[i])) ++i;
        if (b.n >= 8 && memcmp(b.p, "DFQCSR01", 8) == 0) format = DFQ_FMT_BIN;
        else if (i < b.n && b.p[i] == '#') format = DFQ_FMT_SNAP;
        else format = DFQ_FMT_DAT;
    }
    switch (format) {
        case DFQ_FMT_SNAP: return parse_snap(b, path, flags, out);
        case DFQ_FMT_DAT: rc = parse_dat(b, path, out); break;
        case DFQ_FMT_BIN: rc = read_bin(b, path, out); break;
        default: return fail(DFQ_EINVAL, "unknown format %d", format);
    }
    if (rc == DFQ_OK && (flags & (DFQ_CSR_SYMMETRIZE | DFQ_CSR_DEDUP | DFQ_CSR_NO_SELF_LOOPS))) {
        // re-run the edge list through the builder so flags mean the same for every format
        std::vector<int32_t> s(out->e), d(out->e);
        for (int32_t u = 0; u < out->n; ++u)
            for (int32_t k = out->offsets[u]; k < out->offsets[u + 1]; ++k) { s[k] = u; d[k] = out->cols[k]; }
        int32_t src = out->source, n = out->n;
        dfq_csr_free(out);
        rc = dfq_csr_from_edges(s.data(), d.data(), (int64_t)s.size(), n, flags, out);
        if (rc == DFQ_OK) out->source = src;
    }
    return rc;
}

int dfq_csr_save(const char* path, const dfq_csr* g, int32_t format) {
    clear_error();
    if (!path || !g || (g->n > 0 && !g->offsets) || (g->e > 0 && !g->cols))
        return fail(DFQ_EINVAL, "dfq_csr_save: bad arguments");
    if (format == DFQ_FMT_BIN) {
        std::vector<char> v(24 + 4 * ((size_t)g->n + 1) + 4 * (size_t)g->e);
        memcpy(v.data(), "DFQCSR01", 8);
        memcpy(v.data() + 8, &g->n, 4);
        memcpy(v.data() + 12, &g->source, 4);
        memcpy(v.data() + 16, &g->e, 8);
        memcpy(v.data() + 24, g->offsets, 4 * ((size_t)g->n + 1));
        if (g->e) memcpy(v.data() + 24 + 4 * ((size_t)g->n + 1), g->cols, 4 * (size_t)g->e);
        return write_all(path, v.data(), v.size());
    }
    Out o;
    o.v.reserve((size_t)g->e * 16 + (size_t)g->n * 16 + 128);
    if (format == DFQ_FMT_SNAP) {
        o.put("# Nodes: "); o.put_int(g->n); o.put(" Edges: "); o.put_int(g->e); o.ch('\n');
        o.put("# FromNodeId\tToNodeId\n");
        for (int32_t u = 0; u < g->n; ++u)
            for (int32_t k = g->offsets[u]; k < g->offsets[u + 1]; ++k) {
                o.put_int(u); o.ch('\t'); o.put_int(g->cols[k]); o.ch('\n');
            }
    } else if (format == DFQ_FMT_DAT) {
        // the second column of the edge records is ignored by the reference
        // loader (DFQ:199); it is written as 1
        o.put_int(g->n); o.ch(' '); o.put_int(g->e); o.ch(' '); o.put_int(g->source); o.ch('\n');
        for (int32_t u = 0; u < g->n; ++u) {
            o.put_int(g->offsets[u]); o.ch(' '); o.put_int(g->offsets[u + 1] - g->offsets[u]); o.ch('\n');
        }
        for (int64_t k = 0; k < g->e; ++k) { o.put_int(g->cols[k]); o.put(" 1\n"); }
    } else {
        return fail(DFQ_EINVAL, "dfq_csr_save: unknown format %d", format);
    }
    return write_all(path, o.v.data(), o.v.size());
}

}  // extern "C"
