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
#include <new>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

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

static std::atomic<int> g_threads{0};  // 0: DFQ_HOST_THREADS or the hardware count

static int default_threads() {
    static const int t = [] {
        const char* env = getenv("DFQ_HOST_THREADS");
        int v = env ? atoi(env) : 0;
        if (v <= 0) v = (int)std::thread::hardware_concurrency();
        if (v <= 0) v = 1;
        return v > 64 ? 64 : v;
    }();
    return t;
}

int host_threads() {
    const int t = g_threads.load(std::memory_order_relaxed);
    return t > 0 ? t : default_threads();
}

// Pieces to cut `units` of work into: with a thread count set explicitly,
// that many (down to 16 units per piece, so small inputs still take the
// parallel path); by default one piece per `min_per_piece` units, at most one
// per host thread.
static int pieces_for(int64_t units, int64_t min_per_piece) {
    const int forced = g_threads.load(std::memory_order_relaxed);
    const int64_t want = forced > 0 ? std::max<int64_t>(1, units / 16) : std::max<int64_t>(1, units / min_per_piece);
    return (int)std::min<int64_t>(forced > 0 ? forced : default_threads(), want);
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

// Parallel stable counting sort by row over an edge list given as consecutive
// spans.  The list is cut into T chunks (whole spans when there are several,
// equal slices of the one span otherwise); hist[c][v] counts the entries chunk
// c adds to row v.  Row v receives chunk 0's entries first, then chunk 1's,
// ..., each chunk in input order: exactly the order of one serial pass, so the
// result does not depend on T.  T is bounded so the T x (n+1) histogram stays
// <= 1 GiB, and raised so no chunk can count 2^31 entries into one row.
int build_csr(const std::vector<EdgeSpan>& spans, int32_t n, int32_t flags, dfq_csr* out) {
    memset(out, 0, sizeof *out);
    const bool sym = flags & DFQ_CSR_SYMMETRIZE;
    const bool noself = flags & DFQ_CSR_NO_SELF_LOOPS;
    int64_t m = 0;
    for (const EdgeSpan& sp : spans) m += sp.m;
    const int64_t n1 = (int64_t)n + 1;
    int64_t T = pieces_for(m, 1 << 16);
    T = std::min<int64_t>(T, std::max<int64_t>(1, ((int64_t)1 << 28) / n1));
    T = std::max<int64_t>(T, (m + ((int64_t)1 << 29) - 1) >> 29);
    // chunk c = edges [cut[c], cut[c+1]) of the concatenated list
    std::vector<int64_t> cut{0};
    if (spans.size() > 1) {  // group whole spans, about m / T edges per chunk
        int64_t at = 0;
        for (size_t i = 0; i + 1 < spans.size(); ++i) {
            at += spans[i].m;
            if (at * T >= m * (int64_t)cut.size() && at > cut.back()) cut.push_back(at);
        }
        cut.push_back(m);
        T = (int64_t)cut.size() - 1;
    } else {
        for (int64_t c = 1; c <= T; ++c) cut.push_back(m * c / T);
    }
    if (T < 1) T = 1, cut = {0, m};
    // visit edges [lo, hi) of the concatenation in order
    std::vector<int64_t> span_at{0};
    for (const EdgeSpan& sp : spans) span_at.push_back(span_at.back() + sp.m);
    auto for_edges = [&](int64_t lo, int64_t hi, auto&& f) {
        size_t k = (size_t)(std::upper_bound(span_at.begin(), span_at.end(), lo) - span_at.begin()) - 1;
        for (; lo < hi && k < spans.size(); ++k) {
            const int64_t a = lo - span_at[k], b = std::min(hi, span_at[k + 1]) - span_at[k];
            for (int64_t i = a; i < b; ++i) f(spans[k].src[i], spans[k].dst[i]);
            lo = span_at[k + 1];
        }
    };
    // validate ids: report the first bad edge in list order
    std::vector<int64_t> bad((size_t)T, -1);
    run_threads((int)T, [&](int c) {
        int64_t i = cut[c];
        bool found = false;
        for_edges(cut[c], cut[c + 1], [&](int32_t u, int32_t v) {
            if (!found && ((uint32_t)u >= (uint32_t)n || (uint32_t)v >= (uint32_t)n)) { bad[c] = i; found = true; }
            ++i;
        });
    });
    for (int64_t c = 0; c < T; ++c)
        if (bad[c] >= 0) {
            int32_t u = 0, v = 0;
            for_edges(bad[c], bad[c] + 1, [&](int32_t a, int32_t b) { u = a; v = b; });
            return fail(DFQ_EFORMAT, "edge %lld (%d -> %d) has an id outside [0, %d)", (long long)bad[c], u, v, n);
        }
    std::vector<uint32_t> hist;
    try {
        hist.assign((size_t)(T * n1), 0u);
    } catch (const std::bad_alloc&) {
        return fail(DFQ_ENOMEM, "CSR build: no host memory for a %lld x %lld histogram", (long long)T,
                    (long long)n1);
    }
    run_threads((int)T, [&](int c) {
        uint32_t* h = hist.data() + (size_t)c * n1;
        for_edges(cut[c], cut[c + 1], [&](int32_t u, int32_t v) {
            if (noself && u == v) return;
            h[u]++;
            if (sym) h[v]++;
        });
    });
    std::vector<int64_t> deg((size_t)n1, 0);
    parallel_for(n, [&](int64_t lo, int64_t hi) {
        for (int64_t v = lo; v < hi; ++v) {
            int64_t d = 0;
            for (int64_t c = 0; c < T; ++c) d += hist[(size_t)(c * n1 + v)];
            deg[v] = d;
        }
    });
    int64_t total = 0;
    for (int32_t u = 0; u < n; ++u) { int64_t d = deg[u]; deg[u] = total; total += d; }
    deg[n] = total;
    if (total >= ((int64_t)1 << 31))
        return fail(DFQ_EINVAL, "graph has %lld directed edges; int32 offsets need < 2^31",
                    (long long)total);
    int rc = alloc_csr(n, total, out);
    if (rc) return rc;
    // hist[c][v] becomes the first position chunk c writes in row v
    parallel_for(n1, [&](int64_t lo, int64_t hi) {
        for (int64_t v = lo; v < hi; ++v) {
            out->offsets[v] = (int32_t)deg[v];
            uint32_t run = (uint32_t)deg[v];
            for (int64_t c = 0; c < T; ++c) {
                uint32_t& h = hist[(size_t)(c * n1 + v)];
                const uint32_t k = h;
                h = run;
                run += k;
            }
        }
    });
    run_threads((int)T, [&](int c) {
        uint32_t* pos = hist.data() + (size_t)c * n1;
        int32_t* col = out->cols;
        for_edges(cut[c], cut[c + 1], [&](int32_t u, int32_t v) {
            if (noself && u == v) return;
            col[pos[u]++] = v;
            if (sym) col[pos[v]++] = u;
        });
    });
    if (flags & DFQ_CSR_DEDUP) dedup_rows(out);
    return DFQ_OK;
}

int hub_first_csr(const dfq_csr& in, int mode, dfq_csr* out, std::vector<int32_t>* rank_out,
                  std::vector<int32_t>* order_out) {
    const int32_t n = in.n;
    const int64_t e = in.e;
    if (mode == 1 || n < 1 || e == 0) return 0;
    std::vector<int32_t> indeg((size_t)n, 0);
    for (int64_t k = 0; k < e; ++k) indeg[in.cols[k]]++;
    const int32_t mx = *std::max_element(indeg.begin(), indeg.end());
    if (mode == 0 && (n < (1 << 16) || (double)mx < 64.0 * ((double)e / (double)n))) return 0;
    std::vector<int32_t>& order = *order_out;
    std::vector<int32_t>& rank = *rank_out;
    order.resize(n);
    rank.resize(n);
    if ((int64_t)mx <= 4 * (int64_t)n + 1024) {  // stable counting sort by descending in-degree
        std::vector<int64_t> at((size_t)mx + 2, 0);
        for (int32_t v = 0; v < n; ++v) at[(size_t)(mx - indeg[v]) + 1]++;
        for (size_t k = 1; k < at.size(); ++k) at[k] += at[k - 1];
        for (int32_t v = 0; v < n; ++v) order[at[(size_t)(mx - indeg[v])]++] = v;
    } else {
        for (int32_t v = 0; v < n; ++v) order[v] = v;
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return indeg[a] > indeg[b]; });
    }
    for (int32_t i = 0; i < n; ++i) rank[order[i]] = i;
    int rc = alloc_csr(n, e, out);
    if (rc) return rc;
    out->source = in.source;
    out->offsets[0] = 0;
    for (int32_t i = 0; i < n; ++i) out->offsets[i + 1] = out->offsets[i] + (in.offsets[order[i] + 1] - in.offsets[order[i]]);
    parallel_for(n, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            const int32_t o = order[i];
            int32_t* row = out->cols + out->offsets[i];
            const int32_t d = in.offsets[o + 1] - in.offsets[o];
            int32_t best = 0;
            for (int32_t k = 0; k < d; ++k) {
                row[k] = rank[in.cols[in.offsets[o] + k]];
                if (row[k] < row[best]) best = k;
            }
            if (best > 0) std::swap(row[0], row[best]);
        }
    }, 1 << 12);
    return 1;
}

}  // namespace dfq

using namespace dfq;

extern "C" {

const char* dfq_last_error(void) { return g_err.c_str(); }

int dfq_set_host_threads(int32_t threads) {
    clear_error();
    if (threads < 0 || threads > 256) return fail(DFQ_EINVAL, "dfq_set_host_threads: %d not in [0, 256]", threads);
    g_threads.store(threads, std::memory_order_relaxed);
    return DFQ_OK;
}

int32_t dfq_host_threads(void) { return host_threads(); }

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
    return build_csr({EdgeSpan{src, dst, m}}, n, flags, out);
}

}  // extern "C"

// ------------------------------------------------------------------ text I/O
namespace {

// A whole input file: mapped read-only (text and binary parsers only read
// it, every parser is bounded by p + n, nothing relies on a terminating NUL).
struct Buf {
    char* p = nullptr;
    size_t n = 0;
    bool mapped = false;
    ~Buf() {
        if (mapped) munmap(p, n);
        else free(p);
    }
};

int read_file(const char* path, Buf& b) {
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return fail(DFQ_EIO, "cannot open '%s': %s", path, strerror(errno));
    struct stat st;
    if (fstat(fd, &st) != 0) { close(fd); return fail(DFQ_EIO, "cannot size '%s': %s", path, strerror(errno)); }
    b.n = (size_t)st.st_size;
    if (b.n > 0) {
        void* m = mmap(nullptr, b.n, PROT_READ, MAP_PRIVATE, fd, 0);
        if (m != MAP_FAILED) {
            b.p = (char*)m;
            b.mapped = true;
            madvise(m, b.n, MADV_SEQUENTIAL);
            close(fd);
            return DFQ_OK;
        }
    }
    // not mappable (empty file, special file): read it
    b.p = (char*)malloc(b.n + 1);
    if (!b.p) { close(fd); return fail(DFQ_ENOMEM, "cannot buffer %zu bytes of '%s'", b.n, path); }
    size_t got = 0;
    while (got < b.n) {
        const ssize_t r = read(fd, b.p + got, b.n - got);
        if (r <= 0) break;
        got += (size_t)r;
    }
    close(fd);
    if (got != b.n) return fail(DFQ_EIO, "short read on '%s'", path);
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

// Cut [lo, hi) into at most t pieces whose boundaries sit on bytes for which
// at(p) holds (a whitespace byte for token streams, the byte after '\n' for
// line streams); returns t + 1 boundaries.
template <class At>
std::vector<const char*> split_text(const char* lo, const char* hi, int t, At at) {
    std::vector<const char*> cut{lo};
    const size_t len = (size_t)(hi - lo);
    for (int i = 1; i < t; ++i) {
        const char* q = lo + len * (size_t)i / (size_t)t;
        if (q < cut.back()) q = cut.back();
        while (q < hi && !at(q)) ++q;
        cut.push_back(q);
    }
    cut.push_back(hi);
    return cut;
}

inline int text_threads(size_t bytes) { return pieces_for((int64_t)bytes, 1 << 22); }

// One whitespace-separated token as Cursor::next_int reads it: optional sign,
// decimal digits, |value| <= 2^40.  false if it is not such an integer.
inline bool token_int(const char* p, const char* e, int64_t& v) {
    bool neg = false;
    if (p < e && (*p == '-' || *p == '+')) { neg = (*p == '-'); ++p; }
    if (p >= e) return false;
    int64_t x = 0;
    for (; p < e; ++p) {
        if (*p < '0' || *p > '9') return false;
        x = x * 10 + (*p - '0');
        if (x > ((int64_t)1 << 40)) return false;
    }
    v = neg ? -x : x;
    return true;
}

// .dat body after the header: N "start length" records, then E "dst x"
// records.  Two parallel passes over the text: count tokens per piece, then
// parse every token into its record slot.  Errors are reported for the first
// bad record in file order, as a serial reader would.
int parse_dat(const Buf& b, const char* path, dfq_csr* out) {
    Cursor c{b.p, b.p + b.n};
    int64_t n, e, s;
    if (c.next_int(n) || c.next_int(e) || c.next_int(s))
        return fail(DFQ_EFORMAT, "%s: .dat header must be 'N E SOURCE'", path);
    if (n < 0 || n >= ((int64_t)1 << 31) || e < 0 || e >= ((int64_t)1 << 31))
        return fail(DFQ_EFORMAT, "%s: header N=%lld E=%lld out of range", path, (long long)n, (long long)e);
    std::vector<int32_t> start(n), len(n), edge(e > 0 ? e : 1);
    const int64_t want = 2 * n + 2 * e;  // tokens after the header
    const auto cut = split_text(c.p, c.end, text_threads((size_t)(c.end - c.p)),
                                [](const char* q) { return is_space(*q); });
    const int T = (int)cut.size() - 1;
    std::vector<int64_t> base((size_t)T + 1, 0);
    run_threads(T, [&](int t) {
        int64_t k = 0;
        for (const char* q = cut[t]; q < cut[t + 1];) {
            while (q < cut[t + 1] && is_space(*q)) ++q;
            if (q >= cut[t + 1]) break;
            ++k;
            while (q < cut[t + 1] && !is_space(*q)) ++q;
        }
        base[t + 1] = k;
    });
    for (int t = 0; t < T; ++t) base[t + 1] += base[t];
    // first bad record in file order: node i -> key i, edge j -> key n + j
    std::atomic<int64_t> bad_key{INT64_MAX};
    auto note_bad = [&](int64_t key) {
        int64_t cur = bad_key.load(std::memory_order_relaxed);
        while (key < cur && !bad_key.compare_exchange_weak(cur, key)) {}
    };
    run_threads(T, [&](int t) {
        int64_t k = base[t];
        if (k >= want) return;
        for (const char* q = cut[t]; q < cut[t + 1] && k < want; ++k) {
            while (q < cut[t + 1] && is_space(*q)) ++q;
            if (q >= cut[t + 1]) break;
            const char* tok = q;
            while (q < cut[t + 1] && !is_space(*q)) ++q;
            int64_t v;
            const bool ok = token_int(tok, q, v);
            if (k < 2 * n) {
                const int64_t i = k >> 1;
                if (!ok || v < 0 || v > e) { note_bad(i); continue; }
                if (k & 1) len[i] = (int32_t)v;
                else start[i] = (int32_t)v;
            } else {
                const int64_t j = (k - 2 * n) >> 1;
                if (!ok) { note_bad(n + j); continue; }
                if (!((k - 2 * n) & 1)) {
                    if (v < 0 || v >= n) { note_bad(n + j); continue; }
                    edge[j] = (int32_t)v;
                }
            }
        }
    });
    if (base[T] < want) note_bad(base[T] < 2 * n ? base[T] >> 1 : n + ((base[T] - 2 * n) >> 1));
    // the start + length bound needs both fields of a record
    parallel_for(n, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i)
            if ((int64_t)start[i] + len[i] > e) { note_bad(i); return; }
    });
    const int64_t key = bad_key.load();
    if (key != INT64_MAX) {
        if (key < n) {
            const int64_t t0 = 2 * key;
            int64_t st = -1, ln = -1;
            // re-read this record serially for the message
            Cursor r{c.p, c.end};
            for (int64_t k = 0; k < t0; ++k) { int64_t x; if (r.next_int(x)) break; }
            const bool have = r.next_int(st) == 0 && r.next_int(ln) == 0;
            if (!have)
                return fail(DFQ_EFORMAT, "%s: node record %lld missing or malformed", path, (long long)key);
            return fail(DFQ_EFORMAT, "%s: node %lld has start=%lld length=%lld outside E=%lld", path,
                        (long long)key, (long long)st, (long long)ln, (long long)e);
        }
        const int64_t j = key - n;
        Cursor r{c.p, c.end};
        bool have = true;
        for (int64_t k = 0; k < 2 * n + 2 * j; ++k) { int64_t x; if (r.next_int(x)) { have = false; break; } }
        int64_t d = 0, ignored = 0;
        if (!have || r.next_int(d) || r.next_int(ignored))
            return fail(DFQ_EFORMAT, "%s: edge record %lld missing or malformed", path, (long long)j);
        return fail(DFQ_EFORMAT, "%s: edge %lld targets %lld outside [0,%lld)", path, (long long)j,
                    (long long)d, (long long)n);
    }
    if (s < 0 || s >= n) s = 0;  // the reference re-prompts instead (DFQ:204-214)
    int64_t total = 0;
    bool plain = true;  // rows already laid out back to back from 0?
    for (int64_t i = 0; i < n; ++i) {
        if (start[i] != total) plain = false;
        total += len[i];
    }
    if (total != e) plain = false;
    int rc = alloc_csr((int32_t)n, total, out);
    if (rc) return rc;
    out->source = (int32_t)s;
    out->offsets[0] = 0;
    for (int64_t i = 0; i < n; ++i) out->offsets[i + 1] = out->offsets[i] + len[i];
    if (plain) {
        memcpy(out->cols, edge.data(), sizeof(int32_t) * total);
    } else {  // arbitrary (start, length) records: gather rows in vertex order
        parallel_for(n, [&](int64_t lo, int64_t hi) {
            for (int64_t i = lo; i < hi; ++i)
                memcpy(out->cols + out->offsets[i], edge.data() + start[i], sizeof(int32_t) * len[i]);
        }, 1 << 12);
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
    // bounded decimal read (the buffer is not NUL-terminated)
    auto num = [&](const char* r) -> int64_t {
        while (r < end && (*r == ' ' || *r == '\t')) ++r;
        int64_t x = 0;
        bool any = false;
        while (r < end && *r >= '0' && *r <= '9' && x < ((int64_t)1 << 40)) { x = x * 10 + (*r++ - '0'); any = true; }
        return any ? x : 0;
    };
    n = num(a);
    e = b ? num(b) : -1;
    return true;
}

// SNAP edge list, parsed in parallel over line-aligned pieces of the text.
// Each piece keeps its own edges, largest id, first "# Nodes:" header and first
// error; pieces are then joined in file order, so the edge order, the header
// taken and the error reported are those of a serial reader.
int parse_snap(const Buf& b, const char* path, int32_t flags, dfq_csr* out) {
    const char* end = b.p + b.n;
    const auto cut = split_text(b.p, end, text_threads(b.n), [&](const char* q) { return q > b.p && q[-1] == '\n'; });
    const int T = (int)cut.size() - 1;
    struct Piece {
        std::vector<int32_t> src, dst;
        int64_t maxid = -1, lines = 0, hdr_n = -1, hdr_e = -1;
        int err = 0;  // 1: not 'FromNodeId ToNodeId', 2: id out of int32 range
    };
    std::vector<Piece> pc((size_t)T);
    run_threads(T, [&](int t) {
        Piece& P = pc[t];
        P.src.reserve((size_t)(cut[t + 1] - cut[t]) / 10);
        P.dst.reserve((size_t)(cut[t + 1] - cut[t]) / 10);
        Cursor c{cut[t], cut[t + 1]};
        while (true) {
            c.skip_space();
            if (c.p >= c.end) break;
            if (*c.p == '#') {
                int64_t nn, ee;
                if (P.hdr_n < 0 && parse_nodes_header(c.p, c.end, nn, ee)) { P.hdr_n = nn; P.hdr_e = ee; }
                c.skip_line();
                continue;
            }
            int64_t u, v;
            ++P.lines;
            if (c.next_int(u) || c.next_int(v)) { P.err = 1; return; }
            if (u < 0 || v < 0 || u >= ((int64_t)1 << 31) - 1 || v >= ((int64_t)1 << 31) - 1) { P.err = 2; return; }
            // anything after the two ids on the line (weights, timestamps) is ignored
            while (c.p < c.end && *c.p != '\n') ++c.p;
            P.src.push_back((int32_t)u);
            P.dst.push_back((int32_t)v);
            if (u > P.maxid) P.maxid = u;
            if (v > P.maxid) P.maxid = v;
        }
    });
    int64_t hdr_n = -1, lines = 0, maxid = -1, m = 0;
    for (int t = 0; t < T; ++t) {
        const Piece& P = pc[t];
        if (P.err) {
            const int64_t line = lines + P.lines;
            if (P.err == 1)
                return fail(DFQ_EFORMAT, "%s: edge line %lld is not 'FromNodeId ToNodeId'", path, (long long)line);
            return fail(DFQ_EFORMAT, "%s: edge line %lld has id out of int32 range", path, (long long)line);
        }
        if (hdr_n < 0 && P.hdr_n >= 0) hdr_n = P.hdr_n;
        lines += P.lines;
        maxid = std::max(maxid, P.maxid);
        m += (int64_t)P.src.size();
    }
    int64_t n = hdr_n > 0 ? hdr_n : 0;
    if (maxid + 1 > n) n = maxid + 1;  // SNAP ids may exceed the header's count
    if (n >= ((int64_t)1 << 31)) return fail(DFQ_EFORMAT, "%s: too many vertices", path);
    std::vector<EdgeSpan> spans;
    for (const Piece& P : pc)
        if (!P.src.empty()) spans.push_back(EdgeSpan{P.src.data(), P.dst.data(), (int64_t)P.src.size()});
    return build_csr(spans, (int32_t)n, flags, out);
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
        const int32_t* off = out->offsets;
        const int32_t* col = out->cols;
        parallel_for(out->n, [&](int64_t lo, int64_t hi) {
            for (int64_t u = lo; u < hi; ++u)
                for (int32_t k = off[u]; k < off[u + 1]; ++k) { s[k] = (int32_t)u; d[k] = col[k]; }
        }, 1 << 14);
        int32_t src = out->source, n = out->n;
        dfq_csr_free(out);
        rc = build_csr({EdgeSpan{s.data(), d.data(), (int64_t)s.size()}}, n, flags, out);
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
    if (format != DFQ_FMT_SNAP && format != DFQ_FMT_DAT)
        return fail(DFQ_EINVAL, "dfq_csr_save: unknown format %d", format);
    // Text is formatted in parallel, one buffer per piece, and written in order.
    const int T = pieces_for(g->e + g->n, 1 << 18);
    std::vector<Out> part;
    Out head;
    if (format == DFQ_FMT_SNAP) {
        head.put("# Nodes: "); head.put_int(g->n); head.put(" Edges: "); head.put_int(g->e); head.ch('\n');
        head.put("# FromNodeId\tToNodeId\n");
        // pieces: vertex ranges holding about e / T edges each
        std::vector<int32_t> vcut{0};
        for (int t = 1; t < T; ++t) {
            const int32_t want = (int32_t)(g->e * t / T);
            const int32_t v = (int32_t)(std::lower_bound(g->offsets, g->offsets + g->n + 1, want) - g->offsets);
            vcut.push_back(std::max(vcut.back(), std::min(v, g->n)));
        }
        vcut.push_back(g->n);
        part.resize((size_t)T);
        run_threads(T, [&](int t) {
            Out& o = part[t];
            o.v.reserve((size_t)(g->offsets[vcut[t + 1]] - g->offsets[vcut[t]]) * 16 + 64);
            for (int32_t u = vcut[t]; u < vcut[t + 1]; ++u)
                for (int32_t k = g->offsets[u]; k < g->offsets[u + 1]; ++k) {
                    o.put_int(u); o.ch('\t'); o.put_int(g->cols[k]); o.ch('\n');
                }
        });
    } else {
        // the second column of the edge records is ignored by the reference
        // loader (DFQ:199); it is written as 1
        head.put_int(g->n); head.ch(' '); head.put_int(g->e); head.ch(' '); head.put_int(g->source); head.ch('\n');
        part.resize((size_t)(2 * T));
        run_threads(T, [&](int t) {
            Out& o = part[t];
            const int32_t lo = (int32_t)((int64_t)g->n * t / T), hi = (int32_t)((int64_t)g->n * (t + 1) / T);
            o.v.reserve((size_t)(hi - lo) * 20 + 64);
            for (int32_t u = lo; u < hi; ++u) {
                o.put_int(g->offsets[u]); o.ch(' '); o.put_int(g->offsets[u + 1] - g->offsets[u]); o.ch('\n');
            }
            Out& q = part[T + t];
            const int64_t klo = g->e * t / T, khi = g->e * (t + 1) / T;
            q.v.reserve((size_t)(khi - klo) * 12 + 64);
            for (int64_t k = klo; k < khi; ++k) { q.put_int(g->cols[k]); q.put(" 1\n"); }
        });
    }
    FILE* f = fopen(path, "wb");
    if (!f) return fail(DFQ_EIO, "cannot create '%s': %s", path, strerror(errno));
    bool ok = fwrite(head.v.data(), 1, head.v.size(), f) == head.v.size();
    for (const Out& o : part)
        if (ok && !o.v.empty()) ok = fwrite(o.v.data(), 1, o.v.size(), f) == o.v.size();
    const int cl = fclose(f);
    if (!ok || cl != 0) return fail(DFQ_EIO, "short write on '%s'", path);
    return DFQ_OK;
}

}  // extern "C"
