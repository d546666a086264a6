/*
 * gen.c - seeded workload generators restated for the checker side.
 * TEST INFRASTRUCTURE ONLY: tests/ and bench.py's reference arm call it, so
 * that the reference-side measurement builds its graph and sources without
 * loading the product library.  No product code path links or calls it.
 *
 * What it restates (the product's generators, dfq-bfs_gb300/csrc/host_gen.cpp
 * and the CSR builder of dfq-bfs_gb300/csrc/host_graph.cpp), from the
 * published algorithms they use:
 *   splitmix64      Steele, Lea, Flood, "Fast splittable pseudorandom number
 *                   generators", OOPSLA 2014 (stream-seed derivation)
 *   xoshiro256**    Blackman, Vigna, "Scrambled linear pseudorandom number
 *                   generators", 2018 (the per-stream generator)
 *   below()         Lemire, "Fast random integer generation in an interval",
 *                   2019 (multiply-shift with rejection)
 *   R-MAT           Chakrabarti, Zhan, Faloutsos, SDM 2004: per edge, `scale`
 *                   quadrant choices with probabilities a, b, c, d; here
 *                   two 32-bit halves of one 64-bit draw per two levels, then
 *                   a seeded Fisher-Yates relabelling of the vertices
 *   CSR             symmetrised (u->v adds v->u), self-loops dropped, each row
 *                   sorted and de-duplicated: a function of the edge SET, so
 *                   any correct builder gives the same arrays
 *   pick_sources    partial Fisher-Yates over the vertices of out-degree > 0
 *
 * The reference measures on SNAP datasets that are not in its repository;
 * these seeded graphs stand in for them.  tests/test_oracle_gen.py checks
 * every array here against the product's generator byte for byte.
 */
#include <pthread.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { uint64_t s[4]; } gen_rng;

static uint64_t splitmix64(uint64_t* s) {
    uint64_t z = (*s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

/* Seed of stream `stream` of a generator seeded with `seed`. */
static uint64_t mix_seed(uint64_t seed, uint64_t stream) {
    uint64_t s = seed ^ (stream * 0xd1b54a32d192ed03ULL);
    splitmix64(&s);
    return splitmix64(&s);
}

static void rng_init(gen_rng* r, uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) r->s[i] = splitmix64(&x);
}

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t rng_next(gen_rng* r) {
    uint64_t* s = r->s;
    const uint64_t out = rotl64(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return out;
}

/* Uniform integer in [0, bound), bound > 0. */
static uint64_t rng_below(gen_rng* r, uint64_t bound) {
    unsigned __int128 m = (unsigned __int128)rng_next(r) * bound;
    uint64_t lo = (uint64_t)m;
    if (lo < bound) {
        const uint64_t thresh = (0 - bound) % bound;
        while (lo < thresh) {
            m = (unsigned __int128)rng_next(r) * bound;
            lo = (uint64_t)m;
        }
    }
    return (uint64_t)(m >> 64);
}

/* ------------------------------------------------------------ threads */
typedef void (*range_fn)(void* ctx, int64_t lo, int64_t hi);
typedef struct { range_fn f; void* ctx; int64_t lo, hi; } range_job;

static void* range_main(void* a) {
    range_job* j = (range_job*)a;
    j->f(j->ctx, j->lo, j->hi);
    return NULL;
}

/* f(ctx, lo, hi) over [0, n) cut into `threads` contiguous ranges.  Every
 * caller writes disjoint outputs per index, so the split never changes results. */
static void par_range(int threads, int64_t n, range_fn f, void* ctx) {
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    if (n < (int64_t)threads * 1024) threads = 1;
    if (threads == 1) { f(ctx, 0, n); return; }
    pthread_t th[64];
    range_job jobs[64];
    int joined[64] = {0};
    for (int i = 0; i < threads; ++i) {
        jobs[i].f = f;
        jobs[i].ctx = ctx;
        jobs[i].lo = n * i / threads;
        jobs[i].hi = n * (i + 1) / threads;
    }
    for (int i = 1; i < threads; ++i) {
        if (pthread_create(&th[i], NULL, range_main, &jobs[i]) == 0) joined[i] = 1;
        else f(ctx, jobs[i].lo, jobs[i].hi);  /* no thread: run the range here */
    }
    f(ctx, jobs[0].lo, jobs[0].hi);
    for (int i = 1; i < threads; ++i)
        if (joined[i]) pthread_join(th[i], NULL);
}

/* ------------------------------------------------------------ R-MAT edges */
typedef struct {
    int32_t scale;
    int64_t m;
    uint64_t seed, A, AB, ABC;
    const int32_t* perm;
    int32_t* src;
    int32_t* dst;
} rmat_ctx;

enum { kRmatChunk = 1 << 16 };

static void rmat_chunks(void* c_, int64_t lo, int64_t hi) {
    rmat_ctx* c = (rmat_ctx*)c_;
    for (int64_t ch = lo; ch < hi; ++ch) {
        gen_rng r;
        rng_init(&r, mix_seed(c->seed, 1000000 + (uint64_t)ch));
        const int64_t i0 = ch * kRmatChunk;
        const int64_t i1 = (ch + 1) * kRmatChunk < c->m ? (ch + 1) * kRmatChunk : c->m;
        for (int64_t i = i0; i < i1; ++i) {
            uint32_t u = 0, v = 0;
            uint64_t word = 0;
            for (int l = 0; l < c->scale; ++l) {
                uint64_t x;
                if (l & 1) x = word >> 32;
                else { word = rng_next(&r); x = word & 0xffffffffULL; }
                const uint32_t bu = x >= c->AB;
                const uint32_t bv = (x >= c->A && x < c->AB) || x >= c->ABC;
                u = (u << 1) | bu;
                v = (v << 1) | bv;
            }
            c->src[i] = c->perm[u];
            c->dst[i] = c->perm[v];
        }
    }
}

/* ------------------------------------------------------------ CSR build */
typedef struct {
    int32_t* off;
    int32_t* col;
    int32_t* newdeg;
} rows_ctx;

static int cmp_i32(const void* a, const void* b) {
    const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return (x > y) - (x < y);
}

static void sort_unique_rows(void* c_, int64_t lo, int64_t hi) {
    rows_ctx* c = (rows_ctx*)c_;
    for (int64_t u = lo; u < hi; ++u) {
        int32_t* b = c->col + c->off[u];
        const int32_t d = c->off[u + 1] - c->off[u];
        if (d <= 32) {  /* insertion sort for short rows */
            for (int32_t i = 1; i < d; ++i) {
                const int32_t x = b[i];
                int32_t j = i - 1;
                while (j >= 0 && b[j] > x) { b[j + 1] = b[j]; --j; }
                b[j + 1] = x;
            }
        } else {
            qsort(b, (size_t)d, sizeof(int32_t), cmp_i32);
        }
        int32_t w = 0;
        for (int32_t i = 0; i < d; ++i)
            if (w == 0 || b[i] != b[w - 1]) b[w++] = b[i];
        c->newdeg[u] = w;
    }
}

/* Undirected simple graph from an edge list: symmetrised, self-loops dropped,
 * rows sorted and de-duplicated.  *off_out (n+1) and *col_out (e) are
 * malloc'd; returns e, or -1 on allocation failure / bad ids. */
static int64_t csr_undirected(const int32_t* src, const int32_t* dst, int64_t m, int32_t n, int threads,
                              int32_t** off_out, int32_t** col_out) {
    *off_out = NULL;
    *col_out = NULL;
    int64_t* cnt = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    if (!cnt) return -1;
    for (int64_t i = 0; i < m; ++i) {
        const int32_t u = src[i], v = dst[i];
        if ((uint32_t)u >= (uint32_t)n || (uint32_t)v >= (uint32_t)n) { free(cnt); return -1; }
        if (u == v) continue;
        cnt[u]++;
        cnt[v]++;
    }
    int64_t total = 0;
    for (int32_t u = 0; u < n; ++u) { const int64_t d = cnt[u]; cnt[u] = total; total += d; }
    cnt[n] = total;
    if (total >= ((int64_t)1 << 31)) { free(cnt); return -1; }
    int32_t* off = (int32_t*)malloc(sizeof(int32_t) * ((size_t)n + 1));
    int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(total > 0 ? total : 1));
    int32_t* newdeg = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    if (!off || !col || !newdeg) { free(cnt); free(off); free(col); free(newdeg); return -1; }
    for (int32_t u = 0; u <= n; ++u) off[u] = (int32_t)cnt[u];
    for (int64_t i = 0; i < m; ++i) {
        const int32_t u = src[i], v = dst[i];
        if (u == v) continue;
        col[cnt[u]++] = v;
        col[cnt[v]++] = u;
    }
    free(cnt);
    rows_ctx rc = {off, col, newdeg};
    par_range(threads, n, sort_unique_rows, &rc);
    int64_t w = 0;
    for (int32_t u = 0; u < n; ++u) {
        const int32_t b = off[u], d = newdeg[u];
        off[u] = (int32_t)w;
        if (w != b) memmove(col + w, col + b, sizeof(int32_t) * (size_t)d);
        w += d;
    }
    off[n] = (int32_t)w;
    free(newdeg);
    *off_out = off;
    *col_out = col;
    return w;
}

/* ------------------------------------------------------------ public */

/* R-MAT graph of 2^scale vertices and edge_factor * 2^scale generated edges,
 * quadrant probabilities a, b, c (d = 1 - a - b - c), symmetrised, without
 * self-loops, rows sorted and de-duplicated.  Returns e (the directed edge
 * count of the CSR) and sets *off_out (n+1) / *col_out (e), freed with
 * gen_free; -1 on bad arguments or allocation failure. */
int64_t gen_rmat_undirected(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                            int threads, int32_t** off_out, int32_t** col_out) {
    if (!off_out || !col_out || scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 || c < 0 ||
        a + b + c > 1)
        return -1;
    const int32_t n = (int32_t)1 << scale;
    const int64_t m = (int64_t)edge_factor << scale;
    int32_t* perm = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* src = (int32_t*)malloc(sizeof(int32_t) * (size_t)m);
    int32_t* dst = (int32_t*)malloc(sizeof(int32_t) * (size_t)m);
    if (!perm || !src || !dst) { free(perm); free(src); free(dst); return -1; }
    /* vertex relabelling: Fisher-Yates on stream 2 */
    for (int32_t i = 0; i < n; ++i) perm[i] = i;
    gen_rng r;
    rng_init(&r, mix_seed(seed, 2));
    for (int32_t i = n - 1; i > 0; --i) {
        const int32_t j = (int32_t)rng_below(&r, (uint64_t)i + 1);
        const int32_t t = perm[i];
        perm[i] = perm[j];
        perm[j] = t;
    }
    rmat_ctx rc;
    rc.scale = scale;
    rc.m = m;
    rc.seed = seed;
    rc.A = (uint64_t)ldexp(a, 32);
    rc.AB = (uint64_t)ldexp(a + b, 32);
    rc.ABC = (uint64_t)ldexp(a + b + c, 32);
    rc.perm = perm;
    rc.src = src;
    rc.dst = dst;
    par_range(threads, (m + kRmatChunk - 1) / kRmatChunk, rmat_chunks, &rc);
    free(perm);
    const int64_t e = csr_undirected(src, dst, m, n, threads, off_out, col_out);
    free(src);
    free(dst);
    return e;
}

/* k sources among the vertices of out-degree > 0: distinct (partial
 * Fisher-Yates) when k does not exceed their number, else drawn with
 * replacement; stream 3 of `seed`.  Returns 0, or -1 if no vertex qualifies. */
int gen_pick_sources(int32_t n, const int32_t* off, int32_t k, uint64_t seed, int32_t* out) {
    if (n < 1 || !off || k < 0 || (k > 0 && !out)) return -1;
    int32_t* cand = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    if (!cand) return -1;
    int64_t nc = 0;
    for (int32_t u = 0; u < n; ++u)
        if (off[u + 1] > off[u]) cand[nc++] = u;
    if (nc == 0) { free(cand); return -1; }
    gen_rng r;
    rng_init(&r, mix_seed(seed, 3));
    if ((int64_t)k <= nc) {
        for (int32_t i = 0; i < k; ++i) {
            const int64_t j = i + (int64_t)rng_below(&r, (uint64_t)(nc - i));
            const int32_t t = cand[i];
            cand[i] = cand[j];
            cand[j] = t;
            out[i] = cand[i];
        }
    } else {
        for (int32_t i = 0; i < k; ++i) out[i] = cand[rng_below(&r, (uint64_t)nc)];
    }
    free(cand);
    return 0;
}

void gen_free(void* p) { free(p); }
