// Shared host-side helpers for libdfq: thread-local error text, a small
// parallel_for, and the seeded random streams every generator uses.
#pragma once
#include "dfq.h"

#include <cstdint>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

namespace dfqk {
struct Control;
}

namespace dfq {

// Record a message for dfq_last_error() on this host thread and return `code`.
int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();

// Number of host threads the library uses for parallel host work.
int host_threads();

// Run body(lo, hi) over [0, n) split into at most host_threads() contiguous
// ranges.  Work assignment never changes results: every caller either writes
// disjoint outputs per index or combines per-range partials in range order.
template <class F>
void parallel_for(int64_t n, F&& body, int64_t min_per_thread = 1 << 16) {
    int t = host_threads();
    if (n <= 0) return;
    int64_t want = (n + min_per_thread - 1) / min_per_thread;
    if (want < t) t = (int)want;
    if (t <= 1) { body((int64_t)0, n); return; }
    std::vector<std::thread> th;
    th.reserve(t);
    for (int i = 0; i < t; ++i) {
        int64_t lo = n * i / t, hi = n * (i + 1) / t;
        th.emplace_back([&body, lo, hi] { body(lo, hi); });
    }
    for (auto& x : th) x.join();
}

// One run of an edge list: src[i] -> dst[i] for i in [0, m).
struct EdgeSpan {
    const int32_t* src;
    const int32_t* dst;
    int64_t m;
};

// CSR from the concatenation of `spans` (ids already in [0, n) are checked);
// flags as for dfq_csr_from_edges.  Same result for any host thread count.
int build_csr(const std::vector<EdgeSpan>& spans, int32_t n, int32_t flags, dfq_csr* out);

// Hub-first renumbering of a host CSR: new id i is input id order[i], sorted
// by descending in-degree (ties by id), rank[v] the new id of v; each row of
// out lists its neighbours in new ids with the row's hub (smallest new id)
// first.  mode as dfq_opts.vertex_order (0 auto: at least 2^16 vertices and
// a largest in-degree >= 64 x the average; 1 never; 2 always).  Returns 1 if
// renumbered (out allocated), 0 if not, or a negative status.
int hub_first_csr(const dfq_csr& in, int mode, dfq_csr* out, std::vector<int32_t>* rank,
                  std::vector<int32_t>* order);

// Make sure kernel fn's dynamic shared-memory limit on the current device is
// at least what the next launch needs.  The limit is a property of the
// function, shared by every graph, pool and entry point launching it, so it
// only ever rises (under a lock): no caller can lower it under another's launch.
int allow_dyn_smem(const void* fn, int smem_needed);

// DFQ_OK for a launch whose control block reports no device error, else the
// matching status (DFQ_ETIMEOUT, DFQ_EDEVICE) with its message recorded.
int device_status(const dfqk::Control& c);

// DFQ_OK if every field of o is in range and its shared-memory layout fits a
// block, else DFQ_EINVAL with the reason recorded.
int check_opts(const dfq_opts& o);

// The single-source kernel dfqk::dfq_bfs_kernel<block_threads, par>, compiled
// once (in dfq_api.cu) and launched through this handle by every entry point
// that runs one BFS on a whole cooperative grid; null for an unsupported size.
const void* single_source_kernel(int block_threads, bool par);

// The cluster form dfqk::dfq_cluster_kernel<block_threads, par> (compiled in
// dfq_cluster.cu): one thread-block cluster runs the BFS; null for a block
// size it is not built for (512 and 1024 only).
const void* cluster_kernel(int block_threads, bool par);

// Run body(i) for i in [0, t) on t threads (the caller's thread takes i = 0).
template <class F>
void run_threads(int t, F&& body) {
    if (t <= 1) { body(0); return; }
    std::vector<std::thread> th;
    th.reserve(t - 1);
    for (int i = 1; i < t; ++i) th.emplace_back([&body, i] { body(i); });
    body(0);
    for (auto& x : th) x.join();
}

// SplitMix64 (Steele, Lea, Flood 2014): used to derive stream seeds.
inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
inline uint64_t mix_seed(uint64_t seed, uint64_t stream) {
    uint64_t s = seed ^ (stream * 0xd1b54a32d192ed03ULL);
    splitmix64(s);
    return splitmix64(s);
}

// xoshiro256** (Blackman, Vigna 2018): the per-stream generator.
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (auto& w : s) w = splitmix64(x);
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    inline uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    // Uniform integer in [0, bound) without modulo bias (Lemire 2019).
    inline uint64_t below(uint64_t bound) {
        unsigned __int128 m = (unsigned __int128)next() * bound;
        uint64_t lo = (uint64_t)m;
        if (lo < bound) {
            uint64_t thresh = (0 - bound) % bound;
            while (lo < thresh) {
                m = (unsigned __int128)next() * bound;
                lo = (uint64_t)m;
            }
        }
        return (uint64_t)(m >> 64);
    }
    // Uniform double in [0,1) from the top 53 bits.
    inline double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
};

}  // namespace dfq
