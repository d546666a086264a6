// Persistent decentralized-frontier-queue BFS kernel for sm_103a.
//
// Replaces CUDA_BFS_KERNEL_CG_NEW and its VISIT_* helpers of the reference
// (design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu:44-179).  Same contract:
// one cooperative launch runs a whole level-synchronous BFS from one source and
// leaves levels[v] = BFS depth of v (-1 unreached).  Different mechanism:
//
//  * No status-array scan.  The reference rebuilds each frontier by scanning all
//    N levels (bfs.cu:116-124); here a vertex is pushed to the next frontier by
//    the thread that claims it (the scan-free model of
//    design/shared-q/scan-free/non-sep/lower-bound/bfs.cu:28-42).
//  * Claims are atomicOr on a visited bitmap (N/8 bytes, L2-resident), so each
//    vertex enters exactly one frontier; levels/parents are plain stores by the
//    unique claimer.
//  * Decentralized queues: each block keeps frontier entries it discovered in
//    its own shared-memory queue and expands them itself at the next level.
//    A warp reserves slots once for all its lanes, all-or-nothing against the
//    queue's entry capacity and edge budget (one 64-bit CAS on count|degrees);
//    a batch that does not fit goes to the global overflow queue, which all
//    warps of the grid drain with dynamic chunks.
//  * Degree bins (the reference's "our-sep" bins, bfs.cu:16-36,119-123):
//      small  [1, medium_min)      -> warp-level load-balanced gather (prefix sum
//                                     of 32 degrees + binary search: no idle lanes)
//      medium [medium_min, large)  -> one warp per vertex, int4 column loads
//      large  [large_min, inf)     -> global large queue cut into fixed pieces;
//                                     every warp pulls pieces and stages each one
//                                     into its shared-memory buffer with
//                                     cp.async.bulk (TMA), double-buffered
//  * Warps work independently inside a level (no block barrier until the level
//    ends), so a slow warp only delays itself.  One grid barrier per level
//    (bounded spin, error word on timeout) instead of three grid.sync() calls
//    (bfs.cu:114,170,177); termination is decided from a counter every block
//    reads after the barrier, so all blocks leave together (the reference's
//    racy `*done` flag, bfs.cu:115, is gone).
//
// Every queue is sized so it cannot overflow (a vertex is claimed once per
// BFS), and every index is still checked before the store; a violated bound
// sets the error word and skips the store.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// Profiling build only (DFQ_CLAIM_PROBES=1 at build time): with profile on,
// the claim path records when its steps finish.  0 in the product build, so
// the probes are not even compiled there.
#ifndef DFQ_CLAIM_PROBES
#define DFQ_CLAIM_PROBES 0
#endif

namespace dfqk {

constexpr unsigned kFull = 0xffffffffu;

// device error codes (host maps them onto DFQ_E*)
enum : int { kErrNone = 0, kErrBarrierTimeout = 1, kErrTmaTimeout = 2, kErrQueueCap = 3 };

// Counters of one level's output frontier.  Rotated over three slots: level L
// reads lv[L%3], appends to lv[(L+1)%3] and clears lv[(L+2)%3].  Producer
// counters and the two consumer cursors sit on separate 128-byte lines so
// atomics on one do not queue behind atomics on another.
struct alignas(128) LevelCtr {
    unsigned long long ovf_pieces;  // (global overflow queue entries << 32) | large-list pieces
    int pushed;                     // frontier entries (local + overflow + large)
    int pushed_edges;               // sum of the degrees of those entries
    int pad0[28];
    int ovf_grab;                   // chunk cursor over the overflow queue
    int pad1[31];
    int large_grab;                 // piece cursor over the large queue
    int pad2[31];
    // tally barrier: the level's arrivals and tallies in two words, see
    // tally_barrier (bits 54-63 arrivals, 27-53 and 0-26 two tallies)
    unsigned long long tally[2];
    int pad3[28];
};

struct DevStats {
    unsigned long long edges;     // adjacency entries scanned (= E_R)
    unsigned long long claims;    // vertices claimed (source excluded)
    unsigned long long overflow;  // entries that went to the global overflow queue
    unsigned long long large;     // entries that went to the large queue
    int levels;                   // level iterations run
    int depth;                    // deepest level written
    int pad[2];
};

constexpr int kTraceLevels = 64;  // levels with a recorded start time / frontier size

// Per-launch control block; zeroed by the host before every launch.
struct Control {
    LevelCtr lv[3];
    alignas(128) unsigned barrier;  // grid barrier arrivals (monotone within a launch)
    int pad_b[31];
    int status;        // first error (kErr*)
    int err_info[2];
    DevStats stats;
    long long trace_ns[kTraceLevels];   // %globaltimer when level L starts (block 0)
    int trace_frontier[kTraceLevels];   // frontier entries of level L
    // per-level profile (first kTraceLevels levels)
    int trace_edges[kTraceLevels];      // degree sum of level L's frontier (edges it scans)
    int trace_ovf[kTraceLevels];        // of its entries, those in the global overflow queue
    int trace_pieces[kTraceLevels];     // large-list pieces
    int trace_probe[kTraceLevels];      // 1 if level L probed the bitmap before claiming
    unsigned long long trace_done_last[kTraceLevels];   // latest block finish
    unsigned long long trace_done_first[kTraceLevels];  // ~(earliest block finish), 0 = none
    // with profiling: the latest time (ns after its block's level start) a
    // warp finished the own queue, the pieces, the overflow chunks, the claims
    unsigned trace_phase[kTraceLevels][4];
    // profiling build: over all warps, the latest time (ns after the warp's
    // level start) a claim batch had its neighbours in hand, its row bounds
    // loaded, its claim atomics answered, its pushes done
    unsigned trace_claim[kTraceLevels][4];
    // profiling build: sums over all warps of the staged-piece path - pieces
    // expanded, ns waiting for their bulk copies, ns expanding them (claims
    // included) - and ns spent in candidate claim drains on any path
    unsigned long long trace_piece[kTraceLevels][4];
};

struct Params {
    const int* __restrict__ offsets;  // n+1
    const int* __restrict__ cols;     // e; reads stay inside 16-byte chunks holding a valid entry
    int n;
    int src;
    int* levels;
    int* parents;  // null unless parents requested
    unsigned* bitmap;
    int bitmap_words;
    int2* ovf[2];   // (start, degree) overflow entries, ovf_cap each
    int* ovfv[2];   // their vertex ids (parents only)
    int ovf_cap;    // n (a vertex is queued once per BFS) unless a bounded workspace says less
    int2* piece[2];   // large-list pieces: edge range [lo, hi) of the list, piece_cap each
    int* piece_v[2];  // the vertex each piece belongs to (parents only)
    int piece_cap;
    Control* ctl;
    int medium_min;
    int large_min;
    int piece_edges;  // per-warp piece, multiple of 64
    int local_cap;    // local queue entries
    int local_budget; // local queue edges
    int probe_first;
    int use_tma;
    long long timeout_ns;
    // visited bits of vertices [0, 32 * hot_words) cached in shared memory on
    // probe levels (0: no cache); a multiple of 32 words, at most kHotWordsMax
    int hot_words;
    int profile;  // 1: record each block's level finish times
    int trace_from;  // first level of the traced window of kTraceLevels levels
    int direction;  // 1: levels may run bottom-up (undirected graph, checked by the host)
    int e;          // edges (the bottom-up switch compares against the unexplored ones)
    // vertex order: when the graph was relabelled (rank != null) the kernel
    // runs on new ids, with levels / parents above indexed by new id, and at
    // the end writes levels_out[v] = levels[rank[v]] and parents_out[v] =
    // order[parents[rank[v]]] for the caller's ids v.  Without rank, a
    // non-null levels_out / parents_out (mapped host memory) gets a plain copy.
    const int* rank;
    const int* order;
    int* levels_out;
    int* parents_out;
    // hub claim words: vertices below hub_n are claimed through their own
    // word, kHubStride apart, instead of a bit of the shared bitmap (null: off)
    unsigned* hub_claim;
    int hub_n;
    int map_src;  // 1: src is an input id, renumbered here through rank
    // failure-path test hook: k > 0 = at the end of level k-1 the group's last
    // block skips its barrier arrival, so every block's bounded wait runs out
    int stall_level;
    // k > 0: multi-block groups end levels on tally_barrier with frontier
    // edges counted in units of 2^(k-1); 0: on group_barrier
    int tally_bar;
};

// Params::tally_bar for a graph of n vertices and e edges: the tally
// barrier's 27-bit fields hold its level totals exactly below 2^27 of each
// (every group has fewer than 1024 blocks, the arrival field's limit).
__host__ __device__ inline int tally_bar_for(long long n, long long e) {
    return (n < (1LL << 27) && e < (1LL << 27)) ? 1 : 0;
}

// Hub claim words sit a 32-byte sector apart: with hub-first ids ~1000 hubs
// share one 128-byte bitmap line, and claim atomics on one line serialise in
// L2 (a level around hubs makes hundreds of thousands of them).
constexpr int kHubStride = 8;
constexpr int kHubIds = 131072;  // most hub claim words per renumbered graph

// Hub claim words of a renumbered graph of n vertices: an eighth of them,
// at least 32,768 and at most kHubIds (every launch clears the words, so a
// small graph keeps few).  RMAT-20/21/22 with 131,072 instead of 32,768:
// -4.8 / -2.4 / -0.5 % time per BFS.
__host__ __device__ inline int hub_count(long long n) {
    long long h = n >> 3;
    if (h < 32768) h = 32768;
    if (h > kHubIds) h = kHubIds;
    return (int)(n < h ? n : h);
}

// Pieces one level can produce with pieces of at least min_piece (>= 64)
// edges and large lists of at least min_large edges: a list of degree d cut
// from its aligned floor (at most 3 entries before it) makes fewer than
// (d + 3) / piece + 1 pieces, a frontier's degrees sum to at most e, and at
// most min(n, e / min_large) lists are large.
__host__ __device__ inline int piece_capacity(long long n, long long e, int min_large, int min_piece) {
    long long large = e / min_large + 1;
    if (large > n) large = n;
    large += 1;
    const long long cap = e / min_piece + large + large / 16 + 2;
    return (int)(cap < (1LL << 30) ? cap : (1LL << 30));
}

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_add_release(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_s32(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_add_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_add_relaxed_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
__device__ __forceinline__ int4 ldg4(const int* p) { return __ldg(reinterpret_cast<const int4*>(p)); }
// L2 policy for the column stream: each column is read once per BFS, so its
// lines are the first to go and the randomly read row bounds, level array and
// visited bitmap keep their L2 residency; L1 is left to the bitmap.
__device__ __forceinline__ unsigned long long policy_stream() {
    unsigned long long pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ int4 ldg4_stream(const int* ptr) {
    int4 v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(ptr), "l"(policy_stream()));
    return v;
}
__device__ __forceinline__ int ldg_stream(const int* ptr) {
    int v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(ptr), "l"(policy_stream()));
    return v;
}
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bulk copy global -> this CTA's shared memory, completion counted on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, unsigned bytes,
                                            unsigned long long* bar) {
    unsigned long long pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
        "%4;" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}

// First level of the traced window: p.trace_from in the profiling build, 0
// in the product build (whose level loop then compiles as if untouched).
#if DFQ_CLAIM_PROBES
#define DFQ_TRACE_FROM(p) ((p).trace_from)
#else
#define DFQ_TRACE_FROM(p) 0
#endif
// Slot of level L in the traced window of kTraceLevels levels (out of range: not traced).
#define DFQ_TSLOT(p, L) ((L) - DFQ_TRACE_FROM(p))
__device__ __forceinline__ bool in_trace(int t) { return (unsigned)t < (unsigned)kTraceLevels; }

// %globaltimer read after `dep` is available (the input ties the read to it).
__device__ __forceinline__ unsigned long long globaltimer_after(unsigned dep) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t) : "r"(dep));
    return t;
}

// Set when a thread of this block records an error: a one-block group stops
// on it without reading the status word back from global memory.
static __shared__ int s_block_err;

__device__ __forceinline__ void set_error(Control* ctl, int code, int a, int b) {
    s_block_err = 1;
    if (atomicCAS(&ctl->status, 0, code) == 0) {
        ctl->err_info[0] = a;
        ctl->err_info[1] = b;
    }
}

// Wait until `bar` completes phase `parity`; bounded by timeout_ns.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  long long timeout_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    unsigned long long t0 = globaltimer();
    for (unsigned it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63) == 63 && (long long)(globaltimer() - t0) > timeout_ns) return false;
    }
}

// Grid barrier over all co-resident blocks of a cooperative launch.  After the
// block barrier, thread 0 arrives with one release-ordered reduction on a
// monotone counter (release is cumulative over the block's writes it observed
// through the block barrier, so no separate fence is needed) and polls the
// counter with acquire loads until every block of this phase has arrived,
// bounded by timeout_ns.  Thread 0 then reads the counters of the level that
// starts (`next`) into s_in, so the rest of the block never loads them from
// global memory.  Returns false (all threads of the block) if the wait timed
// out or another block reported an error.
__device__ __forceinline__ bool grid_barrier(Control* ctl, unsigned& target, long long timeout_ns,
                                             int* s_flag, const LevelCtr* next, int* s_in, int gsize,
                                             bool skip_arrive = false) {
    __syncthreads();
    if (threadIdx.x == 0) {
        target += (unsigned)gsize;
        int ok = 1;
        if (!skip_arrive) red_add_release(&ctl->barrier, 1u);
        unsigned long long t0 = 0;
        for (unsigned it = 0;; ++it) {
            unsigned cur = ld_acquire(&ctl->barrier);
            if ((int)(cur - target) >= 0) break;
            if ((it & 255) == 255) {
                if (*(volatile int*)&ctl->status != 0) { ok = 0; break; }
                unsigned long long now = globaltimer();
                if (t0 == 0) t0 = now;
                else if ((long long)(now - t0) > timeout_ns) {
                    set_error(ctl, kErrBarrierTimeout, (int)blockIdx.x, (int)target);
                    ok = 0;
                    break;
                }
            }
        }
        if (ok) {
            // the status word and the counters in one round of loads
            const int st = *(volatile int*)&ctl->status;
            const int pushed = __ldcg(&next->pushed);
            const unsigned long long op = __ldcg(&next->ovf_pieces);
            const int edges = __ldcg(&next->pushed_edges);
            ok = st == 0;
            s_in[0] = pushed;
            s_in[1] = (int)(op >> 32);
            s_in[2] = 0;
            s_in[3] = (int)(unsigned)op;
            s_in[4] = edges;
        }
        *s_flag = ok;
    }
    __syncthreads();
    return *s_flag != 0;
}

// Tally barrier: the grid barrier of a level's end with the level's totals
// carried in the arrival words, so the poll that sees the last arrival also
// returns the next level's input (the grid barrier above reads the counters
// in one more round trip after it).  Each block adds, to two 64-bit words of
// the level's counter slot, one arrival (bit 54) plus its tallies:
//   w[0] = arrivals | frontier entries << 27 | frontier edges >> shift
//   w[1] = arrivals | overflow entries << 27 | large-list pieces
// w[1] relaxed, then w[0] with release semantics (cumulative over the
// block's writes it observed through the block barrier).  Thread 0 polls
// the status word and w[1] (relaxed) and w[0] (acquire), three loads in
// flight at once, until both words hold gsize arrivals, bounded by
// timeout_ns.  Fields are 27 bits: the host enables this barrier only for
// graphs of fewer than 2^27 vertices and groups of fewer than 1024 blocks;
// edges are counted in units of 2^shift (each block rounds up), so with
// shift = 0 (graphs of fewer than 2^27 edges) the totals are exact.  The
// slot's words are cleared with its other counters two levels ahead.
__device__ __forceinline__ bool tally_barrier(Control* ctl, int gsize, LevelCtr* next, long long timeout_ns,
                                              int* s_flag, int* s_in, unsigned long long w0,
                                              unsigned long long w1, int shift, bool skip_arrive) {
    __syncthreads();
    if (threadIdx.x == 0) {
        if (!skip_arrive) {
            red_add_relaxed_u64(&next->tally[1], w1);
            red_add_release_u64(&next->tally[0], w0);
        }
        constexpr unsigned long long kMask = (1ull << 27) - 1;
        int ok = 1;
        unsigned long long a = 0, b = 0, t0 = 0;
        for (unsigned it = 0;; ++it) {
            const int st = ld_relaxed_s32(&ctl->status);
            b = ld_relaxed_u64(&next->tally[1]);
            a = ld_acquire_u64(&next->tally[0]);
            if (st != 0) { ok = 0; break; }
            if ((int)(a >> 54) == gsize && (int)(b >> 54) == gsize) break;
            if ((it & 255) == 255) {
                const unsigned long long now = globaltimer();
                if (t0 == 0) t0 = now;
                else if ((long long)(now - t0) > timeout_ns) {
                    set_error(ctl, kErrBarrierTimeout, (int)blockIdx.x, (int)(a >> 54));
                    ok = 0;
                    break;
                }
            }
        }
        if (ok) {
            s_in[0] = (int)((a >> 27) & kMask);
            s_in[1] = (int)((b >> 27) & kMask);
            s_in[2] = 0;
            s_in[3] = (int)(b & kMask);
            s_in[4] = (int)min((a & kMask) << shift, (unsigned long long)0x7fffffff);
        }
        *s_flag = ok;
    }
    __syncthreads();
    return *s_flag != 0;
}

// Level barrier of a group of blocks running one BFS: the grid barrier above
// for several blocks; for a one-block group, the block barrier plus thread 0
// reading the counters its own block's atomics produced.
// With local_in, a one-block group's thread 0 has already written the next
// level's input into s_in from the block's own shared tallies (they are the
// whole group's), so the barrier is just the block barrier.
__device__ __forceinline__ bool group_barrier(Control* ctl, int gsize, unsigned& target, long long timeout_ns,
                                              int* s_flag, const LevelCtr* next, int* s_in, bool local_in,
                                              bool skip_arrive = false) {
    if (gsize > 1) return grid_barrier(ctl, target, timeout_ns, s_flag, next, s_in, gsize, skip_arrive);
    if (local_in) {
        __syncthreads();
        return s_block_err == 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence_block();
        const int ok = *(volatile int*)&ctl->status == 0;
        *s_flag = ok;
        if (ok) {
            s_in[0] = __ldcg(&next->pushed);
            const unsigned long long op = __ldcg(&next->ovf_pieces);
            s_in[1] = (int)(op >> 32);
            s_in[2] = 0;
            s_in[3] = (int)(unsigned)op;
            s_in[4] = __ldcg(&next->pushed_edges);
        }
    }
    __syncthreads();
    return *s_flag != 0;
}

// ------------------------------------------------------------ shared layout
constexpr int kRing = 256;  // per-warp candidate ring (entries, power of two)
constexpr int kHotWordsMax = 8192;  // hot-vertex visited cache: 32 KB, 262,144 vertices

// Words of a hot-vertex cache of `kb` KB (0 if kb <= 0), rounded down to 4 KB,
// at most kHotWordsMax.
__host__ __device__ inline int hot_limit_words(int kb) {
    const int w = kb > 0 ? (kb / 4) * 1024 : 0;
    return w < kHotWordsMax ? w : kHotWordsMax;
}

// Hot-cache words for a graph of n vertices under a launch limit: whole
// 32-word groups of the graph's bitmap (a multiple of 4 for 16-byte copies).
__host__ __device__ inline int hot_words_of(int limit_words, int n) {
    const int words = ((n + 31) / 32) & ~31;
    return words < limit_words ? words : limit_words;
}

// Tallies a block of a cluster group sends at the end of a level: frontier
// entries, overflow entries, large entries, pieces, frontier edges, and 1 if
// the block saw an error (a sum over the cluster, so every block decides alike).
constexpr int kClTally = 6;

struct SmemLayout {
    int q_off;     // local queues: 2 buffers x {start, deg, v} x cap ints
    int wl_off;    // per-warp gather scratch: {scan, start, parent} x 32 ints
    int ring_off;  // per-warp candidate ring: kRing vertices (+ kRing parents)
    int tma_off;   // per-warp piece buffers: 2 x (piece + 16) ints, 128-byte aligned
    int bar_off;   // per-warp mbarriers: 2 x u64
    int hot_off;   // hot-vertex visited cache (last, so its size changes no other offset)
    int bytes;     // without the hot cache: a launch adds 4 * hot_words
};
__host__ __device__ inline SmemLayout smem_layout(int B, int cap, int piece, bool par) {
    SmemLayout L;
    const int NW = B / 32;
    int o = 0;
    L.q_off = o;    o += 2 * 3 * cap * 4;
    L.wl_off = o;   o += NW * 3 * 32 * 4;
    L.ring_off = o; o += NW * kRing * (par ? 2 : 1) * 4;
    o = (o + 127) & ~127;
    L.tma_off = o;  o += NW * 2 * (piece + 16) * 4;
    o = (o + 15) & ~15;
    L.bar_off = o;  o += NW * 2 * 8;
    o = (o + 15) & ~15;
    L.hot_off = o;
    L.bytes = o;
    return L;
}


// ------------------------------------------------------------ block state
// Shared scalars of the running block.  Device functions name them directly
// (static shared addresses cost no registers), and read the launch
// parameters from the parameter bank, so the per-edge code keeps few values
// live across the level loop.
struct BlockShared {
    unsigned long long local_pack;  // (entries << 32) | edges of the next local queue
    int cnt_cur;                    // entries of the local queue being expanded
    int local_grab;                 // cursor over it (32 entries per warp grab)
    int ovf_pushed;                 // entries this block sent to the overflow queue
    int large_pushed;               // entries this block sent to the large queue
    int large_pieces;               // pieces of those entries
    int claimed;                    // this block claimed a vertex at this level
    int flag;                       // barrier result (1 = proceed)
    int in[5];                      // this level's input: pushed, overflow, large entries, pieces, edges
    int ovf_edges;                  // degree sum of this block's overflow pushes at this level
    int large_edges;                // degree sum of this block's large pushes at this level
    int depth;                      // deepest level this block claimed into
    unsigned long long overflow;    // entries this block sent to the overflow queue (whole BFS)
    unsigned long long large;       // entries this block sent to the large queue (whole BFS)
    unsigned long long red[2];
    int hot_off;                    // byte offset of the hot-vertex cache in dynamic shared memory
    // cluster groups: the level barrier's mbarrier (one arrival per block of
    // the cluster each phase), its next phase parity, the tallies this block
    // sends at the end of a level, and three rotating slots in which every
    // block of the cluster adds its tallies to this block's copy
    unsigned long long cl_bar;
    unsigned cl_parity;
    int cl_out[kClTally];
    int cl_in[3][kClTally];
    unsigned long long level_t0[32];  // profiling: when each warp started the level
    unsigned phase_max[4];            // profiling: this block's latest warp phase ends
#if DFQ_CLAIM_PROBES
    unsigned long long acc[32][4];    // profiling build: per-warp sums for trace_piece, flushed per level
    unsigned claim_max[4];            // profiling build: this block's latest claim steps, flushed per level
#endif
};
static __shared__ BlockShared sh;
extern __shared__ __align__(128) unsigned char dfq_smem[];

// Profiling build: add v to this warp's accumulator k (lane 0 calls it).
__device__ __forceinline__ void acc_add(int k, unsigned long long v) {
#if DFQ_CLAIM_PROBES
    sh.acc[threadIdx.x >> 5][k] += v;
#else
    (void)k;
    (void)v;
#endif
}

// ------------------------------------------------------------ cluster groups
__device__ __forceinline__ unsigned cluster_addr(const void* local, unsigned rank) {
    unsigned a;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_u32(local)), "r"(rank));
    return a;
}
__device__ __forceinline__ void red_add_cluster(unsigned addr, int v) {
    asm volatile("red.relaxed.cluster.shared::cluster.add.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ void mbar_arrive_cluster(unsigned addr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(addr) : "memory");
}
// Wait until this block's cluster mbarrier completes phase `parity` (acquire
// at cluster scope); bounded by timeout_ns.
__device__ __forceinline__ bool mbar_wait_cluster(unsigned long long* bar, unsigned parity, long long timeout_ns) {
    unsigned long long t0 = 0;
    for (unsigned it = 0;; ++it) {
        unsigned done;
        asm volatile(
            "{ .reg .pred q; mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 q, [%1], %2; selp.u32 %0, 1, 0, q; }"
            : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
        if (done) return true;
        if ((it & 63) == 63) {
            const unsigned long long now = globaltimer();
            if (t0 == 0) t0 = now;
            else if ((long long)(now - t0) > timeout_ns) return false;
        }
    }
}
// Every thread of every block of the cluster (hardware cluster barrier).  Only
// at the start and the end of a run, which every block reaches: each wait in
// between is bounded, and a block that gives up still comes here.
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Set up the level barrier of a cluster group of gsize blocks, then the
// hardware barrier, so that no block reaches another's shared memory before
// that block has initialised it.
__device__ __forceinline__ void cluster_group_begin(int gsize) {
    if (threadIdx.x == 0) {
        mbar_init(&sh.cl_bar, (unsigned)gsize);
        sh.cl_parity = 0;
        for (int k = 0; k < kClTally; ++k) {
            sh.cl_out[k] = 0;
            for (int j = 0; j < 3; ++j) sh.cl_in[j][k] = 0;
        }
        mbar_fence_init();
    }
    __syncthreads();
    cluster_sync_all();
}

// Level barrier of a cluster group.  Thread r < gsize of each block adds the
// block's tallies (sh.cl_out) to block r's copy of slot `slot`, then arrives
// on block r's mbarrier with release semantics at cluster scope (cumulative
// over the block's writes it observed through the block barrier); thread 0
// waits for its own mbarrier's phase with acquire semantics, bounded.  The
// sums in this block's slot are then the group's, the same in every block.
// A slot is written only at the end of a level and read after its barrier;
// after barrier b this block clears its copy of barrier b-1's slot, which is
// next written for barrier b+2, i.e. by blocks past barrier b+1, which needs
// this block's arrival.  sh.cl_out is rewritten by thread 0 at the end of
// every level, after the block barrier that ends this one.
// first: the counters of level 0 come from the control block (set by the
// group's first thread before the barrier).
__device__ __forceinline__ bool cluster_barrier(Control* ctl, int gsize, int slot, long long timeout_ns,
                                                const LevelCtr* next, bool first, bool skip_arrive) {
    __syncthreads();
    const int tid = (int)threadIdx.x;
    if (tid < gsize && !skip_arrive) {
        const unsigned base = cluster_addr(&sh.cl_in[slot][0], (unsigned)tid);
        for (int k = 0; k < kClTally; ++k)
            if (sh.cl_out[k]) red_add_cluster(base + 4u * k, sh.cl_out[k]);
        mbar_arrive_cluster(cluster_addr(&sh.cl_bar, (unsigned)tid));
    }
    if (tid == 0) {
        int ok = mbar_wait_cluster(&sh.cl_bar, sh.cl_parity, timeout_ns) ? 1 : 0;
        sh.cl_parity ^= 1u;
        if (!ok) {
            set_error(ctl, kErrBarrierTimeout, (int)blockIdx.x, slot);
        } else if (first) {
            sh.in[0] = __ldcg(&next->pushed);
            const unsigned long long op = __ldcg(&next->ovf_pieces);
            sh.in[1] = (int)(op >> 32);
            sh.in[2] = 0;
            sh.in[3] = (int)(unsigned)op;
            sh.in[4] = __ldcg(&next->pushed_edges);
            ok = *(volatile int*)&ctl->status == 0;
        } else {
            for (int k = 0; k < 5; ++k) sh.in[k] = sh.cl_in[slot][k];
            ok = sh.cl_in[slot][5] == 0;
        }
        const int prev = (slot + 2) % 3;  // the previous barrier's slot
        for (int k = 0; k < kClTally; ++k) sh.cl_in[prev][k] = 0;
        sh.flag = ok;
    }
    __syncthreads();
    return sh.flag != 0;
}

// Uniform per-level values.
struct Lv {
    int next;   // level being written (L + 1)
    int out;    // parity of the output queues (L + 1) & 1
    int cslot;  // counter slot of the output frontier (L + 1) % 3
    int qn;     // local queue buffer being filled
    int cap;    // entries this block may keep locally at this level
    int ecap;   // edges (degree sum) this block may keep locally at this level
    int probe;  // probe the bitmap before claiming
    unsigned hot;  // vertices below this id have visited bits in the shared cache (0: none)
    int bottom_up; // this level: every unvisited vertex looks for a parent in the frontier
};

// The block's hot-vertex visited cache (shared memory).  A set bit means the
// vertex is visited (bits are only ever set); a clear bit means "ask the
// global bitmap".
__device__ __forceinline__ unsigned* hot_cache() { return reinterpret_cast<unsigned*>(dfq_smem + sh.hot_off); }

// Record in the shared cache that v is visited (v < lv.hot).  Done for the
// block's own claims only: learning from every probe that finds a visited
// vertex costs more shared-memory atomics than it saves.
__device__ __forceinline__ void hot_learn(const Lv& lv, int v) {
    if ((unsigned)v < lv.hot) atomicOr(&hot_cache()[v >> 5], 1u << (v & 31));
}

// Per-thread tallies (32-bit: one thread never scans 2^32 edges, e < 2^31).
struct Tally {
    unsigned edges;
    unsigned claims;
};

// This warp's ring of unvisited candidates (probe levels): entries
// [head, head + n) modulo kRing; head and n are warp-uniform.
struct Ring {
    int* v;    // kRing vertices, then kRing parents when parents are kept
    int head;
    int n;
};

// Drop from vm the entries the shared hot-vertex cache already knows to be
// visited; the rest go on to the global bitmap.
template <int K>
__device__ __forceinline__ unsigned hot_filter(const Lv& lv, const int (&v)[K], unsigned vm) {
    if (!lv.hot) return vm;
    const unsigned* hc = hot_cache();
    unsigned hw[K];
#pragma unroll
    for (int j = 0; j < K; ++j) hw[j] = ((vm >> j & 1) && (unsigned)v[j] < lv.hot) ? hc[v[j] >> 5] : 0u;
#pragma unroll
    for (int j = 0; j < K; ++j)
        if ((hw[j] >> (v[j] & 31)) & 1u) vm &= ~(1u << j);
    return vm;
}

// Pieces of a list [st, st + dg) cut at multiples of the piece size counted
// from its 16-byte aligned floor a0 = st & ~3: every piece's staged span is
// at most piece_edges entries and starts aligned.
__device__ __forceinline__ int pieces_of(int st, int dg, int P) { return (st + dg - (st & ~3) + P - 1) / P; }

// Push this warp's claimed vertices (bit j of loc / lm: entry j of this lane
// is small / large).  Small entries go to the block's next local queue,
// all-or-nothing per warp against its entry limit and edge budget, else to
// the global overflow queue; large entries become pieces.  The overflow
// slots and the pieces of the whole warp come from ONE 64-bit atomic on the
// level's (overflow entries << 32 | pieces) word, handed out in lane order:
// levels that claim hundreds of thousands of vertices otherwise queue behind
// same-address atomics.  Warp-collective.
template <bool PAR>
__device__ __forceinline__ void push_claims(const Params& p, const Lv& lv, unsigned loc, unsigned lm,
                                            const int (&st)[4], const int (&dg)[4], const int (&v)[4]) {
    if (!__any_sync(kFull, loc | lm)) return;
    const int lane = threadIdx.x & 31;
    const int P = p.piece_edges;
    int cnt = __popc(loc), npl = 0;
    unsigned dsum = 0, dlarge = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (loc >> j & 1) dsum += (unsigned)dg[j];
        if (lm >> j & 1) {
            npl += pieces_of(st[j], dg[j], P);
            dlarge += (unsigned)dg[j];
        }
    }
    // one scan for both prefix sums: small entries (< 2^7 per warp) in the
    // high bits, pieces (< 2^24 per warp) in the low bits
    int incl = (cnt << 24) | npl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int tt = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += tt;
    }
    const int tot_both = __shfl_sync(kFull, incl, 31);
    const int tot = (int)((unsigned)tot_both >> 24), totp = tot_both & 0xffffff;
    const int tsum = (int)__reduce_add_sync(kFull, dsum);
    int base = -1, gbase = 0;
    unsigned pbase = 0;
    if (lane == 0) {
        if (tot > 0) {
            unsigned long long old = *(volatile unsigned long long*)&sh.local_pack;
            while (true) {
                const unsigned n_ent = (unsigned)(old >> 32), n_deg = (unsigned)old;
                if (n_ent + (unsigned)tot > (unsigned)lv.cap || n_deg + (unsigned)tsum > (unsigned)lv.ecap)
                    break;
                const unsigned long long want =
                    ((unsigned long long)(n_ent + tot) << 32) | (unsigned long long)(n_deg + (unsigned)tsum);
                const unsigned long long seen = atomicCAS(&sh.local_pack, old, want);
                if (seen == old) { base = (int)n_ent; break; }
                old = seen;
            }
        }
        const int to_ovf = (tot > 0 && base < 0) ? tot : 0;
        if (to_ovf || totp) {
            const unsigned long long old = atomicAdd(&p.ctl->lv[lv.cslot].ovf_pieces,
                                                     ((unsigned long long)to_ovf << 32) | (unsigned)totp);
            gbase = (int)(old >> 32);
            pbase = (unsigned)old;
        }
        if (to_ovf) {
            atomicAdd(&sh.ovf_pushed, to_ovf);
            atomicAdd(&sh.ovf_edges, tsum);
        }
        if (totp) {
            atomicAdd(&sh.large_pieces, totp);
            if (pbase + (unsigned)totp > (unsigned)p.piece_cap) set_error(p.ctl, kErrQueueCap, (int)pbase, totp);
        }
    }
    if (totp) {  // warp-uniform: entry and edge tallies of the large claims
        const unsigned totc = __reduce_add_sync(kFull, (unsigned)__popc(lm));
        const unsigned totd = __reduce_add_sync(kFull, dlarge);
        if (lane == 0) {
            atomicAdd(&sh.large_pushed, (int)totc);
            atomicAdd(&sh.large_edges, (int)totd);
        }
    }
    base = __shfl_sync(kFull, base, 0);
    gbase = __shfl_sync(kFull, gbase, 0);
    pbase = __shfl_sync(kFull, pbase, 0);

    // small entries
    int pos = (int)((unsigned)incl >> 24) - cnt;
    if (base >= 0) {
        int* qs = reinterpret_cast<int*>(dfq_smem) + lv.qn * 3 * p.local_cap;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (loc >> j & 1) {
                qs[base + pos] = st[j];
                qs[p.local_cap + base + pos] = dg[j];
                if (PAR) qs[2 * p.local_cap + base + pos] = v[j];
                ++pos;
            }
        }
    } else if (tot > 0) {
        int2* ovf = lv.out ? p.ovf[1] : p.ovf[0];
        int* ovfv = lv.out ? p.ovfv[1] : p.ovfv[0];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (loc >> j & 1) {
                const int gi = gbase + pos;
                if (gi < p.ovf_cap) {
                    ovf[gi] = make_int2(st[j], dg[j]);
                    if (PAR) ovfv[gi] = v[j];
                } else {
                    set_error(p.ctl, kErrQueueCap, gi, p.ovf_cap);
                }
                ++pos;
            }
        }
    }
    if (!totp) return;

    // pieces (dropped past the capacity, where the error is recorded above;
    // readers clamp the piece count to the capacity, so every piece read was
    // written at this level).  Lists of a few pieces: each lane writes its
    // own; longer lists (hubs, up to thousands of pieces) the whole warp.
    unsigned poff = pbase + (unsigned)((incl & 0xffffff) - npl);
    int2* pc = lv.out ? p.piece[1] : p.piece[0];
    int* pv = lv.out ? p.piece_v[1] : p.piece_v[0];
    constexpr int kOwn = 32;  // per lane up to this many pieces; giants cooperatively
    unsigned big = 0;
    unsigned boff[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (!(lm >> j & 1)) continue;
        const int np = pieces_of(st[j], dg[j], P);
        boff[j] = poff;
        if (np > kOwn) {
            big |= 1u << j;
        } else {
            const int a0 = st[j] & ~3, e1 = st[j] + dg[j];
            for (int i = 0; i < np && poff + (unsigned)i < (unsigned)p.piece_cap; ++i) {
                pc[poff + i] = make_int2(max(st[j], a0 + i * P), min(e1, a0 + (i + 1) * P));
                if (PAR) pv[poff + i] = v[j];
            }
        }
        poff += (unsigned)np;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        unsigned m = __ballot_sync(kFull, big >> j & 1);
        while (m) {
            const int i = __ffs(m) - 1;
            m &= m - 1;
            const int s0 = __shfl_sync(kFull, st[j], i), d0 = __shfl_sync(kFull, dg[j], i);
            const int v0 = __shfl_sync(kFull, v[j], i);
            const unsigned o0 = __shfl_sync(kFull, boff[j], i);
            const int a0 = s0 & ~3, e1 = s0 + d0, np = pieces_of(s0, d0, P);
            for (int k = lane; k < np && o0 + (unsigned)k < (unsigned)p.piece_cap; k += 32) {
                pc[o0 + k] = make_int2(max(s0, a0 + k * P), min(e1, a0 + (k + 1) * P));
                if (PAR) pv[o0 + k] = v0;
            }
        }
    }
}

// Claim up to four candidates per lane (bit j of vm: v[j]), with each one's
// row bounds loaded alongside its atomicOr; record and push what this warp
// wins.  On levels that do not probe, the winners' rows are also prefetched
// into L2 for the next level.  Warp-collective.
template <bool PAR>
__device__ __forceinline__ void claim4(const Params& p, const Lv& lv, Tally& t, const int (&v)[4], unsigned vm,
                                       const int (&par)[4]) {
    const int slot = DFQ_TSLOT(p, lv.next - 1);  // traced level window
    const bool probes = DFQ_CLAIM_PROBES && p.profile && (unsigned)slot < (unsigned)kTraceLevels &&
                        (threadIdx.x & 31) == 0;
    auto probe_at = [&](int k, unsigned dep) {
#if DFQ_CLAIM_PROBES
        if (probes)
            atomicMax(&sh.claim_max[k], (unsigned)(globaltimer_after(dep) - sh.level_t0[threadIdx.x >> 5]));
#else
        (void)k;
        (void)dep;
#endif
    };
    probe_at(0, (unsigned)v[0]);
    // claim-at-once levels load the row bounds alongside the claim atomics;
    // probe levels, whose candidates often lose the claim (many warps met
    // the same vertex), load them for the winners only (RMAT-22 0.4747 ->
    // 0.4718 ms)
    int so[4], eo[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        so[j] = 0;
        eo[j] = 0;
        if (!lv.probe && (vm >> j & 1)) {
            so[j] = __ldg(p.offsets + v[j]);
            eo[j] = __ldg(p.offsets + v[j] + 1);
        }
    }
    probe_at(1, (unsigned)(so[0] + eo[0] + so[3] + eo[3]));
    // all four claim atomics are issued before any result is looked at, so a
    // lane waits for one atomic round trip, not four in a row (a hub is
    // claimed on its own word; its winner then sets the hub's bitmap bit for
    // the probes with a reduction whose result nobody waits for)
    unsigned old[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        old[j] = 0xffffffffu;
        if (!(vm >> j & 1)) continue;
        const bool hub = v[j] < p.hub_n;
        unsigned* word = hub ? p.hub_claim + v[j] * kHubStride : p.bitmap + (v[j] >> 5);
        old[j] = atomicOr(word, 1u << (v[j] & 31));
    }
    unsigned won = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (!(vm >> j & 1)) continue;
        const unsigned bit = 1u << (v[j] & 31);
        if (!(old[j] & bit)) {
            won |= 1u << j;
            if (v[j] < p.hub_n) atomicOr(&p.bitmap[v[j] >> 5], bit);
        }
        hot_learn(lv, v[j]);  // visited now, whoever won
    }
    if (lv.probe) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (won >> j & 1) {
                so[j] = __ldg(p.offsets + v[j]);
                eo[j] = __ldg(p.offsets + v[j] + 1);
            }
    }
    int st[4], dg[4];
    unsigned loc = 0, lm = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        st[j] = 0;
        dg[j] = 0;
        if (!(won >> j & 1)) continue;
        p.levels[v[j]] = lv.next;
        if (PAR) p.parents[v[j]] = par[j];
        st[j] = so[j];
        dg[j] = eo[j] - so[j];
        if (!lv.probe && dg[j] > 0) {
            // small frontier: pull the row this vertex expands at the next
            // level into L2 now, off the next level's critical path
            prefetch_l2(p.cols + st[j]);
            if (dg[j] > 32) prefetch_l2(p.cols + st[j] + dg[j] - 1);
        }
        if (dg[j] >= p.large_min) lm |= 1u << j;
        else if (dg[j] > 0) loc |= 1u << j;
    }
    probe_at(2, won | old[0] | old[3]);
    if (won) {
        t.claims += __popc(won);
        sh.claimed = 1;
    }
    push_claims<PAR>(p, lv, loc, lm, st, dg, v);
    probe_at(3, (unsigned)sh.local_grab);
}

// Levels that do not probe: claim the scanned neighbours at once.
// Warp-collective.
template <bool PAR>
__device__ __forceinline__ void visit4(const Params& p, const Lv& lv, Tally& t, const int (&v)[4], unsigned vmask,
                                       const int (&par)[4]) {
    t.edges += __popc(vmask);
    claim4<PAR>(p, lv, t, v, vmask, par);
}

// Claim buffered candidates 128 at a time (four per lane) while at least
// 128 are waiting, or until the ring is empty when `all`.  Larger batches
// mean fewer pushes, so fewer atomics on the level's counters.
// Warp-collective.
template <bool PAR>
__device__ __forceinline__ void ring_drain(const Params& p, const Lv& lv, Tally& t, Ring& r, bool all) {
    const int lane = threadIdx.x & 31;
    const int dslot = DFQ_TSLOT(p, lv.next - 1);
    const bool dprobe = DFQ_CLAIM_PROBES && p.profile && in_trace(dslot) && lane == 0 &&
                        (r.n >= 128 || (all && r.n > 0));
    const unsigned long long d0 = dprobe ? globaltimer() : 0ull;
    while (r.n >= 128 || (all && r.n > 0)) {
        const int take = r.n < 128 ? r.n : 128;
        int v[4], par[4];
        unsigned vm = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            v[j] = 0;
            par[j] = 0;
            const int k = j * 32 + lane;
            if (k < take) {
                const int idx = (r.head + k) & (kRing - 1);
                v[j] = r.v[idx];
                if (PAR) par[j] = r.v[kRing + idx];
                vm |= 1u << j;
            }
        }
        __syncwarp();
        r.head = (r.head + take) & (kRing - 1);
        r.n -= take;
        claim4<PAR>(p, lv, t, v, vm, par);
    }
    if (dprobe) acc_add(3, globaltimer_after(t.claims) - d0);
}

// Probe levels: test up to four neighbours per lane against the visited
// bitmap and append the unvisited ones to the warp's ring (prefix-sum
// compaction); claims happen in batches of 128 in ring_drain.  The ring
// holds < 128 entries between calls, so one call (<= 128 appends) never
// wraps onto unclaimed entries.  Warp-collective.
template <bool PAR>
__device__ __forceinline__ void probe4(const Params& p, const Lv& lv, Tally& t, Ring& r, const int (&v)[4],
                                       unsigned vmask, const int (&par)[4]) {
    const int lane = threadIdx.x & 31;
    t.edges += __popc(vmask);
    vmask = hot_filter<4>(lv, v, vmask);
    unsigned w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) w[j] = (vmask >> j & 1) ? p.bitmap[v[j] >> 5] : 0xffffffffu;
    unsigned cm = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if ((vmask >> j & 1) && !((w[j] >> (v[j] & 31)) & 1u)) cm |= 1u << j;
    const int c = __popc(cm);
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int tt = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += tt;
    }
    const int tot = __shfl_sync(kFull, incl, 31);
    if (tot == 0) return;
    int pos = r.head + r.n + incl - c;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (cm >> j & 1) {
            const int idx = pos & (kRing - 1);
            r.v[idx] = v[j];
            if (PAR) r.v[kRing + idx] = par[j];
            ++pos;
        }
    }
    __syncwarp();
    r.n += tot;
    ring_drain<PAR>(p, lv, t, r, false);
}

// Probe levels, eight neighbours per lane (all of one vertex, par0): the
// eight bitmap loads are in flight together; candidates are appended in two
// halves of at most 128 with a drain between, so the ring (< 128 entries
// between calls) never holds more than 255.  One scan serves both halves
// (counts packed in 16-bit fields).  Warp-collective.
template <bool PAR>
__device__ __forceinline__ void probe8(const Params& p, const Lv& lv, Tally& t, Ring& r, const int (&v)[8],
                                       unsigned vm, int par0) {
    const int lane = threadIdx.x & 31;
    t.edges += __popc(vm);
    vm = hot_filter<8>(lv, v, vm);
    unsigned w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) w[j] = (vm >> j & 1) ? p.bitmap[v[j] >> 5] : 0xffffffffu;
    unsigned cm = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if ((vm >> j & 1) && !((w[j] >> (v[j] & 31)) & 1u)) cm |= 1u << j;
    if (!__any_sync(kFull, cm)) return;
    const int c_lo = __popc(cm & 15u), c_hi = __popc(cm >> 4);
    int incl = c_lo | (c_hi << 16);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int tt = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += tt;
    }
    const int tot = __shfl_sync(kFull, incl, 31);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int th = h ? (tot >> 16) : (tot & 0xffff);
        if (th == 0) continue;
        int pos = r.head + r.n + (h ? (incl >> 16) - c_hi : (incl & 0xffff) - c_lo);
#pragma unroll
        for (int j = 4 * h; j < 4 * h + 4; ++j) {
            if (cm >> j & 1) {
                const int idx = pos & (kRing - 1);
                r.v[idx] = v[j];
                if (PAR) r.v[kRing + idx] = par0;
                ++pos;
            }
        }
        __syncwarp();
        r.n += th;
        ring_drain<PAR>(p, lv, t, r, false);
    }
}

// Expand one staged piece on a probe level: buf holds entries [0, tw) of the
// piece's aligned span, the piece itself is [off, tw); lanes take eight
// consecutive entries (two 16-byte shared-memory reads).  Warp-collective.
template <bool PAR>
__device__ __forceinline__ void probe_piece(const Params& p, const Lv& lv, Tally& t, Ring& r, const int* buf,
                                            int off, int tw, int par0) {
    const int lane = threadIdx.x & 31;
    for (int base = 0; base < tw; base += 256) {
        const int w8 = base + 8 * lane;
        int4 x0 = make_int4(0, 0, 0, 0), x1 = x0;
        if (w8 < tw) x0 = *reinterpret_cast<const int4*>(buf + w8);
        if (w8 + 4 < tw) x1 = *reinterpret_cast<const int4*>(buf + w8 + 4);
        const int v[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
        unsigned vm = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (w8 + j >= off && w8 + j < tw) vm |= 1u << j;
        probe8<PAR>(p, lv, t, r, v, vm, par0);
    }
}

// Probe or claim-at-once, by level.  Warp-collective.
template <bool PAR>
__device__ __forceinline__ void scan4(const Params& p, const Lv& lv, Tally& t, Ring& r, const int (&v)[4],
                                      unsigned vmask, const int (&par)[4]) {
    if (lv.probe) probe4<PAR>(p, lv, t, r, v, vmask, par);
    else visit4<PAR>(p, lv, t, v, vmask, par);
}

// One warp expands one list [s, s+d): int4 column loads from the 16-byte
// aligned floor of the list; lanes mask what lies outside it.
template <bool PAR>
__device__ __forceinline__ void warp_expand(const Params& p, const Lv& lv, Tally& t, Ring& r, int s, int d, int u) {
    const int lane = threadIdx.x & 31;
    const int e0 = s, e1 = s + d;
    const int par[4] = {u, u, u, u};
    for (int base = e0 & ~3; base < e1; base += 128) {
        const int k4 = base + lane * 4;
        int4 x = make_int4(0, 0, 0, 0);
        unsigned vm = 0;
        if (k4 < e1) {
            x = lv.probe ? ldg4_stream(p.cols + k4) : ldg4(p.cols + k4);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (k4 + j >= e0 && k4 + j < e1) vm |= 1u << j;
        }
        const int v[4] = {x.x, x.y, x.z, x.w};
        scan4<PAR>(p, lv, t, r, v, vm, par);
    }
}

// Expand one frontier entry per lane (has == false: no entry).  Medium
// entries one at a time with the whole warp; small entries by a warp-level
// gather over the concatenation of their lists (4 edges per lane per round).
// wl: this warp's 96-int scratch (scan, start, parent).  Warp-collective.
template <bool PAR>
__device__ __forceinline__ void warp_process(const Params& p, const Lv& lv, Tally& t, Ring& r, int* wl, bool has,
                                             int s, int d, int u) {
    const int lane = threadIdx.x & 31;
    if (!has) d = 0;
    const bool med = d >= p.medium_min;
    unsigned mmask = __ballot_sync(kFull, med);
    while (mmask) {
        const int i = __ffs(mmask) - 1;
        mmask &= mmask - 1;
        warp_expand<PAR>(p, lv, t, r, __shfl_sync(kFull, s, i), __shfl_sync(kFull, d, i), __shfl_sync(kFull, u, i));
    }
    const int ds = med ? 0 : d;
    int incl = ds;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int tt = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += tt;
    }
    const int T = __shfl_sync(kFull, incl, 31);
    if (T == 0) return;
    __syncwarp();
    wl[lane] = incl - ds;
    wl[32 + lane] = s;
    if (PAR) wl[64 + lane] = u;
    __syncwarp();
    for (int base = 0; base < T; base += 128) {
        int v[4], par[4];
        unsigned vm = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = base + j * 32 + lane;
            v[j] = 0;
            par[j] = 0;
            if (k < T) {
                // owner = largest index with scan <= k (scan[0] = 0 <= k and scan
                // is non-decreasing, so this lands on an entry with k inside its
                // list); steps 16+8+4+2+1 keep own + step <= 31
                int own = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (wl[own + step] <= k) own += step;
                const int* cp = p.cols + wl[32 + own] + (k - wl[own]);
                v[j] = lv.probe ? ldg_stream(cp) : __ldg(cp);
                if (PAR) par[j] = wl[64 + own];
                vm |= 1u << j;
            }
        }
        scan4<PAR>(p, lv, t, r, v, vm, par);
    }
}

// Bottom-up level: every unvisited vertex v looks among its neighbours for
// one at the current level; the first found becomes its parent.  A lane
// checks its own vertices' first 32 neighbours (with hub-first ids the row's
// hub comes first); lists still unresolved after that are finished by the
// whole warp, 32 neighbours at a time.  Only v's lane writes v, so no claim
// atomics are needed; levels are read through L2 (other blocks wrote this
// level's).  Found vertices are pushed like claims, so the next level can run
// either way.  Warp-collective.
template <bool PAR>
__device__ __forceinline__ void bottom_up_level(const Params& p, const Lv& lv, Tally& t, int gwarp, int nwarps) {
    const int lane = threadIdx.x & 31;
    const int L = lv.next - 1;
    // four vertices per lane: their first checks (own level, row bounds, the
    // first neighbour - the row's hub - and its level) are in flight together
    for (int base = gwarp * 128; base < p.n; base += nwarps * 128) {
        int s0[4], e0[4], par[4], v[4];
        unsigned unv = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            v[j] = base + j * 32 + lane;
            s0[j] = e0[j] = 0;
            par[j] = -1;
            if (v[j] < p.n && __ldcg(p.levels + v[j]) == -1) unv |= 1u << j;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (unv >> j & 1) {
                s0[j] = __ldg(p.offsets + v[j]);
                e0[j] = __ldg(p.offsets + v[j] + 1);
            }
        int u0[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) u0[j] = ((unv >> j & 1) && e0[j] > s0[j]) ? __ldg(p.cols + s0[j]) : -1;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (u0[j] >= 0 && __ldcg(p.levels + u0[j]) == L) par[j] = u0[j];
        unsigned open = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (!(unv >> j & 1) || par[j] >= 0) continue;
            // the rest of the first 32 neighbours, one at a time
            const int lim = min(e0[j], s0[j] + 32);
            for (int k = s0[j] + 1; k < lim; ++k) {
                const int u = __ldg(p.cols + k);
                if (__ldcg(p.levels + u) == L) { par[j] = u; break; }
            }
            if (par[j] < 0 && e0[j] > s0[j] + 32) open |= 1u << j;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            unsigned rest = __ballot_sync(kFull, open >> j & 1);
            while (rest) {  // long lists, one at a time with the whole warp
                const int i = __ffs(rest) - 1;
                rest &= rest - 1;
                const int rs = __shfl_sync(kFull, s0[j], i) + 32, re = __shfl_sync(kFull, e0[j], i);
                int got = -1;
                for (int k0 = rs; k0 < re && got < 0; k0 += 32) {
                    const int k = k0 + lane;
                    const int u = k < re ? __ldg(p.cols + k) : -1;
                    const bool hit = u >= 0 && __ldcg(p.levels + u) == L;
                    const unsigned hm = __ballot_sync(kFull, hit);
                    if (hm) got = __shfl_sync(kFull, u, __ffs(hm) - 1);
                }
                if (lane == i) par[j] = got;
            }
        }
        int st[4], dg[4];
        unsigned loc = 0, lm = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            st[j] = dg[j] = 0;
            if (par[j] < 0) continue;
            p.levels[v[j]] = lv.next;
            if (PAR) p.parents[v[j]] = par[j];
            atomicOr(&p.bitmap[v[j] >> 5], 1u << (v[j] & 31));
            if (v[j] < p.hub_n) p.hub_claim[v[j] * kHubStride] = 1u << (v[j] & 31);
            t.claims += 1;
            sh.claimed = 1;
            st[j] = s0[j];
            dg[j] = e0[j] - s0[j];
            if (dg[j] >= p.large_min) lm |= 1u << j;
            else if (dg[j] > 0) loc |= 1u << j;
        }
        push_claims<PAR>(p, lv, loc, lm, st, dg, v);
    }
}

// Per-warp state that outlives one BFS within a launch: the parity of each
// of the warp's two mbarriers, and whether a bulk copy ever failed to land.
struct WarpState {
    unsigned phase_bits;
    bool failed;
};

// One whole BFS (init, levels, statistics) run by a group of `gsize` blocks;
// this block is number `grank` of the group.  The group is the whole grid of
// a cooperative launch, or a single block; with CL, the one thread-block
// cluster of the launch (cluster barrier between levels).  Block-collective.
template <int B, bool PAR, bool CL = false>
__device__ __forceinline__ bool bfs_run(const Params& p, int gsize, int grank, WarpState& ws) {
    constexpr int NW = B / 32;
    if (gsize < 1 || grank < 0 || grank >= gsize) {  // a caller bug: refuse rather than loop
        if (threadIdx.x == 0) set_error(p.ctl, kErrQueueCap, gsize, grank);
        return false;
    }
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // group-wide warp index, interleaved across blocks so that consecutive
    // statically assigned chunks land on different SMs
    const int gwarp = warp * gsize + grank, nwarps = gsize * NW;
    const SmemLayout lay = smem_layout(B, p.local_cap, p.piece_edges, PAR);
    const int P = p.piece_edges;
    int* wl = reinterpret_cast<int*>(dfq_smem + lay.wl_off) + warp * 96;
    Ring ring;
    ring.v = reinterpret_cast<int*>(dfq_smem + lay.ring_off) + warp * kRing * (PAR ? 2 : 1);
    ring.head = 0;
    ring.n = 0;
    int* wbuf0 = reinterpret_cast<int*>(dfq_smem + lay.tma_off) + warp * 2 * (P + 16);
    unsigned long long* wbar = reinterpret_cast<unsigned long long*>(dfq_smem + lay.bar_off) + warp * 2;
    Control* ctl = p.ctl;

    // ---- init: levels, parents, bitmap (source pre-set so no ordering is needed)
    const int src = p.map_src ? __ldg(p.rank + p.src) : p.src;
    {
        const long long gtid = (long long)grank * B + tid;
        const long long nth = (long long)gsize * B;
        for (long long i = gtid; i < p.n; i += nth) {
            p.levels[i] = (i == src) ? 0 : -1;
            if (PAR) p.parents[i] = (i == src) ? src : -1;
        }
        for (long long w = gtid; w < p.bitmap_words; w += nth)
            p.bitmap[w] = (w == (src >> 5)) ? (1u << (src & 31)) : 0u;
        for (long long h = gtid; h < p.hub_n; h += nth)
            p.hub_claim[h * kHubStride] = (h == src) ? (1u << (src & 31)) : 0u;
        if (gtid == 0) {
            const int s0 = p.offsets[src], d = p.offsets[src + 1] - s0;
            if (d > 0) {
                if (d >= p.large_min) {
                    // the source's list in pieces, cut as push_claims cuts lists
                    const int a0 = s0 & ~3, np = (s0 + d - a0 + P - 1) / P;
                    if (np <= p.piece_cap) {
                        for (int i = 0; i < np; ++i) {
                            p.piece[0][i] = make_int2(max(s0, a0 + i * P), min(s0 + d, a0 + (i + 1) * P));
                            if (PAR) p.piece_v[0][i] = src;
                        }
                        ctl->lv[0].ovf_pieces = (unsigned)np;
                    } else {
                        set_error(ctl, kErrQueueCap, np, p.piece_cap);
                    }
                } else {
                    p.ovf[0][0] = make_int2(s0, d);
                    if (PAR) p.ovfv[0][0] = src;
                    ctl->lv[0].ovf_pieces = 1ull << 32;
                }
                ctl->lv[0].pushed = 1;
                ctl->lv[0].pushed_edges = d;
            }
        }
    }
    if (tid == 0) {
        s_block_err = 0;
        sh.hot_off = lay.hot_off;
        for (int k = 0; k < 4; ++k) sh.phase_max[k] = 0;
#if DFQ_CLAIM_PROBES
        for (int w = 0; w < 32; ++w)
            for (int k = 0; k < 4; ++k) sh.acc[w][k] = 0ull;
        for (int k = 0; k < 4; ++k) sh.claim_max[k] = 0;
#endif
        sh.local_pack = 0ull;
        sh.cnt_cur = sh.local_grab = sh.ovf_pushed = sh.large_pushed = sh.large_pieces = sh.claimed = 0;
        sh.ovf_edges = sh.large_edges = 0;
        sh.depth = 0;
        sh.overflow = sh.large = 0ull;
    }
    unsigned& phase_bits = ws.phase_bits;  // parity of the next completion of wbar[0], wbar[1]
    bool& warp_failed = ws.failed;
    unsigned bar_target = 0;
    int cur = 0;
    int L = 0;
    Tally t{0u, 0u};
    long long explored = 0;  // degree sum of the vertices visited so far (direction switch)
    bool bottom_up = false;
    int prev_pushed = 0;

    if constexpr (CL) cluster_group_begin(gsize);
    bool ok = CL ? cluster_barrier(ctl, gsize, 0, p.timeout_ns, &ctl->lv[0], true, false)
                 : group_barrier(ctl, gsize, bar_target, p.timeout_ns, &sh.flag, &ctl->lv[0], sh.in, false);

    for (; ok; ++L) {
        const int pushed = sh.in[0];
        if (grank == 0 && tid == 0 && in_trace(DFQ_TSLOT(p, L))) {
            const int TL = DFQ_TSLOT(p, L);
            ctl->trace_ns[TL] = (long long)globaltimer();
            ctl->trace_frontier[TL] = pushed;
        }
        if (pushed == 0) break;
        LevelCtr* cin = &ctl->lv[L % 3];
        if (grank == 0 && tid == 0) {
            LevelCtr* cz = &ctl->lv[(L + 2) % 3];

            cz->ovf_grab = 0;
            cz->large_grab = 0;
            cz->pushed = 0;
            cz->pushed_edges = 0;
            cz->ovf_pieces = 0ull;
            cz->tally[0] = 0ull;
            cz->tally[1] = 0ull;
        }
        const int in = L & 1;
        // counts past a queue's capacity (recorded as an error when pushed)
        // are clamped so only entries written at this level are read
        const int n_ovf = min(sh.in[1], p.ovf_cap);
        const int total_pieces = min(sh.in[3], p.piece_cap);
        Lv lv;
        lv.next = L + 1;
        lv.out = in ^ 1;
        lv.cslot = (L + 1) % 3;
        lv.qn = cur ^ 1;
        {
            // a block keeps at most about twice its fair share of what this
            // level may discover - at least the frontier's size, and up to an
            // eighth of its edges (levels around hubs discover far more
            // vertices than they expand); the rest is shared through the
            // global queue.  Never fewer than 96 entries: on small levels of
            // high-diameter graphs what a block keeps skips the global queue's
            // reservation atomic and the next level's L2 read (4096^2 grid,
            // 16 sources: floors of 32, 96, 128 and 192 entries gave 7.70,
            // 7.30, 7.35 and 7.57 us a level)
            // (32-bit divisions: every warp works these out at every level)
            const int out = max(pushed, sh.in[4] >> 3);
            const unsigned share = ((unsigned)out + (unsigned)gsize - 1u) / (unsigned)gsize;
            lv.cap = (int)min((unsigned)p.local_cap, max(96u, 2u * min(share, 1u << 30)));
            // likewise in edges: while the frontier is small, the lists a block
            // finds (around hubs, long ones) go to the shared queue, where all
            // warps of the group can take them, instead of its own few warps
            const unsigned eshare = ((unsigned)sh.in[4] + (unsigned)gsize - 1u) / (unsigned)gsize;
            lv.ecap = (int)min((unsigned)p.local_budget, max(1024u, 2u * min(eshare, 1u << 30)));
        }
        // probe-then-claim where the level scans many edges (most of them hit
        // visited vertices); claim at once, with row bounds fetched alongside,
        // where it scans fewer edges than one 4-edge round per lane of the
        // grid; 2 = decide per level.  A graph stored hub-first (skewed
        // degrees) probes every level: its small levels are the source's hub
        // lists and the tail, whose neighbours were mostly claimed before
        // (RMAT-22 0.4771 vs 0.4870 ms, RMAT-20 -1.6 %, 262k Zipf -3 %), while
        // on even graphs small levels meet mostly unvisited neighbours and
        // claim at once
        lv.probe = p.probe_first == 2 ? ((sh.in[4] >= 128 * nwarps || p.hub_n > 0) ? 1 : 0) : p.probe_first;
        // direction (Beamer, Asanovic and Patterson, SC 2012): go bottom-up when
        // the frontier grows and its edges exceed 1/14 of the edges of
        // unvisited vertices, back to top-down once the frontier falls below
        // n/24 and shrinks (a small frontier late in the search stays
        // top-down: a bottom-up level would read every vertex's level).
        // Every block sees the same counters, so all decide alike.
        explored += sh.in[4];
        if (p.direction) {
            const long long unexplored = (long long)p.e - explored;
            if (!bottom_up && pushed > prev_pushed && 14LL * sh.in[4] > unexplored) bottom_up = true;
            else if (bottom_up && 24LL * pushed < (long long)p.n && pushed < prev_pushed) bottom_up = false;
        }
        prev_pushed = pushed;
        lv.bottom_up = bottom_up ? 1 : 0;
        if (p.profile && lane == 0) sh.level_t0[warp] = globaltimer();
        // probe levels consult the shared hot-vertex cache, refreshed here from
        // the global bitmap (everything visited before this level) and added
        // to during the level as this block meets visited vertices
        lv.hot = 0u;
        if (lv.probe && !lv.bottom_up && p.hot_words > 0) {
            lv.hot = 32u * (unsigned)p.hot_words;
            const uint4* src4 = reinterpret_cast<const uint4*>(p.bitmap);
            uint4* dst4 = reinterpret_cast<uint4*>(hot_cache());
            for (int i = tid; i < (p.hot_words >> 2); i += B) dst4[i] = __ldcg(src4 + i);
            __syncthreads();
        }
        if (grank == 0 && tid == 0 && in_trace(DFQ_TSLOT(p, L))) {
            const int TL = DFQ_TSLOT(p, L);
            ctl->trace_edges[TL] = sh.in[4];
            ctl->trace_ovf[TL] = n_ovf;
            ctl->trace_pieces[TL] = total_pieces;
            ctl->trace_probe[TL] = lv.bottom_up ? 2 : lv.probe;
        }
        if (lv.bottom_up && grank == 0 && tid == 0) {
            // E_R stays the degree sum of reached vertices: a bottom-up level
            // does not scan the frontier's lists, so count them here
            atomicAdd(&ctl->stats.edges, (unsigned long long)(unsigned)sh.in[4]);
        }

        // frontier lists averaging 16+ edges: short queues are split finely
        // over the warps; shorter lists are best gathered 32 to a warp
        const bool fine = sh.in[4] >= 16 * max(pushed, 1);
        if (lv.bottom_up) {
            // the frontier is read from the levels; this level's queues are not expanded
            bottom_up_level<PAR>(p, lv, t, gwarp, nwarps);
        } else {
            // (1) this block's own queue from the previous level; a short queue
            //     is shared by all the block's warps (a few entries per grab),
            //     since its lists may be long and a warp expands them in turn
            {
                const int nloc = sh.cnt_cur;
                const int grab = fine ? min(32, max(1, (nloc + NW - 1) / NW)) : 32;
                const int* qc = reinterpret_cast<const int*>(dfq_smem) + cur * 3 * p.local_cap;
                while (true) {
                    int j = 0;
                    if (lane == 0) j = atomicAdd(&sh.local_grab, grab);
                    j = __shfl_sync(kFull, j, 0);
                    if (j >= nloc) break;
                    const int i = j + lane;
                    const bool has = lane < grab && i < nloc;
                    warp_process<PAR>(p, lv, t, ring, wl, has, has ? qc[i] : 0, has ? qc[p.local_cap + i] : 0,
                                      (PAR && has) ? qc[2 * p.local_cap + i] : 0);
                }
            }

            // (2) large pieces: each warp pulls pieces and double-buffers their
            //     bulk copies into its own shared-memory buffers.  Schedule: when
            //     there are no more pieces than warps each piece goes to one warp;
            //     otherwise the first 3/4 go round-robin and the rest are pulled
            //     from a counter
                if (p.profile && lane == 0 && in_trace(DFQ_TSLOT(p, L)))
                    atomicMax(&sh.phase_max[0], (unsigned)(globaltimer() - sh.level_t0[warp]));
            // far fewer pieces than warps (a level around a few long lists):
            // each piece is cut into up to 8 ranges, expanded straight from
            // global memory by separate warps
            const int split = total_pieces * 8 <= nwarps ? 8 : total_pieces * 4 <= nwarps ? 4
                                                             : total_pieces * 2 <= nwarps ? 2 : 1;
            if (total_pieces > 0 && split > 1) {
                const int2* pin = p.piece[in];
                const int* pvin = p.piece_v[in];
                for (int g = gwarp; g < total_pieces * split; g += nwarps) {
                    const int k = g / split;
                    const int2 d = __ldcg(pin + k);
                    const int par0 = PAR ? __ldcg(pvin + k) : 0;
                    const int step = (d.y - d.x + split - 1) / split;
                    const int lo = d.x + (g - k * split) * step;
                    const int hi = min(d.y, lo + step);
                    if (hi > lo) warp_expand<PAR>(p, lv, t, ring, lo, hi - lo, par0);
                }
            } else if (total_pieces > 0 && !warp_failed) {
                const int2* pin = p.piece[in];
                const int* pvin = p.piece_v[in];
                const int p_static = total_pieces <= nwarps ? total_pieces : total_pieces - total_pieces / 4;
                // lane 0 runs a pipeline one piece deep in each stage: while piece
                // k is expanded, piece k+1's copy is in flight, piece k+2's range
                // is being loaded and piece k+3's index has been taken, so no
                // dependent load or atomic sits between two pieces.  The next
                // static index lives in the warp's gather scratch (unused while
                // pieces are expanded).
                // The dynamic tail is handed out in runs of g_run pieces per atomic:
                // one counter serves every warp of the grid, and on a level of
                // ~10^5 tail pieces one atomic per piece queued behind each other
                // at that counter's L2 slice.  pq[1], pq[2]: this warp's run.
                const int g_run = max(1, (total_pieces - p_static) / (4 * nwarps));
                int* pq = wl;
                auto grab = [&]() -> int {  // lane 0: next piece index (total_pieces: none)
                    const int sn = pq[0];
                    if (sn < p_static) { pq[0] = sn + nwarps; return sn; }
                    if (p_static < total_pieces) {
                        if (pq[1] < pq[2]) return pq[1]++;
                        const int b = p_static + atomicAdd(&cin->large_grab, g_run);
                        if (b >= total_pieces) return total_pieces;
                        pq[1] = b + 1;
                        pq[2] = min(b + g_run, total_pieces);
                        return b;
                    }
                    return total_pieces;
                };
                auto desc = [&](int g, int2& d, int& u) {  // lane 0: piece g's range (empty: none)
                    d = make_int2(0, 0);
                    u = 0;
                    if (g < total_pieces) {
                        d = __ldcg(pin + g);
                        if (PAR) u = __ldcg(pvin + g);
                    }
                };
                auto issue = [&](const int2& d, int b) {  // lane 0: stage piece d into buffer b
                    if (p.use_tma && d.y > d.x) {
                        const int a0 = d.x & ~3, a1 = (d.y + 3) & ~3;
                        const unsigned bytes = (unsigned)(a1 - a0) * 4u;
                        mbar_arrive_expect_tx(&wbar[b], bytes);
                        tma_load_1d(wbuf0 + b * (P + 16), p.cols + a0, bytes, &wbar[b]);
                    }
                };
                int2 dc = make_int2(0, 0), dn = dc;
                int uc = 0, un = 0, gn = total_pieces;
                if (lane == 0) {
                    pq[0] = gwarp;
                    pq[1] = pq[2] = 0;
                    desc(grab(), dc, uc);
                    issue(dc, 0);
                    desc(grab(), dn, un);
                    gn = grab();
                }
                int cb = 0;
                while (true) {
                    const int lo = __shfl_sync(kFull, dc.x, 0), hi = __shfl_sync(kFull, dc.y, 0);
                    if (hi <= lo) break;
                    const int par0 = PAR ? __shfl_sync(kFull, uc, 0) : 0;
                    if (lane == 0) {
                        issue(dn, cb ^ 1);
                        dc = dn;
                        uc = un;
                        desc(gn, dn, un);
                        gn = grab();
                    }
                    if (p.use_tma) {
                        const unsigned long long pw0 = DFQ_CLAIM_PROBES && p.profile ? globaltimer() : 0ull;
                        const bool landed = mbar_wait_bounded(&wbar[cb], (phase_bits >> cb) & 1u, p.timeout_ns);
                        const unsigned long long pw1 = DFQ_CLAIM_PROBES && p.profile ? globaltimer() : 0ull;
                        if (__any_sync(kFull, !landed)) {
                            // never expand a buffer whose copy did not land: record the
                            // error, give this warp's copies one more bounded wait, stop
                            if (lane == 0) {
                                set_error(ctl, kErrTmaTimeout, (int)blockIdx.x, lo);
                                mbar_wait_bounded(&wbar[cb], (phase_bits >> cb) & 1u, p.timeout_ns);
                                if (dc.y > dc.x)
                                    mbar_wait_bounded(&wbar[cb ^ 1], (phase_bits >> (cb ^ 1)) & 1u, p.timeout_ns);
                            }
                            warp_failed = true;
                            break;
                        }
                        phase_bits ^= 1u << cb;
                        const int* buf = wbuf0 + cb * (P + 16);
                        const int a0 = lo & ~3, off = lo - a0, tw = hi - a0;
                        if (lv.probe) {
                            probe_piece<PAR>(p, lv, t, ring, buf, off, tw, par0);
                            if (DFQ_CLAIM_PROBES && p.profile && lane == 0 && in_trace(DFQ_TSLOT(p, L))) {
                                acc_add(0, 1ull);
                                acc_add(1, pw1 - pw0);
                                acc_add(2, globaltimer_after(t.edges) - pw1);
                            }
                        } else {
                            const int par[4] = {par0, par0, par0, par0};
                            for (int base = 0; base < tw; base += 128) {
                                const int w4 = base + 4 * lane;
                                int4 x = make_int4(0, 0, 0, 0);
                                unsigned vm = 0;
                                if (w4 < tw) {
                                    x = *reinterpret_cast<const int4*>(buf + w4);
    #pragma unroll
                                    for (int j = 0; j < 4; ++j)
                                        if (w4 + j >= off && w4 + j < tw) vm |= 1u << j;
                                }
                                const int v[4] = {x.x, x.y, x.z, x.w};
                                scan4<PAR>(p, lv, t, ring, v, vm, par);
                            }
                        }
                    } else {
                        warp_expand<PAR>(p, lv, t, ring, lo, hi - lo, par0);
                    }
                    __syncwarp();
                    cb ^= 1;
                }
            }

                if (p.profile && lane == 0 && in_trace(DFQ_TSLOT(p, L)))
                    atomicMax(&sh.phase_max[1], (unsigned)(globaltimer() - sh.level_t0[warp]));
            // (3) global overflow queue in chunks, same schedule as the
            //     pieces; the next chunk index is fetched before the current one
            //     is expanded
            if (n_ovf > 0) {
                const int2* ovf_in = p.ovf[in];
                const int* ovfv_in = p.ovfv[in];
                // chunks of up to 32 entries; a short queue is cut finer so its
                // (possibly long) lists spread over the group's warps
                const int csz = fine ? min(32, max(1, (n_ovf + nwarps - 1) / nwarps)) : 32;
                const int n_chunks = (n_ovf + csz - 1) / csz;
                const int c_static = n_chunks <= nwarps ? n_chunks : n_chunks - (n_chunks >> 2);
                // The dynamic tail goes out in runs of g_run chunks per atomic, as
                // for pieces.  g_run is a power of two and run k is chunks
                // c_static + [k*g_run, (k+1)*g_run), so one register holds the
                // warp's position: the next static chunk, then the next chunk of
                // its run, and n_chunks when it must take a new run.
                const int g_run = 1 << (31 - __clz(max(1, (n_chunks - c_static) / (4 * nwarps))));
                int s_next = gwarp < c_static ? gwarp : n_chunks;
                auto next_chunk = [&]() -> int {  // lane 0 only
                    if (s_next < c_static) {
                        const int ci = s_next;
                        s_next += nwarps;
                        if (s_next >= c_static) s_next = n_chunks;
                        return ci;
                    }
                    if (c_static < n_chunks) {
                        if (s_next < n_chunks && ((s_next - c_static) & (g_run - 1))) return s_next++;
                        const int b = c_static + atomicAdd(&cin->ovf_grab, g_run);
                        if (b >= n_chunks) return n_chunks;
                        s_next = b + 1;
                        return b;
                    }
                    return n_chunks;
                };
                int nxt = 0;
                if (lane == 0) nxt = next_chunk();
                while (true) {
                    const int ci = __shfl_sync(kFull, nxt, 0);
                    if (ci >= n_chunks) break;
                    const int c0 = ci * csz;
                    if (lane == 0) nxt = next_chunk();
                    const int i = c0 + lane;
                    const bool has = lane < csz && i < n_ovf;
                    int2 x = make_int2(0, 0);
                    int u = 0;
                    if (has) {
                        x = __ldcg(ovf_in + i);
                        if (PAR) u = __ldcg(ovfv_in + i);
                    }
                    warp_process<PAR>(p, lv, t, ring, wl, has, x.x, x.y, u);
                }
            }
        }
        // claim whatever candidates this warp still holds
        if (!lv.bottom_up) {
            if (p.profile && lane == 0 && in_trace(DFQ_TSLOT(p, L)))
                atomicMax(&sh.phase_max[2], (unsigned)(globaltimer() - sh.level_t0[warp]));
        }
        ring_drain<PAR>(p, lv, t, ring, true);
        if (p.profile && lane == 0 && in_trace(DFQ_TSLOT(p, L)))
            atomicMax(&sh.phase_max[3], (unsigned)(globaltimer() - sh.level_t0[warp]));

#if DFQ_CLAIM_PROBES
        if (p.profile && lane == 0) {
            if (in_trace(DFQ_TSLOT(p, L)))
                for (int k = 0; k < 4; ++k)
                    if (sh.acc[warp][k]) atomicAdd(&ctl->trace_piece[DFQ_TSLOT(p, L)][k], sh.acc[warp][k]);
            for (int k = 0; k < 4; ++k) sh.acc[warp][k] = 0ull;
        }
#endif
        // end of level: publish how much this block pushed, keep its queue
        __syncthreads();
        unsigned long long done_ns = 0;  // when this block finished the level (thread 0, profiling)
        unsigned long long tw0 = 0, tw1 = 0;  // tally barrier words (thread 0)
        if (tid == 0) {
            if (p.profile) done_ns = globaltimer();
            const int kept = (int)(sh.local_pack >> 32);
            const int tot = kept + sh.ovf_pushed + sh.large_pushed;
            const int tot_edges = (int)(unsigned)sh.local_pack + sh.ovf_edges + sh.large_edges;
            if (gsize == 1) {
                // a one-block group: what this block pushed is the next level's
                // whole input (the barrier reads nothing back from global memory)
                sh.in[0] = tot;
                sh.in[1] = sh.ovf_pushed;
                sh.in[2] = sh.large_pushed;
                sh.in[3] = sh.large_pieces;
                sh.in[4] = tot_edges;
            } else if (CL) {
                // a cluster group: the tallies the barrier sums over the cluster
                sh.cl_out[0] = tot;
                sh.cl_out[1] = sh.ovf_pushed;
                sh.cl_out[2] = sh.large_pushed;
                sh.cl_out[3] = sh.large_pieces;
                sh.cl_out[4] = tot_edges;
                sh.cl_out[5] = (s_block_err || *(volatile int*)&ctl->status != 0) ? 1 : 0;
            } else if (p.tally_bar) {
                constexpr unsigned long long kArrive = 1ull << 54;
                const unsigned eu = ((unsigned)tot_edges + (1u << (p.tally_bar - 1)) - 1) >> (p.tally_bar - 1);
                tw0 = kArrive | ((unsigned long long)(unsigned)tot << 27) | (unsigned long long)eu;
                tw1 = kArrive | ((unsigned long long)(unsigned)sh.ovf_pushed << 27) |
                      (unsigned long long)(unsigned)sh.large_pieces;
            } else if (tot) {
                atomicAdd(&ctl->lv[lv.cslot].pushed, tot);
                atomicAdd(&ctl->lv[lv.cslot].pushed_edges, tot_edges);
            }
            if (sh.claimed) sh.depth = L + 1;
            sh.overflow += (unsigned long long)sh.ovf_pushed;
            sh.large += (unsigned long long)sh.large_pushed;
            sh.cnt_cur = kept;
            sh.local_pack = 0ull;
            sh.local_grab = 0;
            sh.ovf_pushed = sh.large_pushed = sh.large_pieces = sh.claimed = 0;
            sh.ovf_edges = sh.large_edges = 0;
        }
        cur ^= 1;
        const bool stall = p.stall_level == L + 1 && grank == gsize - 1;
        ok = CL ? cluster_barrier(ctl, gsize, (L + 1) % 3, p.timeout_ns, nullptr, false, stall)
           : (p.tally_bar && gsize > 1)
                ? tally_barrier(ctl, gsize, &ctl->lv[(L + 1) % 3], p.timeout_ns, &sh.flag, sh.in, tw0, tw1,
                                p.tally_bar - 1, stall)
                : group_barrier(ctl, gsize, bar_target, p.timeout_ns, &sh.flag, &ctl->lv[(L + 1) % 3], sh.in,
                                         true, stall);
        if (p.profile && tid == 0 && in_trace(DFQ_TSLOT(p, L))) {
            const int TL = DFQ_TSLOT(p, L);
            // recorded after the barrier: its release would otherwise wait for them
            atomicMax(&ctl->trace_done_last[TL], done_ns);
            atomicMax(&ctl->trace_done_first[TL], ~done_ns);
#if DFQ_CLAIM_PROBES
            for (int k = 0; k < 4; ++k) {
                atomicMax(&ctl->trace_claim[TL][k], sh.claim_max[k]);
                sh.claim_max[k] = 0;
            }
#endif
            for (int k = 0; k < 4; ++k) {
                atomicMax(&ctl->trace_phase[TL][k], sh.phase_max[k]);
                sh.phase_max[k] = 0;
            }
        }
    }

    // ---- results to the caller's buffers: on a relabelled graph levels (and
    // parents) back to the caller's ids; otherwise a plain copy into mapped
    // host memory.  Every block passed the final barrier after its last
    // write, so all of them are visible here (read through L2).
    if (ok && (p.levels_out || (PAR && p.parents_out))) {
        const long long gtid = (long long)grank * B + tid;
        const long long nth = (long long)gsize * B;
        for (long long v = gtid; v < p.n; v += nth) {
            const int r = p.rank ? __ldg(p.rank + v) : (int)v;
            if (p.levels_out) p.levels_out[v] = __ldcg(p.levels + r);
            if (PAR && p.parents_out) {
                const int q = __ldcg(p.parents + r);
                p.parents_out[v] = !p.order ? q : q >= 0 ? __ldg(p.order + q) : -1;
            }
        }
    }

    // ---- statistics
    unsigned long long e = t.edges, cl = t.claims;  // warp sums may pass 2^32
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e += __shfl_down_sync(kFull, e, o);
        cl += __shfl_down_sync(kFull, cl, o);
    }
    if (tid == 0) { sh.red[0] = 0; sh.red[1] = 0; }
    __syncthreads();
    if (lane == 0) {
        atomicAdd(&sh.red[0], e);
        atomicAdd(&sh.red[1], cl);
    }
    __syncthreads();
    if (tid == 0) {
        atomicAdd(&ctl->stats.edges, sh.red[0]);
        atomicAdd(&ctl->stats.claims, sh.red[1]);
        atomicAdd(&ctl->stats.overflow, sh.overflow);
        atomicAdd(&ctl->stats.large, sh.large);
        if (sh.depth) atomicMax(&ctl->stats.depth, sh.depth);
        if (grank == 0) ctl->stats.levels = L;
    }
    __syncthreads();
    // a cluster group's blocks leave together: none exits while another may
    // still add to its tallies or arrive on its mbarrier
    if constexpr (CL) cluster_sync_all();
    return ok || *(volatile int*)&ctl->status == 0;
}

// Per-warp mbarriers, initialised once per launch.
template <int B, bool PAR>
__device__ __forceinline__ void init_warp_barriers(int local_cap, int piece) {
    const SmemLayout lay = smem_layout(B, local_cap, piece, PAR);
    unsigned long long* wbar = reinterpret_cast<unsigned long long*>(dfq_smem + lay.bar_off) + (threadIdx.x >> 5) * 2;
    if ((threadIdx.x & 31) == 0) {
        mbar_init(&wbar[0], 1);
        mbar_init(&wbar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
}

// Single-source BFS: the whole grid of a cooperative launch is one group.
template <int B, bool PAR>
__global__ void __launch_bounds__(B, 1024 / B) dfq_bfs_kernel(const __grid_constant__ Params p) {
    init_warp_barriers<B, PAR>(p.local_cap, p.piece_edges);
    WarpState ws{0u, false};
    bfs_run<B, PAR>(p, (int)gridDim.x, (int)blockIdx.x, ws);
}

// Single-source BFS on one thread-block cluster (the launch is that cluster):
// the cluster's hardware co-scheduling stands in for the cooperative launch,
// and levels end on the cluster barrier in distributed shared memory.
template <int B, bool PAR>
__global__ void __launch_bounds__(B, 1024 / B) dfq_cluster_kernel(const __grid_constant__ Params p) {
    init_warp_barriers<B, PAR>(p.local_cap, p.piece_edges);
    WarpState ws{0u, false};
    bfs_run<B, PAR, true>(p, (int)gridDim.x, (int)blockIdx.x, ws);
}

}  // namespace dfqk
