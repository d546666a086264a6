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
//  * Decentralized queues: each block keeps the frontier entries it discovered
//    in its own shared-memory queue and expands them itself at the next level;
//    slots are reserved once per warp (ballot/popc/shuffle).  When the block's
//    queue is full the excess goes to a global overflow queue that all blocks
//    share with dynamic chunking.
//  * Degree bins (the reference's "our-sep" bins, bfs.cu:16-36,119-123):
//      small  [1, medium_min)      -> block-wide load-balanced gather (prefix sum
//                                     of degrees + binary search: no idle lanes)
//      medium [medium_min, large)  -> one warp per vertex, int4 column loads
//      large  [large_min, inf)     -> global large queue, split into fixed pieces
//                                     that every block pulls; each piece is staged
//                                     into shared memory by cp.async.bulk (TMA)
//  * One grid barrier per level (bounded spin, error word on timeout) instead of
//    three grid.sync() calls (bfs.cu:114,170,177); termination is decided from
//    a counter that every block reads after the barrier, so all blocks leave
//    together (the reference's racy `*done` flag, bfs.cu:115, is gone).
//
// Every queue is sized so it cannot overflow (a vertex is claimed once per
// BFS), and every index is still checked before the store; a violated bound
// sets the error word and skips the store.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dfqk {

constexpr unsigned kFull = 0xffffffffu;

// device error codes (host maps them onto DFQ_E*)
enum : int { kErrNone = 0, kErrBarrierTimeout = 1, kErrTmaTimeout = 2, kErrQueueCap = 3 };

// Counters of one level's output frontier.  Rotated over three slots: level L
// reads lv[L%3], appends to lv[(L+1)%3] and clears lv[(L+2)%3].
struct LevelCtr {
    int ovf_count;                  // entries in the global overflow queue
    int ovf_grab;                   // chunk cursor over that queue
    int large_grab;                 // piece cursor over the large queue
    int pushed;                     // frontier entries (local + overflow + large)
    unsigned long long large_pack;  // (large entries << 32) | pieces
    int pad[2];
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

// Per-launch control block; zeroed by the host before every launch.
struct Control {
    LevelCtr lv[3];
    unsigned barrier;  // grid barrier arrivals (monotone within a launch)
    int status;        // first error (kErr*)
    int err_info[2];
    DevStats stats;
};

struct Params {
    const int* __restrict__ offsets;  // n+1
    const int* __restrict__ cols;     // e, padded by >= 16 entries
    int n;
    int src;
    int* levels;
    int* parents;  // null unless parents requested
    unsigned* bitmap;
    int bitmap_words;
    int2* ovf[2];   // (start, degree) overflow entries, capacity n each
    int* ovfv[2];   // their vertex ids (parents only)
    int4* large[2]; // (start, degree, first piece, vertex), capacity large_cap
    int* piece_owner[2];  // piece -> large-queue slot, capacity piece_cap
    int large_cap;
    int piece_cap;
    Control* ctl;
    int medium_min;
    int large_min;
    int piece_edges;  // multiple of 64
    int local_cap;
    int probe_first;
    int use_tma;
    long long timeout_ns;
};

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
__device__ __forceinline__ int4 ldg4(const int* p) { return __ldg(reinterpret_cast<const int4*>(p)); }
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
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void set_error(Control* ctl, int code, int a, int b) {
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

// Grid barrier over all co-resident blocks of a cooperative launch.  One
// arrival per block on a monotone counter, then a bounded acquire-spin until
// every block of this phase has arrived.  Returns false (all threads of the
// block) if the wait timed out or another block reported an error.
__device__ __forceinline__ bool grid_barrier(Control* ctl, unsigned& target, long long timeout_ns,
                                             int* s_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        target += gridDim.x;
        int ok = 1;
        __threadfence();
        atomicAdd(&ctl->barrier, 1u);
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
        __threadfence();
        if (ok && *(volatile int*)&ctl->status != 0) ok = 0;
        *s_flag = ok;
    }
    __syncthreads();
    return *s_flag != 0;
}

// ------------------------------------------------------------ shared layout
struct SmemLayout {
    int q_off;      // local queues: 2 buffers x {start, deg, v} x cap ints
    int st_off;     // chunk staging: {start, deg, v} x B ints
    int scan_off;   // B ints
    int mlist_off;  // B ints
    int tma_off;    // 2 x (piece + 16) ints, 128-byte aligned
    int bar_off;    // 2 x u64
    int bytes;
};
__host__ __device__ inline SmemLayout smem_layout(int B, int cap, int piece) {
    SmemLayout L;
    int o = 0;
    L.q_off = o;     o += 2 * 3 * cap * 4;
    L.st_off = o;    o += 3 * B * 4;
    L.scan_off = o;  o += B * 4;
    L.mlist_off = o; o += B * 4;
    o = (o + 127) & ~127;
    L.tma_off = o;   o += 2 * (piece + 16) * 4;
    o = (o + 15) & ~15;
    L.bar_off = o;   o += 16;
    L.bytes = o;
    return L;
}

// ------------------------------------------------------------ per-level context
template <bool PAR>
struct Ctx {
    const int* __restrict__ offsets;
    const int* __restrict__ cols;
    int* levels;
    int* parents;
    unsigned* bitmap;
    // next-level outputs
    int2* ovf_out;
    int* ovfv_out;
    int4* large_out;
    int* piece_owner_out;
    LevelCtr* cout;
    int* qn_start;
    int* qn_deg;
    int* qn_v;
    int* s_cnt_next;
    int* s_ovf_pushed;
    int* s_large_pushed;
    int* s_claimed;
    Control* ctl;
    int cap;
    int n;
    int large_cap;
    int piece_cap;
    int lvl_next;
    int large_min;
    int piece_edges;
    int probe_first;
    // per-thread statistics
    unsigned long long edges;
    unsigned long long claims;
};

// Push up to four claimed vertices per lane into the block's next local queue;
// whatever does not fit goes to the global overflow queue.  Warp-collective:
// every lane of the warp must call it (with loc == 0 if it has nothing).
template <bool PAR>
__device__ __forceinline__ void push_local(Ctx<PAR>& c, unsigned loc, const int (&st)[4],
                                           const int (&dg)[4], const int (&v)[4]) {
    const int lane = threadIdx.x & 31;
    const int cnt = __popc(loc);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    const int tot = __shfl_sync(kFull, incl, 31);
    if (tot == 0) return;
    int base = 0;
    if (lane == 0) base = atomicAdd(c.s_cnt_next, tot);
    base = __shfl_sync(kFull, base, 0);
    const int ofirst = base > c.cap ? base : c.cap;
    const int ocnt = base + tot - ofirst;
    int gbase = 0;
    if (ocnt > 0) {
        if (lane == 0) {
            gbase = atomicAdd(&c.cout->ovf_count, ocnt);
            atomicAdd(c.s_ovf_pushed, ocnt);
        }
        gbase = __shfl_sync(kFull, gbase, 0);
    }
    int pos = base + incl - cnt;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (loc >> j & 1) {
            if (pos < c.cap) {
                c.qn_start[pos] = st[j];
                c.qn_deg[pos] = dg[j];
                if (PAR) c.qn_v[pos] = v[j];
            } else {
                const int gi = gbase + (pos - ofirst);
                if (gi < c.n) {
                    c.ovf_out[gi] = make_int2(st[j], dg[j]);
                    if (PAR) c.ovfv_out[gi] = v[j];
                } else {
                    set_error(c.ctl, kErrQueueCap, gi, c.n);
                }
            }
            ++pos;
        }
    }
}

template <bool PAR>
__device__ __forceinline__ void push_large(Ctx<PAR>& c, int st, int dg, int v) {
    const unsigned np = (unsigned)((dg + c.piece_edges - 1) / c.piece_edges);
    unsigned long long old = atomicAdd(&c.cout->large_pack, (1ull << 32) | np);
    const int slot = (int)(old >> 32);
    const unsigned poff = (unsigned)old;
    atomicAdd(c.s_large_pushed, 1);
    if (slot >= c.large_cap || poff + np > (unsigned)c.piece_cap) {
        set_error(c.ctl, kErrQueueCap, slot, (int)poff);
        return;
    }
    c.large_out[slot] = make_int4(st, dg, (int)poff, v);
    for (unsigned i = 0; i < np; ++i) c.piece_owner_out[poff + i] = slot;
}

// Scan up to four neighbours per lane: probe, claim, record, push.
// Warp-collective (calls push_local).
template <bool PAR>
__device__ __forceinline__ void visit4(Ctx<PAR>& c, const int (&v)[4], unsigned vmask,
                                       const int (&par)[4]) {
    unsigned claim = 0;
    if (vmask) {
        unsigned w[4] = {0u, 0u, 0u, 0u};
        if (c.probe_first) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (vmask >> j & 1) w[j] = c.bitmap[v[j] >> 5];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const unsigned bit = 1u << (v[j] & 31);
            if ((vmask >> j & 1) && !(w[j] & bit)) {
                const unsigned old = atomicOr(&c.bitmap[v[j] >> 5], bit);
                if (!(old & bit)) claim |= 1u << j;
            }
        }
        c.edges += __popc(vmask);
    }
    int st[4], dg[4];
    unsigned loc = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        st[j] = 0;
        dg[j] = 0;
        if (claim >> j & 1) {
            c.levels[v[j]] = c.lvl_next;
            if (PAR) c.parents[v[j]] = par[j];
            st[j] = __ldg(c.offsets + v[j]);
            dg[j] = __ldg(c.offsets + v[j] + 1) - st[j];
        }
    }
    if (claim) {
        c.claims += __popc(claim);
        *c.s_claimed = 1;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (!(claim >> j & 1) || dg[j] == 0) continue;
            if (dg[j] >= c.large_min) push_large(c, st[j], dg[j], v[j]);
            else loc |= 1u << j;
        }
    }
    push_local(c, loc, st, dg, v);
}

// One warp expands one medium vertex: int4 column loads from the 16-byte
// aligned floor of its list; lanes mask what lies outside [e0, e1).
template <bool PAR>
__device__ __forceinline__ void warp_expand(Ctx<PAR>& c, int s, int d, int u) {
    const int lane = threadIdx.x & 31;
    const int e0 = s, e1 = s + d, a0 = e0 & ~3;
    const int par[4] = {u, u, u, u};
    for (int base = a0; base < e1; base += 128) {
        const int k4 = base + lane * 4;
        int4 x = make_int4(0, 0, 0, 0);
        unsigned vm = 0;
        if (k4 < e1) {
            x = ldg4(c.cols + k4);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (k4 + j >= e0 && k4 + j < e1) vm |= 1u << j;
        }
        const int v[4] = {x.x, x.y, x.z, x.w};
        visit4(c, v, vm, par);
    }
}

// Expand m (<= B) frontier entries held in shared memory: medium entries one
// warp each, small entries by a block-wide load-balanced gather.
// Block-collective; ends with __syncthreads.
template <int B, bool PAR>
__device__ __forceinline__ void process_entries(Ctx<PAR>& c, const int* es, const int* ed,
                                                const int* ev, int m, int* scan, int* mlist,
                                                int2* s_warp, int medium_min) {
    constexpr int NW = B / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int d = tid < m ? ed[tid] : 0;
    const int med = d >= medium_min ? 1 : 0;
    const int ds = med ? 0 : d;
    // block exclusive scan of (small degree, medium flag)
    int x = ds, y = med;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int tx = __shfl_up_sync(kFull, x, o), ty = __shfl_up_sync(kFull, y, o);
        if (lane >= o) { x += tx; y += ty; }
    }
    if (lane == 31) s_warp[warp] = make_int2(x, y);
    __syncthreads();
    if (warp == 0) {
        int2 w = lane < NW ? s_warp[lane] : make_int2(0, 0);
        int wx = w.x, wy = w.y;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int tx = __shfl_up_sync(kFull, wx, o), ty = __shfl_up_sync(kFull, wy, o);
            if (lane >= o) { wx += tx; wy += ty; }
        }
        if (lane < NW) s_warp[lane] = make_int2(wx, wy);
    }
    __syncthreads();
    const int2 pre = warp > 0 ? s_warp[warp - 1] : make_int2(0, 0);
    const int2 tot = s_warp[NW - 1];
    scan[tid] = pre.x + x - ds;
    if (med) mlist[pre.y + y - 1] = tid;
    __syncthreads();
    // medium: one warp per vertex
    for (int j = warp; j < tot.y; j += NW) {
        const int i = mlist[j];
        warp_expand(c, es[i], ed[i], PAR ? ev[i] : 0);
    }
    // small: 4 edges per thread per round, owner by binary search over scan
    const int T = tot.x;
    for (int base = 0; base < T; base += 4 * B) {
        int v[4], par[4];
        unsigned vm = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k = base + j * B + tid;
            v[j] = 0;
            par[j] = 0;
            if (k < T) {
                int lo = 0, hi = B;  // first index with scan > k
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (scan[mid] <= k) lo = mid + 1;
                    else hi = mid;
                }
                const int own = lo - 1;
                v[j] = __ldg(c.cols + es[own] + (k - scan[own]));
                if (PAR) par[j] = ev[own];
                vm |= 1u << j;
            }
        }
        visit4(c, v, vm, par);
    }
    __syncthreads();
}

template <int B, bool PAR>
__global__ void __launch_bounds__(B) dfq_bfs_kernel(Params p) {
    constexpr int NW = B / 32;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_cnt_next, s_cnt_cur, s_ovf_pushed, s_large_pushed, s_claimed, s_flag;
    __shared__ int s_bc;
    __shared__ int s_pc[2][4];  // staged piece: {e0, count, offset in buffer, parent}
    __shared__ int2 s_warp[NW];
    __shared__ unsigned long long s_red[4];

    const int tid = threadIdx.x;
    const SmemLayout lay = smem_layout(B, p.local_cap, p.piece_edges);
    const int cap = p.local_cap;
    int* qbase = reinterpret_cast<int*>(smem + lay.q_off);
    int* st_start = reinterpret_cast<int*>(smem + lay.st_off);
    int* st_deg = st_start + B;
    int* st_v = st_deg + B;
    int* scan = reinterpret_cast<int*>(smem + lay.scan_off);
    int* mlist = reinterpret_cast<int*>(smem + lay.mlist_off);
    int* tma_buf[2] = {reinterpret_cast<int*>(smem + lay.tma_off),
                       reinterpret_cast<int*>(smem + lay.tma_off) + p.piece_edges + 16};
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + lay.bar_off);
    Control* ctl = p.ctl;

    // ---- init: levels, parents, bitmap (source pre-set so no ordering is needed)
    const int src = p.src;
    {
        const long long gtid = (long long)blockIdx.x * B + tid;
        const long long nth = (long long)gridDim.x * B;
        for (long long i = gtid; i < p.n; i += nth) {
            p.levels[i] = (i == src) ? 0 : -1;
            if (PAR) p.parents[i] = (i == src) ? src : -1;
        }
        for (long long w = gtid; w < p.bitmap_words; w += nth)
            p.bitmap[w] = (w == (src >> 5)) ? (1u << (src & 31)) : 0u;
        if (gtid == 0) {
            const int s0 = p.offsets[src], d = p.offsets[src + 1] - s0;
            if (d > 0) {
                if (d >= p.large_min) {
                    const int np = (d + p.piece_edges - 1) / p.piece_edges;
                    p.large[0][0] = make_int4(s0, d, 0, src);
                    for (int i = 0; i < np; ++i) p.piece_owner[0][i] = 0;
                    ctl->lv[0].large_pack = (1ull << 32) | (unsigned)np;
                } else {
                    p.ovf[0][0] = make_int2(s0, d);
                    if (PAR) p.ovfv[0][0] = src;
                    ctl->lv[0].ovf_count = 1;
                }
                ctl->lv[0].pushed = 1;
            }
        }
    }
    if (tid == 0) {
        s_cnt_next = s_cnt_cur = s_ovf_pushed = s_large_pushed = s_claimed = 0;
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
    }
    unsigned phase_bits = 0;  // parity of the next completion of bars[0], bars[1]
    unsigned bar_target = 0;
    unsigned long long my_overflow = 0, my_large = 0;
    int cur = 0;
    int L = 0;

    Ctx<PAR> c;
    c.offsets = p.offsets;
    c.cols = p.cols;
    c.levels = p.levels;
    c.parents = p.parents;
    c.bitmap = p.bitmap;
    c.s_cnt_next = &s_cnt_next;
    c.s_ovf_pushed = &s_ovf_pushed;
    c.s_large_pushed = &s_large_pushed;
    c.s_claimed = &s_claimed;
    c.ctl = ctl;
    c.cap = cap;
    c.n = p.n;
    c.large_cap = p.large_cap;
    c.piece_cap = p.piece_cap;
    c.large_min = p.large_min;
    c.piece_edges = p.piece_edges;
    c.probe_first = p.probe_first;
    c.edges = 0;
    c.claims = 0;

    bool ok = grid_barrier(ctl, bar_target, p.timeout_ns, &s_flag);

    for (; ok; ++L) {
        LevelCtr* cin = &ctl->lv[L % 3];
        const int pushed = __ldcg(&cin->pushed);
        if (pushed == 0) break;
        if (blockIdx.x == 0 && tid == 0) {
            LevelCtr* cz = &ctl->lv[(L + 2) % 3];
            cz->ovf_count = 0;
            cz->ovf_grab = 0;
            cz->large_grab = 0;
            cz->pushed = 0;
            cz->large_pack = 0ull;
        }
        const int in = L & 1, out = in ^ 1;
        const int n_ovf = __ldcg(&cin->ovf_count);
        const unsigned long long lp = __ldcg(&cin->large_pack);
        const int total_pieces = (int)(unsigned)(lp & 0xffffffffull);

        c.ovf_out = p.ovf[out];
        c.ovfv_out = p.ovfv[out];
        c.large_out = p.large[out];
        c.piece_owner_out = p.piece_owner[out];
        c.cout = &ctl->lv[(L + 1) % 3];
        c.qn_start = qbase + (cur ^ 1) * 3 * cap;
        c.qn_deg = c.qn_start + cap;
        c.qn_v = c.qn_deg + cap;
        c.lvl_next = L + 1;
        const int* qc_start = qbase + cur * 3 * cap;
        const int* qc_deg = qc_start + cap;
        const int* qc_v = qc_deg + cap;

        // (1) this block's own queue from the previous level
        const int nloc = s_cnt_cur;
        for (int b0 = 0; b0 < nloc; b0 += B) {
            const int m = nloc - b0 < B ? nloc - b0 : B;
            process_entries<B, PAR>(c, qc_start + b0, qc_deg + b0, qc_v + b0, m, scan, mlist, s_warp,
                                    p.medium_min);
        }

        // (2) large pieces, double-buffered: the next piece's copy is in flight
        //     while the current one is expanded
        if (total_pieces > 0) {
            const int4* large_in = p.large[in];
            const int* owner_in = p.piece_owner[in];
            const int P = p.piece_edges;
            auto fetch = [&](int b) {  // thread 0 only
                const int g = atomicAdd(&cin->large_grab, 1);
                if (g >= total_pieces) { s_pc[b][1] = -1; return; }
                const int slot = __ldcg(owner_in + g);
                const int4 ent = __ldcg(large_in + slot);
                const int e0 = ent.x + (g - ent.z) * P;
                const int e1 = min(e0 + P, ent.x + ent.y);
                const int a0 = e0 & ~3, a1 = (e1 + 3) & ~3;
                s_pc[b][0] = e0;
                s_pc[b][1] = e1 - e0;
                s_pc[b][2] = e0 - a0;
                s_pc[b][3] = ent.w;
                if (p.use_tma) {
                    const unsigned bytes = (unsigned)(a1 - a0) * 4u;
                    mbar_arrive_expect_tx(&bars[b], bytes);
                    tma_load_1d(tma_buf[b], p.cols + a0, bytes, &bars[b]);
                }
            };
            if (tid == 0) fetch(0);
            __syncthreads();
            int cb = 0;
            while (true) {
                const int cnt = s_pc[cb][1];
                if (cnt < 0) break;
                const int e0 = s_pc[cb][0], off = s_pc[cb][2], par0 = s_pc[cb][3];
                if (tid == 0) fetch(cb ^ 1);
                const int par[4] = {par0, par0, par0, par0};
                if (p.use_tma) {
                    const bool landed = mbar_wait_bounded(&bars[cb], (phase_bits >> cb) & 1u, p.timeout_ns);
                    if (__syncthreads_or(!landed)) {
                        // never expand a buffer whose copy did not land: record the
                        // error, give both copies of this block one more bounded
                        // wait, and leave the level (the barrier then stops the grid)
                        if (tid == 0) {
                            set_error(ctl, kErrTmaTimeout, (int)blockIdx.x, e0);
                            mbar_wait_bounded(&bars[cb], (phase_bits >> cb) & 1u, p.timeout_ns);
                            if (s_pc[cb ^ 1][1] >= 0)
                                mbar_wait_bounded(&bars[cb ^ 1], (phase_bits >> (cb ^ 1)) & 1u, p.timeout_ns);
                        }
                        __syncthreads();
                        break;
                    }
                    phase_bits ^= 1u << cb;
                    const int* buf = tma_buf[cb];
                    const int tw = off + cnt;
                    for (int base = 0; base < tw; base += 4 * B) {
                        const int w4 = base + 4 * tid;
                        int4 x = make_int4(0, 0, 0, 0);
                        unsigned vm = 0;
                        if (w4 < tw) {
                            x = *reinterpret_cast<const int4*>(buf + w4);
#pragma unroll
                            for (int j = 0; j < 4; ++j)
                                if (w4 + j >= off && w4 + j < tw) vm |= 1u << j;
                        }
                        const int v[4] = {x.x, x.y, x.z, x.w};
                        visit4(c, v, vm, par);
                    }
                } else {
                    const int a0 = e0 - off, e1 = e0 + cnt;
                    for (int base = a0; base < e1; base += 4 * B) {
                        const int k4 = base + 4 * tid;
                        int4 x = make_int4(0, 0, 0, 0);
                        unsigned vm = 0;
                        if (k4 < e1) {
                            x = ldg4(p.cols + k4);
#pragma unroll
                            for (int j = 0; j < 4; ++j)
                                if (k4 + j >= e0 && k4 + j < e1) vm |= 1u << j;
                        }
                        const int v[4] = {x.x, x.y, x.z, x.w};
                        visit4(c, v, vm, par);
                    }
                }
                __syncthreads();
                cb ^= 1;
            }
            __syncthreads();
        }

        // (3) global overflow queue, dynamic chunks
        if (n_ovf > 0) {
            const int G4 = 4 * (int)gridDim.x;
            int CH = (n_ovf + G4 - 1) / G4;
            CH = CH < 32 ? 32 : (CH > B ? B : CH);
            const int2* ovf_in = p.ovf[in];
            const int* ovfv_in = p.ovfv[in];
            while (true) {
                if (tid == 0) s_bc = atomicAdd(&cin->ovf_grab, CH);
                __syncthreads();
                const int c0 = s_bc;
                if (c0 >= n_ovf) break;
                const int m = n_ovf - c0 < CH ? n_ovf - c0 : CH;
                if (tid < m) {
                    const int2 x = __ldcg(ovf_in + c0 + tid);
                    st_start[tid] = x.x;
                    st_deg[tid] = x.y;
                    if (PAR) st_v[tid] = __ldcg(ovfv_in + c0 + tid);
                }
                __syncthreads();
                process_entries<B, PAR>(c, st_start, st_deg, st_v, m, scan, mlist, s_warp, p.medium_min);
            }
            __syncthreads();
        }

        // end of level: publish how much this block pushed, keep its queue
        __syncthreads();
        if (tid == 0) {
            const int kept = s_cnt_next < cap ? s_cnt_next : cap;
            const int tot = kept + s_ovf_pushed + s_large_pushed;
            if (tot) atomicAdd(&c.cout->pushed, tot);
            if (s_claimed) atomicMax(&ctl->stats.depth, L + 1);
            my_overflow += (unsigned long long)s_ovf_pushed;
            my_large += (unsigned long long)s_large_pushed;
            s_cnt_cur = kept;
            s_cnt_next = 0;
            s_ovf_pushed = s_large_pushed = s_claimed = 0;
        }
        cur ^= 1;
        ok = grid_barrier(ctl, bar_target, p.timeout_ns, &s_flag);
    }

    // ---- statistics
    unsigned long long e = c.edges, cl = c.claims;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e += __shfl_down_sync(kFull, e, o);
        cl += __shfl_down_sync(kFull, cl, o);
    }
    if (tid == 0) { s_red[0] = 0; s_red[1] = 0; }
    __syncthreads();
    if ((tid & 31) == 0) {
        atomicAdd(&s_red[0], e);
        atomicAdd(&s_red[1], cl);
    }
    __syncthreads();
    if (tid == 0) {
        atomicAdd(&ctl->stats.edges, s_red[0]);
        atomicAdd(&ctl->stats.claims, s_red[1]);
        atomicAdd(&ctl->stats.overflow, my_overflow);
        atomicAdd(&ctl->stats.large, my_large);
        if (blockIdx.x == 0) ctl->stats.levels = L;
    }
}

}  // namespace dfqk
