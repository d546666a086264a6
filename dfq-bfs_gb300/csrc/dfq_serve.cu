// Serving: continuous batching of single-source BFS requests over a resident
// pool.  No reference counterpart (a reference program serves one source per
// launch, design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu:202-309).
//
// Device side: one persistent cooperative serving kernel.
//   * Requests are published by the host in two rings in mapped pinned memory
//     (narrow / wide), each slot written before the ring's published count.
//   * Block 0 is the scheduler.  It mirrors the host's narrow count into
//     device memory, starts a "gang" run for each published wide request -
//     every block joins it between its own requests and the whole grid runs
//     the BFS (bfs_run with the grid as group) - and decides when the kernel
//     leaves: all published work claimed and either the host asked to stop or
//     nothing arrived for idle_ns.
//   * Every other block claims narrow requests with a CAS on a device cursor
//     and runs each alone (bfs_run with one block as group, bounded per-block
//     queues), then writes a completion record to mapped memory behind a
//     system-scope fence.
//   All waits are bounded: the scheduler by idle_ns, the workers by the exit
//   flag plus a hard limit, the gang by the grid barrier's timeout.
// Host side: FIFO admission of queued requests by HBM-arena budget and free
// ring slots, relaunch after an idle exit, completion polling, and a rerun on
// the whole grid for a narrow request that outgrew its block's queues.
#include "dfq_pool.cuh"

#include <atomic>
#include <cstddef>
#include <chrono>
#include <deque>
#include <map>
#include <thread>
#include <unordered_map>

using namespace dfq;
using namespace dfqk;

namespace dfqk {

struct ServeReq {  // host -> device, mapped pinned memory
    int graph;
    int source;
    int* levels;
    int* parents;
    unsigned long long seq;  // ring index + 1, written after the fields
};

struct ServeDone {  // device -> host, mapped pinned memory
    long long t_start;
    long long t_end;
    long long reached;
    long long edges;
    int status;
    int depth;
    unsigned long long seq;  // ring index + 1, written after the fields
};

struct ServeHost {  // counters written by the host, mapped
    unsigned long long avail[2];  // published narrow / wide requests
    int stop;
    int pad;
};

struct ServeDev {  // device memory
    // persist across launches
    unsigned long long narrow_next;   // next narrow request to claim
    unsigned long long narrow_avail;  // block 0's copy of the host's narrow count
    unsigned long long gang_done;     // wide requests completed
    // reset by the host before each launch (from `gang` on)
    unsigned long long gang_word;     // (gang index << 32) | kGangOpen while joinable | members
    int exit;                         // 1: every block leaves
    int error;                        // a block gave up waiting (1 scheduler gone, 2 slot, 3 gang)
    int narrow_active;                // blocks running a narrow request now
    int gang_left;                    // members that finished the current gang run
    unsigned long long gang_size;     // ((gang index + 1) << 32) | members, once the window closed
                                      // (+1: the reset value 0 must not name gang 0)
};
constexpr unsigned long long kGangOpen = 0x80000000ull;
constexpr unsigned long long kGangCount = 0x7fffffffull;

struct ServeParams {
    const PoolGraph* graphs;
    const ServeReq* ring[2];
    ServeDone* done[2];
    const ServeHost* host;
    ServeDev* dev;
    Control* ctls[2];  // one per ring slot
    int cap;           // ring slots (power of two)
    Workspace wide_ws;
    int wide_ovf_cap;
    unsigned char* block_ws;
    size_t block_ws_stride;
    WsLayout block_lay;
    int block_ovf_cap;
    int* block_state;  // per block: (loop iterations << 4) | last action, for diagnosis
    int narrow_limit;  // at most this many blocks run narrow requests at once
    int gang_min;      // a gang forms once this many blocks joined ...
    long long join_ns; // ... or its window has been open this long
    int medium_min, large_min, piece_edges, local_cap, local_budget, probe_first, use_tma;
    long long timeout_ns;
    int hot_words;     // hot-vertex cache words the launch reserves (0: none)
    long long idle_ns;
};

__device__ __forceinline__ unsigned long long ld_acquire_sys_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_acquire_sys_s32(const int* p) {
    int v;
    asm volatile("ld.acquire.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void serve_params(Params& sp, const ServeParams& s, const ServeReq& q, const Workspace& ws,
                                             int ovf_cap, Control* ctl) {
    const PoolGraph& g = s.graphs[q.graph];
    sp = Params{};  // shared memory starts undefined: every field not set below is zero / null
    sp.offsets = g.offsets;
    sp.cols = g.cols;
    sp.n = g.n;
    sp.src = q.source;
    sp.levels = q.levels;
    sp.parents = q.parents;
    sp.bitmap = ws.bitmap;
    sp.bitmap_words = (g.n + 31) / 32;
    for (int i = 0; i < 2; ++i) {
        sp.ovf[i] = ws.ovf[i];
        sp.ovfv[i] = ws.ovfv[i];
        sp.piece[i] = ws.piece[i];
        sp.piece_v[i] = ws.piece_v[i];
    }
    sp.ovf_cap = min(ovf_cap, g.n);
    sp.piece_cap = ws.piece_cap;
    sp.ctl = ctl;
    sp.medium_min = s.medium_min;
    sp.large_min = s.large_min;
    sp.piece_edges = s.piece_edges;
    sp.local_cap = s.local_cap;
    sp.local_budget = s.local_budget;
    sp.probe_first = s.probe_first;
    sp.use_tma = s.use_tma;
    sp.timeout_ns = s.timeout_ns;
    sp.hot_words = hot_words_of(s.hot_words, g.n);
    sp.tally_bar = tally_bar_for(g.n, g.e);
    remap_params(sp, g, ws);  // renumbered graphs are wide: only the gang's workspace has room
}

// Copy one ring slot (seq checked: the host writes the fields before the count).
__device__ __forceinline__ bool read_req(const ServeReq* slot, unsigned long long k, ServeReq& out,
                                         long long timeout_ns) {
    const unsigned long long t0 = globaltimer();
    while (ld_acquire_sys_u64(&slot->seq) != k + 1)
        if ((long long)(globaltimer() - t0) > timeout_ns) return false;
    const volatile ServeReq* v = slot;
    out.graph = v->graph;
    out.source = v->source;
    out.levels = v->levels;
    out.parents = v->parents;
    return true;
}

__device__ __forceinline__ void publish_done(ServeDone* d, unsigned long long k, const Control* ctl, long long t0,
                                             long long t1) {
    volatile ServeDone* v = d;
    v->t_start = t0;
    v->t_end = t1;
    v->reached = (long long)ctl->stats.claims + 1;
    v->edges = (long long)ctl->stats.edges;
    v->status = *(volatile const int*)&ctl->status;
    v->depth = ctl->stats.depth;
    __threadfence_system();
    v->seq = k + 1;
}

__device__ __forceinline__ void zero_ctl(Control* c, int tid, int nth) {
    int* w = reinterpret_cast<int*>(c);
    for (int i = tid; i < (int)(sizeof(Control) / 4); i += nth) w[i] = 0;
}

enum : int { kActWait = 0, kActNarrow = 1, kActGang = 2, kActExit = 3, kActRetry = 4 };

// Scheduler (block 0, thread 0): form the gang for wide request k.  Opens the
// join window with itself as member 0, waits until gang_min members joined or
// join_ns passed, closes the window atomically and publishes the size.
// Returns the number of members.
__device__ __forceinline__ int form_gang(const ServeParams& s, unsigned long long k) {
    ServeDev* dev = s.dev;
    *(volatile int*)&dev->gang_left = 0;
    __threadfence();
    *(volatile unsigned long long*)&dev->gang_word = (k << 32) | kGangOpen | 1ull;
    __threadfence();
    // close when every block joined, or when at least gang_min joined and no
    // one else arrived for 3 us, or when the window has been open join_ns
    const unsigned long long t0 = globaltimer();
    const unsigned long long want = (unsigned long long)min(s.gang_min, (int)gridDim.x);
    unsigned long long last_n = 1, t_last = t0;
    while (true) {
        const unsigned long long n = *(volatile unsigned long long*)&dev->gang_word & kGangCount;
        const unsigned long long now = globaltimer();
        if (n != last_n) { last_n = n; t_last = now; }
        if (n >= gridDim.x) break;
        if (n >= want && (long long)(now - t_last) > 3000) break;
        if ((long long)(now - t0) > s.join_ns) break;
    }
    const unsigned long long old = atomicAnd(&dev->gang_word, ~kGangOpen);
    const int m = (int)(old & kGangCount);
    __threadfence();
    *(volatile unsigned long long*)&dev->gang_size = ((k + 1) << 32) | (unsigned long long)m;
    __threadfence();
    return m;
}

// This block's narrow-request workspace.
__device__ __forceinline__ Workspace block_workspace(const ServeParams& s) {
    Workspace bw;
    unsigned char* base = s.block_ws + s.block_ws_stride * blockIdx.x;
    bw.bitmap = (unsigned*)(base + s.block_lay.bitmap);
    for (int i = 0; i < 2; ++i) {
        bw.ovf[i] = (int2*)(base + s.block_lay.ovf[i]);
        bw.ovfv[i] = (int*)(base + s.block_lay.ovfv[i]);
        bw.piece[i] = (int2*)(base + s.block_lay.piece[i]);
        bw.piece_v[i] = (int*)(base + s.block_lay.piece_v[i]);
    }
    bw.piece_cap = s.block_lay.piece_cap;
    bw.levels_int = nullptr;  // one-block workspaces take no renumbered graph
    bw.parents_int = nullptr;
    bw.hub_claim = nullptr;
    return bw;
}

template <int B, bool PAR>
__global__ void __launch_bounds__(B, 1024 / B) dfq_serve_kernel(const __grid_constant__ ServeParams s) {
    __shared__ Params sp;
    __shared__ ServeReq s_req;
    __shared__ int s_act, s_rank, s_size;
    __shared__ long long s_k;
    __shared__ unsigned long long s_next_gang;  // the first gang this block may still join
    init_warp_barriers<B, PAR>(s.local_cap, s.piece_edges);
    WarpState ws{0u, false};
    const int tid = threadIdx.x;
    ServeDev* dev = s.dev;
    const unsigned mask = (unsigned)s.cap - 1;

    if (tid == 0) s_next_gang = *(volatile unsigned long long*)&dev->gang_done;
    __syncthreads();

    unsigned long long last_a0 = ~0ull, last_a1 = ~0ull, last_nn = ~0ull;
    unsigned long long idle_since = globaltimer();
    while (true) {
        if (tid == 0) {
            int act = kActWait;
            if (blockIdx.x == 0) {
                // scheduler
                const int stop = ld_acquire_sys_s32(&s.host->stop);
                const unsigned long long a1 = ld_acquire_sys_u64(&s.host->avail[1]);
                const unsigned long long a0 = ld_acquire_sys_u64(&s.host->avail[0]);
                *(volatile unsigned long long*)&dev->narrow_avail = a0;
                const unsigned long long nn = *(volatile unsigned long long*)&dev->narrow_next;
                const unsigned long long gd = *(volatile unsigned long long*)&dev->gang_done;
                const unsigned long long now = globaltimer();
                if (a0 != last_a0 || a1 != last_a1 || nn != last_nn) idle_since = now;
                last_a0 = a0; last_a1 = a1; last_nn = nn;
                if (a1 > gd) {
                    zero_ctl(&s.ctls[1][gd & mask], 0, 1);
                    __threadfence();
                    s_size = form_gang(s, gd);
                    s_rank = 0;
                    s_k = (long long)gd;
                    act = kActGang;
                } else if (nn >= a0 && (stop || (long long)(now - idle_since) > s.idle_ns)) {
                    act = kActExit;
                    *(volatile int*)&dev->exit = 1;
                    __threadfence();
                }
            } else {
                // worker: join an open gang, else claim a narrow request (while
                // fewer than narrow_limit blocks hold one), else wait
                // one word names the gang and its window, so a join is tied to
                // the gang the worker saw
                const unsigned long long w = *(volatile unsigned long long*)&dev->gang_word;
                const unsigned long long g = w >> 32;
                bool handled = false;
                if ((w & kGangOpen) && g >= s_next_gang) {
                    handled = true;
                    act = kActRetry;
                    if (atomicCAS(&dev->gang_word, w, w + 1) == w) {
                        // joined as member w & count; wait (bounded) for the size
                        const unsigned long long t0 = globaltimer();
                        unsigned long long sz;
                        while (((sz = *(volatile unsigned long long*)&dev->gang_size) >> 32) != g + 1)
                            if ((long long)(globaltimer() - t0) > s.timeout_ns) break;
                        if ((sz >> 32) == g + 1 && (int)(unsigned)sz >= 1) {
                            s_rank = (int)(w & kGangCount);
                            s_size = (int)(unsigned)sz;
                            s_k = (long long)g;
                            act = kActGang;
                        } else {
                            atomicExch(&dev->error, 3);
                            act = kActExit;
                        }
                    }
                    idle_since = globaltimer();
                }
                if (!handled) {
                    const unsigned long long nn = *(volatile unsigned long long*)&dev->narrow_next;
                    const unsigned long long av = *(volatile unsigned long long*)&dev->narrow_avail;
                    if (nn < av && *(volatile int*)&dev->narrow_active < s.narrow_limit) {
                        act = kActRetry;
                        if (atomicAdd(&dev->narrow_active, 1) < s.narrow_limit) {
                            if (atomicCAS(&dev->narrow_next, nn, nn + 1) == nn) {
                                act = kActNarrow;
                                s_k = (long long)nn;
                            } else {
                                atomicSub(&dev->narrow_active, 1);
                            }
                        } else {
                            atomicSub(&dev->narrow_active, 1);
                        }
                        idle_since = globaltimer();
                    } else if (*(volatile int*)&dev->exit) {
                        act = kActExit;
                    } else if ((long long)(globaltimer() - idle_since) > s.idle_ns + s.timeout_ns) {
                        // the scheduler stopped answering: leave rather than wait on
                        atomicExch(&dev->error, 1);
                        act = kActExit;
                    }
                }
            }
            if (act == kActGang || act == kActNarrow) {
                const int r = act == kActGang ? 1 : 0;
                if (!read_req(&s.ring[r][(unsigned long long)s_k & mask], (unsigned long long)s_k, s_req,
                              s.timeout_ns)) {
                    atomicExch(&dev->error, 2);
                    if (act == kActNarrow) atomicSub(&dev->narrow_active, 1);
                    act = kActExit;
                }
            }
            s_act = act;
            const int prev = s.block_state[blockIdx.x];
            *(volatile int*)&s.block_state[blockIdx.x] = (((prev >> 4) + 1) << 4) | act;
        }
        __syncthreads();
        const int act = s_act;
        if (act == kActExit) break;
        if (act == kActWait || act == kActRetry) {
            if (tid == 0 && act == kActWait) __nanosleep(blockIdx.x == 0 ? 500 : 2000);
            __syncthreads();
            continue;
        }
        const unsigned long long k = (unsigned long long)s_k;
        const unsigned slot = (unsigned)k & mask;
        // one call site of bfs_run for both shapes keeps one inlined copy
        const bool gang = act == kActGang;
        if (!gang) zero_ctl(&s.ctls[0][slot], tid, B);
        if (tid == 0) {
            if (gang) serve_params(sp, s, s_req, s.wide_ws, s.wide_ovf_cap, &s.ctls[1][slot]);
            else serve_params(sp, s, s_req, block_workspace(s), s.block_ovf_cap, &s.ctls[0][slot]);
        }
        __syncthreads();
        const long long t0 = (long long)globaltimer();
        bfs_run<B, PAR>(sp, gang ? s_size : 1, gang ? s_rank : 0, ws);
        if (tid == 0) {
            if (gang) {
                s_next_gang = k + 1;
                // a member's statistics are in once it counts itself out
                __threadfence();
                atomicAdd(&dev->gang_left, 1);
                if (blockIdx.x == 0) {
                    const unsigned long long tw = globaltimer();
                    while (*(volatile int*)&dev->gang_left < s_size)
                        if ((long long)(globaltimer() - tw) > s.timeout_ns) { atomicExch(&dev->error, 3); break; }
                    __threadfence();
                    publish_done(&s.done[1][slot], k, &s.ctls[1][slot], t0, (long long)globaltimer());
                    *(volatile unsigned long long*)&dev->gang_done = k + 1;
                    __threadfence();
                }
            } else {
                publish_done(&s.done[0][slot], k, &s.ctls[0][slot], t0, (long long)globaltimer());
                atomicSub(&dev->narrow_active, 1);
            }
        }
        __syncthreads();
    }
}

}  // namespace dfqk

// ------------------------------------------------------------------ host side
struct dfq_server {
    dfq_pool* pool = nullptr;
    dfq_server_opts opts{};
    cudaStream_t stream = nullptr;
    cudaEvent_t kernel_done = nullptr;
    bool running = false;
    // mapped rings
    ServeReq* h_ring[2] = {nullptr, nullptr};
    ServeReq* d_ring[2] = {nullptr, nullptr};
    ServeDone* h_done[2] = {nullptr, nullptr};
    ServeDone* d_done[2] = {nullptr, nullptr};
    ServeHost* h_host = nullptr;
    ServeHost* d_host = nullptr;
    ServeDev* d_dev = nullptr;
    int* d_block_state = nullptr;
    Control* d_ctls[2] = {nullptr, nullptr};
    // per-block workspaces for narrow requests
    unsigned char* block_mem = nullptr;
    WsLayout block_lay{};
    size_t block_stride = 0;
    int grid = 0;
    int smem = 0;
    int hot_words = 0;  // hot-vertex cache words per block (the largest graph's)
    const void* fn = nullptr;
    // HBM arena for per-request outputs: offset -> size of free runs
    unsigned char* arena = nullptr;
    size_t arena_bytes = 0;
    std::map<size_t, size_t> free_runs;
    // bookkeeping
    struct Req {
        int64_t id, tag;
        int32_t graph, source;
        int wide, retried;
        size_t off, bytes;
        double submit_us;
        uint64_t k;  // ring index while on the device
        bool on_device, done;
        dfq_server_result res;
    };
    std::deque<int64_t> queue;
    std::unordered_map<int64_t, Req> reqs;
    std::map<uint64_t, int64_t> owner[2];  // ring index -> request id (outstanding)
    uint64_t published[2] = {0, 0};
    std::deque<int64_t> completed;
    int64_t next_id = 1;
    int64_t pending = 0;
    std::chrono::steady_clock::time_point t0;
    double now_us() const {
        return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

using namespace dfqpool;

template <int B, bool PAR>
const void* serve_fn() { return (const void*)dfq_serve_kernel<B, PAR>; }

const void* pick_serve(int B, bool par) {
    switch (B) {
        case 256: return par ? serve_fn<256, true>() : serve_fn<256, false>();
        case 512: return par ? serve_fn<512, true>() : serve_fn<512, false>();
        case 1024: return par ? serve_fn<1024, true>() : serve_fn<1024, false>();
        default: return nullptr;
    }
}

bool arena_alloc(dfq_server* s, size_t bytes, size_t* off) {
    bytes = al256(bytes);
    for (auto it = s->free_runs.begin(); it != s->free_runs.end(); ++it) {
        if (it->second >= bytes) {
            *off = it->first;
            const size_t rest = it->second - bytes, start = it->first + bytes;
            s->free_runs.erase(it);
            if (rest) s->free_runs[start] = rest;
            return true;
        }
    }
    return false;
}

void arena_free(dfq_server* s, size_t off, size_t bytes) {
    bytes = al256(bytes);
    auto it = s->free_runs.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != s->free_runs.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        s->free_runs.erase(nx);
    }
    if (it != s->free_runs.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            s->free_runs.erase(it);
        }
    }
}

void server_release_all(dfq_server* s) {
    if (!s) return;
    cudaSetDevice(s->pool->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (int r = 0; r < 2; ++r) {
        if (s->h_ring[r]) cudaFreeHost(s->h_ring[r]);
        if (s->h_done[r]) cudaFreeHost(s->h_done[r]);
        cudaFree(s->d_ctls[r]);
    }
    if (s->h_host) cudaFreeHost(s->h_host);
    cudaFree(s->d_dev);
    cudaFree(s->d_block_state);
    cudaFree(s->block_mem);
    cudaFree(s->arena);
    if (s->kernel_done) cudaEventDestroy(s->kernel_done);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int launch_serve(dfq_server* s) {
    dfq_pool* p = s->pool;
    const dfq_opts& o = p->opts;
    ServeParams sp;
    memset(&sp, 0, sizeof sp);
    sp.graphs = p->d_graphs;
    for (int r = 0; r < 2; ++r) {
        sp.ring[r] = s->d_ring[r];
        sp.done[r] = s->d_done[r];
        sp.ctls[r] = s->d_ctls[r];
    }
    sp.host = s->d_host;
    sp.dev = s->d_dev;
    sp.cap = s->opts.ring_capacity;
    sp.wide_ws = ws_from(p->wide_mem, p->wide_lay);
    sp.wide_ovf_cap = 1 << 30;
    sp.block_ws = s->block_mem;
    sp.block_ws_stride = s->block_stride;
    sp.block_lay = s->block_lay;
    sp.block_ovf_cap = s->opts.narrow_queue_cap;
    sp.block_state = s->d_block_state;
    sp.gang_min = std::max(1, s->grid / 2);
    sp.narrow_limit = std::max(1, s->grid - sp.gang_min);
    sp.join_ns = 200000;
    sp.medium_min = o.medium_min_degree;
    sp.large_min = o.large_min_degree;
    sp.piece_edges = o.piece_edges;
    sp.local_cap = o.local_queue_cap;
    sp.local_budget = o.local_edge_budget;
    sp.probe_first = o.probe_first;
    sp.use_tma = o.use_tma;
    sp.timeout_ns = (long long)o.timeout_ms * 1000000LL;
    sp.hot_words = s->hot_words;
    sp.idle_ns = (long long)s->opts.idle_ms * 1000000LL;
    // reset the per-launch state; claim cursors persist across launches
    ServeDev reset;
    memset(&reset, 0, sizeof reset);
    const size_t from = offsetof(ServeDev, gang_word);
    cudaError_t err = cudaMemcpyAsync(reinterpret_cast<char*>(s->d_dev) + from, reinterpret_cast<char*>(&reset) + from,
                                      sizeof(ServeDev) - from, cudaMemcpyHostToDevice, s->stream);
    if (err != cudaSuccess) return fail(DFQ_ECUDA, "serve reset: %s", cudaGetErrorString(err));
    void* args[] = {&sp};
    err = cudaLaunchCooperativeKernel(s->fn, dim3(s->grid), dim3(o.block_threads), args, s->smem, s->stream);
    if (err != cudaSuccess) return fail(DFQ_ECUDA, "serving kernel launch: %s", cudaGetErrorString(err));
    cudaEventRecord(s->kernel_done, s->stream);
    s->running = true;
    return DFQ_OK;
}

// Write request r into the next slot of its ring and publish it.
void publish(dfq_server* s, dfq_server::Req& r) {
    const int ring = r.wide ? 1 : 0;
    const uint64_t k = s->published[ring];
    ServeReq* slot = &s->h_ring[ring][k & (uint64_t)(s->opts.ring_capacity - 1)];
    volatile ServeReq* v = slot;
    int32_t* lv = (int32_t*)(s->arena + r.off);
    v->graph = r.graph;
    v->source = r.source;
    v->levels = lv;
    v->parents = s->opts.with_parents ? lv + s->pool->n[r.graph] : nullptr;
    std::atomic_thread_fence(std::memory_order_release);
    v->seq = k + 1;
    std::atomic_thread_fence(std::memory_order_release);
    s->published[ring] = k + 1;
    reinterpret_cast<std::atomic<unsigned long long>*>(&s->h_host->avail[ring])->store(k + 1, std::memory_order_release);
    r.k = k;
    r.on_device = true;
    s->owner[ring][k] = r.id;
}

void admit(dfq_server* s) {
    while (!s->queue.empty()) {
        dfq_server::Req& r = s->reqs[s->queue.front()];
        const int ring = r.wide ? 1 : 0;
        if ((int)s->owner[ring].size() >= s->opts.ring_capacity) break;
        // the ring slot must not still be read by the device: the oldest
        // outstanding index bounds reuse
        if (!s->owner[ring].empty() &&
            s->published[ring] - s->owner[ring].begin()->first >= (uint64_t)s->opts.ring_capacity)
            break;
        if (!r.bytes) {
            r.bytes = sizeof(int32_t) * (size_t)s->pool->n[r.graph] * (s->opts.with_parents ? 2 : 1);
            if (!arena_alloc(s, r.bytes, &r.off)) { r.bytes = 0; break; }
        }
        publish(s, r);
        s->queue.pop_front();
    }
}

void collect(dfq_server* s) {
    for (int ring = 0; ring < 2; ++ring) {
        for (auto it = s->owner[ring].begin(); it != s->owner[ring].end();) {
            const uint64_t k = it->first;
            const ServeDone* d = &s->h_done[ring][k & (uint64_t)(s->opts.ring_capacity - 1)];
            const unsigned long long seq =
                reinterpret_cast<const std::atomic<unsigned long long>*>(&d->seq)->load(std::memory_order_acquire);
            if (seq != k + 1) { ++it; continue; }
            dfq_server::Req& r = s->reqs[it->second];
            const volatile ServeDone* v = d;
            const int st = v->status;
            it = s->owner[ring].erase(it);
            r.on_device = false;
            if (st == kErrQueueCap && !r.wide) {
                // outgrew the block's bounded queues: rerun on the whole grid
                r.wide = 1;
                r.retried = 1;
                s->queue.push_front(r.id);
                continue;
            }
            r.done = true;
            r.res.id = r.id;
            r.res.tag = r.tag;
            r.res.status = st == kErrNone ? DFQ_OK : (st == kErrQueueCap ? DFQ_EDEVICE : DFQ_ETIMEOUT);
            r.res.wide = r.wide;
            r.res.retried = r.retried;
            r.res.depth = v->depth;
            r.res.reached = v->reached;
            r.res.edges = v->edges;
            r.res.submit_us = r.submit_us;
            r.res.done_us = s->now_us();
            r.res.device_us = (double)(v->t_end - v->t_start) * 1e-3;
            s->completed.push_back(r.id);
            --s->pending;
        }
    }
}

}  // namespace

extern "C" {

int dfq_server_create(dfq_pool* pool, const dfq_server_opts* opts, dfq_server** out) {
    clear_error();
    if (!pool || !out) return fail(DFQ_EINVAL, "dfq_server_create: null argument");
    *out = nullptr;
    dfq_server_opts o{};
    if (opts) o = *opts;
    if (o.ring_capacity <= 0) o.ring_capacity = 4096;
    if (o.ring_capacity & (o.ring_capacity - 1)) return fail(DFQ_EINVAL, "ring_capacity must be a power of two");
    if (o.idle_ms <= 0) o.idle_ms = 20;
    if (o.narrow_queue_cap <= 0) o.narrow_queue_cap = 1 << 20;
    cudaSetDevice(pool->device);
    dfq_server* s = new dfq_server();
    s->pool = pool;
    s->t0 = std::chrono::steady_clock::now();
#define S_TRY(x) do { int rc_ = (x); if (rc_) { server_release_all(s); return rc_; } } while (0)
#define S_CUDA(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { server_release_all(s); return fail(DFQ_ECUDA, "%s: %s", #x, cudaGetErrorString(e_)); } } while (0)
    const bool par = o.with_parents != 0;
    const dfq_opts& po = pool->opts;
    s->fn = pick_serve(po.block_threads, par);
    if (!s->fn) { server_release_all(s); return fail(DFQ_EINVAL, "block_threads %d", po.block_threads); }
    s->hot_words = 0;
    if (hot_limit_words(po.hot_cache) > 0)  // the cache only on request
        for (int i = 0; i < pool->ngraphs; ++i)
            s->hot_words = std::max(s->hot_words, hot_words_of(hot_limit_words(po.hot_cache), pool->n[i]));
    s->smem = smem_layout(po.block_threads, po.local_queue_cap, po.piece_edges, par).bytes + 4 * s->hot_words;
    S_TRY(grid_for(pool, s->fn, po.block_threads, s->smem, &s->grid));
    S_TRY(ensure_wide(pool, par));
    // narrow workspaces: bitmap for the largest narrow graph, bounded queues
    long long nmax = 1;
    for (int i = 0; i < pool->ngraphs; ++i)
        if (!pool->wide[i]) nmax = std::max<long long>(nmax, pool->n[i]);
    const long long qcap = std::min<long long>(nmax, o.narrow_queue_cap);
    WsLayout l = ws_layout(nmax, 0, kMinLarge, kMinPiece, par);
    {
        // queues for qcap entries, at most 1 << 18 large-list pieces per level
        size_t off = 0;
        l.bitmap = off;
        off = al256(off + 4 * (size_t)(((nmax + 31) / 32 + 31) & ~31LL));
        for (int i = 0; i < 2; ++i) { l.ovf[i] = off; off = al256(off + 8 * (size_t)qcap); }
        for (int i = 0; i < 2; ++i) { l.ovfv[i] = off; off = al256(off + (par ? 4 * (size_t)qcap : 256)); }
        l.piece_cap = 1 << 18;
        for (int i = 0; i < 2; ++i) { l.piece[i] = off; off = al256(off + 8 * (size_t)l.piece_cap); }
        for (int i = 0; i < 2; ++i) { l.piece_v[i] = off; off = al256(off + (par ? 4 * (size_t)l.piece_cap : 256)); }
        l.total = off;
    }
    s->block_lay = l;
    s->block_stride = al256(l.total);
    o.narrow_queue_cap = (int)qcap;
    s->opts = o;
    S_TRY(dmalloc(&s->block_mem, s->block_stride * (size_t)s->grid));
    // arena
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    s->arena_bytes = o.hbm_budget_bytes > 0 ? (size_t)o.hbm_budget_bytes : free_b / 4;
    s->arena_bytes &= ~(size_t)255;
    S_TRY(dmalloc(&s->arena, s->arena_bytes));
    s->free_runs[0] = s->arena_bytes;
    // rings and counters
    const size_t cap = (size_t)o.ring_capacity;
    for (int r = 0; r < 2; ++r) {
        S_CUDA(cudaHostAlloc((void**)&s->h_ring[r], sizeof(ServeReq) * cap, cudaHostAllocMapped));
        S_CUDA(cudaHostAlloc((void**)&s->h_done[r], sizeof(ServeDone) * cap, cudaHostAllocMapped));
        memset(s->h_ring[r], 0, sizeof(ServeReq) * cap);
        memset(s->h_done[r], 0, sizeof(ServeDone) * cap);
        S_CUDA(cudaHostGetDevicePointer((void**)&s->d_ring[r], s->h_ring[r], 0));
        S_CUDA(cudaHostGetDevicePointer((void**)&s->d_done[r], s->h_done[r], 0));
        S_TRY(dmalloc(&s->d_ctls[r], sizeof(Control) * cap));
    }
    S_CUDA(cudaHostAlloc((void**)&s->h_host, sizeof(ServeHost), cudaHostAllocMapped));
    memset(s->h_host, 0, sizeof(ServeHost));
    S_CUDA(cudaHostGetDevicePointer((void**)&s->d_host, s->h_host, 0));
    S_TRY(dmalloc(&s->d_dev, sizeof(ServeDev)));
    S_TRY(dmalloc(&s->d_block_state, sizeof(int) * (size_t)s->grid));
    S_CUDA(cudaMemset(s->d_block_state, 0, sizeof(int) * (size_t)s->grid));
    S_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    S_CUDA(cudaEventCreateWithFlags(&s->kernel_done, cudaEventDisableTiming));
    S_CUDA(cudaMemsetAsync(s->d_dev, 0, sizeof(ServeDev), s->stream));
    S_CUDA(cudaStreamSynchronize(s->stream));
#undef S_TRY
#undef S_CUDA
    *out = s;
    return DFQ_OK;
}

int dfq_server_submit(dfq_server* s, int32_t graph, int32_t source, int64_t tag, int64_t* id) {
    clear_error();
    if (!s || graph < 0 || graph >= s->pool->ngraphs) return fail(DFQ_EINVAL, "dfq_server_submit: bad graph");
    if (source < 0 || source >= s->pool->n[graph]) return fail(DFQ_EINVAL, "dfq_server_submit: bad source");
    const size_t need = sizeof(int32_t) * (size_t)s->pool->n[graph] * (s->opts.with_parents ? 2 : 1);
    if (al256(need) > s->arena_bytes) return fail(DFQ_ENOMEM, "request needs %zu bytes, arena holds %zu", need, s->arena_bytes);
    dfq_server::Req r{};
    r.id = s->next_id++;
    r.tag = tag;
    r.graph = graph;
    r.source = source;
    r.wide = s->pool->wide[graph];
    r.submit_us = s->now_us();
    s->reqs[r.id] = r;
    s->queue.push_back(r.id);
    ++s->pending;
    if (id) *id = r.id;
    return DFQ_OK;
}

int dfq_server_poll(dfq_server* s, dfq_server_result* out, int32_t max, int32_t* count) {
    clear_error();
    if (!s || (max > 0 && !out)) return fail(DFQ_EINVAL, "dfq_server_poll: bad arguments");
    cudaSetDevice(s->pool->device);
    int rc = DFQ_OK;
    if (s->running) {
        const cudaError_t q = cudaEventQuery(s->kernel_done);
        if (q == cudaSuccess) s->running = false;
        else if (q != cudaErrorNotReady) return fail(DFQ_ECUDA, "serving kernel: %s", cudaGetErrorString(q));
    }
    collect(s);
    admit(s);
    const bool outstanding = !s->owner[0].empty() || !s->owner[1].empty();
    if (outstanding && !s->running) rc = launch_serve(s);
    int n = 0;
    while (n < max && !s->completed.empty()) {
        out[n++] = s->reqs[s->completed.front()].res;
        s->completed.pop_front();
    }
    if (count) *count = n;
    return rc;
}

int dfq_server_levels(dfq_server* s, int64_t id, int32_t* levels, int32_t* parents) {
    clear_error();
    if (!s) return fail(DFQ_EINVAL, "dfq_server_levels: null server");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || !it->second.done) return fail(DFQ_EINVAL, "request %lld is not completed", (long long)id);
    const dfq_server::Req& r = it->second;
    const size_t n = (size_t)s->pool->n[r.graph];
    cudaSetDevice(s->pool->device);
    if (levels && cudaMemcpy(levels, s->arena + r.off, 4 * n, cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(DFQ_ECUDA, "copy of levels failed");
    if (parents) {
        if (!s->opts.with_parents) return fail(DFQ_EINVAL, "server keeps no parents");
        if (cudaMemcpy(parents, s->arena + r.off + 4 * n, 4 * n, cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail(DFQ_ECUDA, "copy of parents failed");
    }
    return DFQ_OK;
}

int dfq_server_release(dfq_server* s, int64_t id) {
    clear_error();
    if (!s) return fail(DFQ_EINVAL, "dfq_server_release: null server");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || !it->second.done) return fail(DFQ_EINVAL, "request %lld is not completed", (long long)id);
    if (it->second.bytes) arena_free(s, it->second.off, it->second.bytes);
    s->reqs.erase(it);
    return DFQ_OK;
}

int64_t dfq_server_pending(const dfq_server* s) { return s ? s->pending : -1; }

int dfq_server_replay(dfq_server* s, const int32_t* graph, const int32_t* source, const double* arrival_us,
                      int32_t n, const int32_t* keep, dfq_server_result* results) {
    clear_error();
    if (!s || n < 0 || (n > 0 && (!graph || !source || !arrival_us || !results)))
        return fail(DFQ_EINVAL, "dfq_server_replay: bad arguments");
    for (int32_t i = 0; i < n; ++i) {
        if (graph[i] < 0 || graph[i] >= s->pool->ngraphs || source[i] < 0 || source[i] >= s->pool->n[graph[i]])
            return fail(DFQ_EINVAL, "dfq_server_replay: request %d is out of range", i);
        if (i && arrival_us[i] < arrival_us[i - 1]) return fail(DFQ_EINVAL, "arrival times must not decrease");
    }
    const double base = s->now_us();
    std::vector<dfq_server_result> buf(1024);
    int32_t next = 0, done = 0;
    int rc = DFQ_OK;
    while (done < n) {
        const double now = s->now_us() - base;
        while (next < n && arrival_us[next] <= now) {
            int64_t id = 0;
            if ((rc = dfq_server_submit(s, graph[next], source[next], next, &id))) return rc;
            ++next;
        }
        int32_t got = 0;
        if ((rc = dfq_server_poll(s, buf.data(), (int32_t)buf.size(), &got))) return rc;
        for (int32_t j = 0; j < got; ++j) {
            dfq_server_result r = buf[j];
            const int64_t i = r.tag;
            r.submit_us = arrival_us[i];
            r.done_us -= base;
            results[i] = r;
            ++done;
            if (!keep || !keep[i]) dfq_server_release(s, r.id);
        }
    }
    return DFQ_OK;
}

int dfq_server_destroy(dfq_server* s) {
    clear_error();
    if (!s) return fail(DFQ_EINVAL, "dfq_server_destroy: null server");
    reinterpret_cast<std::atomic<int>*>(&s->h_host->stop)->store(1, std::memory_order_release);
    cudaSetDevice(s->pool->device);
    // the serving kernel leaves once it sees stop; wait for that, bounded
    const auto t0 = std::chrono::steady_clock::now();
    while (s->running) {
        const cudaError_t q = cudaEventQuery(s->kernel_done);
        if (q != cudaErrorNotReady) { s->running = false; break; }
        if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(10)) {
            // report what every block was doing, read on a side stream while
            // the kernel still runs; the server is left allocated
            cudaStream_t side;
            cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
            ServeDev dv;
            std::vector<int> st((size_t)s->grid);
            cudaMemcpyAsync(&dv, s->d_dev, sizeof dv, cudaMemcpyDeviceToHost, side);
            cudaMemcpyAsync(st.data(), s->d_block_state, sizeof(int) * st.size(), cudaMemcpyDeviceToHost, side);
            cudaStreamSynchronize(side);
            cudaStreamDestroy(side);
            int hist[8] = {0};
            for (int v : st) hist[v & 7]++;
            fprintf(stderr,
                    "dfq_server_destroy: serving kernel still running: narrow_next=%llu narrow_avail=%llu "
                    "gang_done=%llu gang_word=%llx exit=%d error=%d narrow_active=%d gang_left=%d "
                    "published=%llu/%llu; block actions wait=%d narrow=%d gang=%d exit=%d retry=%d; "
                    "block0 state=%d iters=%d\n",
                    (unsigned long long)dv.narrow_next, (unsigned long long)dv.narrow_avail,
                    (unsigned long long)dv.gang_done, (unsigned long long)dv.gang_word, dv.exit, dv.error,
                    dv.narrow_active, dv.gang_left, (unsigned long long)s->published[0],
                    (unsigned long long)s->published[1], hist[0], hist[1], hist[2], hist[3], hist[4], st[0] & 15,
                    st[0] >> 4);
            return fail(DFQ_ETIMEOUT, "serving kernel did not stop within 10 s");
        }
        std::this_thread::sleep_for(std::chrono::milliseconds(1));
    }
    server_release_all(s);
    return DFQ_OK;
}

}  // extern "C"
