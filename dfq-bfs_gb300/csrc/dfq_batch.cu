// Graph pools and batched BFS: many graphs resident on the device, many
// (graph, source) queries in one persistent cooperative launch.
//
// No reference counterpart: a reference program handles one graph and runs
// one source per launch (design/shared-q/atomic-sa/our-sep/upper-bound/
// bfs.cu:202-309).  The batch kernel reuses the single-source BFS body
// (bfs_run) with two group shapes:
//   wide queries   - graphs with many edges and a short diameter - run one
//                    after another on the whole grid (grid barrier per level);
//   narrow queries - small or high-diameter graphs - are pulled by blocks, and
//                    each block runs its query alone, its block barrier being
//                    the level barrier.  A level then costs a __syncthreads
//                    instead of a grid barrier, and 2 x SMs queries proceed at
//                    once.
// Narrow queries are handed out largest-estimated-cost first.
#include "common.hpp"
#include "dfq_pool.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

using namespace dfq;

namespace dfqk {

struct BatchParams {
    const PoolGraph* graphs;
    BatchQuery* queries;
    Control* ctls;          // one per query, zeroed before the launch
    const int* wide_list;   // query indices run on the whole grid, in order
    int n_wide;
    const int* narrow_list; // query indices run by one block, costliest first
    int n_narrow;
    int* narrow_next;       // cursor over narrow_list
    long long* t0;          // device clock at the start of the launch
    Workspace wide_ws;
    unsigned char* block_ws;  // per-block workspaces, block_ws_stride bytes apart
    size_t block_ws_stride;
    WsLayout block_lay;       // layout of each of them
    int medium_min, large_min, piece_edges, local_cap, local_budget, probe_first, use_tma;
    long long timeout_ns;
    int hot_words;  // hot-vertex cache words this launch reserves (0: none)
    int reserve;    // blocks that skip the wide phase (the gangs, then narrow starters)
    // gangs: the last n_gangs * gang_size blocks form n_gangs fixed groups of
    // gang_size blocks; each gang runs the gang queries (large high-diameter
    // graphs, costliest first) one after another from the launch's start,
    // then its blocks pull narrow queries like the others
    const int* gang_list;
    int n_gang;
    int* gang_next;                 // cursor over gang_list
    unsigned long long* gang_word;  // per gang: (round << 32) | (query + 1), set by its first block
    int n_gangs, gang_size;
    unsigned char* gang_ws;         // per-gang workspaces, gang_ws_stride bytes apart
    size_t gang_ws_stride;
    WsLayout gang_lay;
};

// Published-query word of a gang: release store by the gang's first block,
// acquire loads (ld_acquire_u64) by every member.
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void fill_params(Params& sp, const BatchParams& bp, int qi, const Workspace& ws) {
    const BatchQuery& q = bp.queries[qi];
    const PoolGraph& g = bp.graphs[q.graph];
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
    sp.piece_cap = ws.piece_cap;
    sp.ovf_cap = g.n;
    sp.ctl = bp.ctls + qi;
    sp.medium_min = bp.medium_min;
    sp.large_min = bp.large_min;
    sp.piece_edges = bp.piece_edges;
    sp.local_cap = bp.local_cap;
    sp.local_budget = bp.local_budget;
    sp.probe_first = bp.probe_first;
    sp.use_tma = bp.use_tma;
    sp.timeout_ns = bp.timeout_ns;
    sp.hot_words = hot_words_of(bp.hot_words, g.n);
    sp.tally_bar = tally_bar_for(g.n, g.e);
    remap_params(sp, g, ws);  // renumbered graphs are wide: only the grid's workspace has room
}

// This block's narrow-query workspace.
__device__ __forceinline__ Workspace block_workspace(const BatchParams& bp) {
    Workspace bw;
    unsigned char* base = bp.block_ws + bp.block_ws_stride * blockIdx.x;
    const WsLayout& l = bp.block_lay;
    bw.bitmap = (unsigned*)(base + l.bitmap);
    for (int i = 0; i < 2; ++i) {
        bw.ovf[i] = (int2*)(base + l.ovf[i]);
        bw.ovfv[i] = (int*)(base + l.ovfv[i]);
        bw.piece[i] = (int2*)(base + l.piece[i]);
        bw.piece_v[i] = (int*)(base + l.piece_v[i]);
    }
    bw.piece_cap = l.piece_cap;
    bw.levels_int = nullptr;  // one-block workspaces take no renumbered graph
    bw.parents_int = nullptr;
    bw.hub_claim = nullptr;
    return bw;
}

// This gang's workspace.
__device__ __forceinline__ Workspace gang_workspace(const BatchParams& bp, int gang) {
    Workspace gw;
    unsigned char* base = bp.gang_ws + bp.gang_ws_stride * gang;
    const WsLayout& l = bp.gang_lay;
    gw.bitmap = (unsigned*)(base + l.bitmap);
    for (int i = 0; i < 2; ++i) {
        gw.ovf[i] = (int2*)(base + l.ovf[i]);
        gw.ovfv[i] = (int*)(base + l.ovfv[i]);
        gw.piece[i] = (int2*)(base + l.piece[i]);
        gw.piece_v[i] = (int*)(base + l.piece_v[i]);
    }
    gw.piece_cap = l.piece_cap;
    gw.levels_int = nullptr;  // gang queries are narrow graphs, kept in input ids
    gw.parents_int = nullptr;
    gw.hub_claim = nullptr;
    return gw;
}

// Gangs run the gang queries from the launch's start; wide queries run one
// after another on the wide blocks; then every block pulls narrow queries
// and runs each alone.  One call site of bfs_run (the group shape is chosen
// per query) keeps the kernel to one inlined copy.
template <int B, bool PAR>
__global__ void __launch_bounds__(B, 1024 / B) dfq_batch_kernel(const __grid_constant__ BatchParams bp) {
    __shared__ Params sp;
    __shared__ int s_q, s_gsize, s_grank;
    // thread 0's schedule state lives in shared memory and the block's shape
    // (wide / gang, rank) is recomputed from the launch parameters per round,
    // so no register stays live across bfs_run beyond the warp state
    __shared__ unsigned s_round;  // gang rounds taken (0: this block is in no gang or left it)
    __shared__ int s_k;           // next wide query of this block
    init_warp_barriers<B, PAR>(bp.local_cap, bp.piece_edges);
    WarpState ws{0u, false};
    if (threadIdx.x == 0) {
        if (blockIdx.x == 0) *bp.t0 = (long long)globaltimer();
        const int gang_rel = (int)blockIdx.x - ((int)gridDim.x - bp.n_gangs * bp.gang_size);
        s_round = bp.n_gangs > 0 && gang_rel >= 0 ? 1u : 0u;
        s_k = (int)blockIdx.x < (int)gridDim.x - bp.reserve ? 0 : bp.n_wide;
    }
    // The last `reserve` blocks skip the wide queries: first the gangs, then
    // blocks that start on the narrow ones (costliest first) at once, so the
    // longest narrow runs overlap the wide phase instead of trailing it; the
    // wide queries run on the others.
    // Gang phase first (gang blocks): the gang's first block takes the next
    // gang query and publishes it; every member waits for the publication
    // (bounded), then the gang runs the query with its blocks as the group.
    // A member reads a round's word before that run's first group barrier,
    // and the first block publishes the next round only after the run, so no
    // round is missed.  Then wide queries (wide blocks), then narrow pulls.
    for (;;) {
        if (threadIdx.x == 0) {
            s_q = -1;
            if (s_round) {
                const int gang_rel = (int)blockIdx.x - ((int)gridDim.x - bp.n_gangs * bp.gang_size);
                const int gang = gang_rel / bp.gang_size, gang_rank = gang_rel % bp.gang_size;
                const unsigned round = s_round;
                unsigned long long* word = bp.gang_word + gang;
                if (gang_rank == 0) {
                    const int j = atomicAdd(bp.gang_next, 1);
                    const int q = j < bp.n_gang ? bp.gang_list[j] : -1;
                    st_release_u64(word, ((unsigned long long)round << 32) | (unsigned)(q + 1));
                }
                unsigned long long w = ld_acquire_u64(word);
                const unsigned long long t_wait = globaltimer();
                while ((unsigned)(w >> 32) != round) {
                    if ((long long)(globaltimer() - t_wait) > bp.timeout_ns) break;  // leave the gang
                    w = ld_acquire_u64(word);
                }
                const int q = (unsigned)(w >> 32) == round ? (int)(unsigned)w - 1 : -1;
                if (q >= 0) {
                    s_q = q;
                    s_gsize = bp.gang_size;
                    s_grank = gang_rank;
                    s_round = round + 1;
                    fill_params(sp, bp, q, gang_workspace(bp, gang));
                    if (gang_rank == 0) bp.queries[q].t_start = (long long)globaltimer();
                } else {
                    s_round = 0;
                }
            }
            if (s_q < 0) {
                if (s_k < bp.n_wide) {
                    s_q = bp.wide_list[s_k++];
                    s_gsize = (int)gridDim.x - bp.reserve;
                    s_grank = (int)blockIdx.x;
                    fill_params(sp, bp, s_q, bp.wide_ws);
                    if (blockIdx.x == 0) bp.queries[s_q].t_start = (long long)globaltimer();
                } else {
                    const int j = atomicAdd(bp.narrow_next, 1);
                    s_q = j < bp.n_narrow ? bp.narrow_list[j] : -1;
                    s_gsize = 1;
                    s_grank = 0;
                    if (s_q >= 0) {
                        fill_params(sp, bp, s_q, block_workspace(bp));
                        bp.queries[s_q].t_start = (long long)globaltimer();
                    }
                }
            }
        }
        __syncthreads();
        if (s_q < 0) break;
        bfs_run<B, PAR>(sp, s_gsize, s_grank, ws);
        // the group's first block records the end (block 0 for wide queries)
        if (threadIdx.x == 0 && s_grank == 0) bp.queries[s_q].t_end = (long long)globaltimer();
        __syncthreads();
    }
}

}  // namespace dfqk

using namespace dfqk;

using namespace dfqpool;

namespace {

// (Re)allocate the per-block workspaces for the largest narrow graph.
int ensure_blocks(dfq_pool* p, int grid, bool par) {
    long long nmax = 1, emax = 0;
    for (int i = 0; i < p->ngraphs; ++i)
        if (!p->wide[i]) { nmax = std::max<long long>(nmax, p->n[i]); emax = std::max<long long>(emax, p->e[i]); }
    if (p->block_mem && p->block_grid >= grid && (p->block_par || !par) && p->block_n >= nmax) return DFQ_OK;
    cudaFree(p->block_mem);
    p->block_mem = nullptr;
    p->block_lay = ws_layout(nmax, emax, kMinLarge, kMinPiece, par);
    p->block_stride = al256(p->block_lay.total);
    p->block_grid = grid;
    p->block_n = (int)nmax;
    p->block_par = par;
    return dmalloc(&p->block_mem, p->block_stride * (size_t)grid);
}

// Gangs: a narrow graph with at least kGangMinVertices vertices and an
// average degree below kGangMaxDegree (a high-diameter graph: a grid, a
// road-like mesh) runs thousands of levels; on one block each level is slow
// (a few warps carry its whole frontier), so such queries get a gang of
// blocks when the batch leaves enough of them: the gang budget is half the
// grid, shared evenly (at most kGangMax blocks per gang, at most kGangsMax
// gangs); with fewer than 2 blocks per query they stay narrow.  Half rather
// than a quarter measured better on the 256-graph pool: batches of 256 went
// from 13.4k to 15.7k queries/s with the gang p99 from 19.9 to 16.1 ms.
constexpr int32_t kGangMinVertices = 1 << 16;
constexpr int kGangMaxDegree = 8;
constexpr int kGangMax = 16;
constexpr int kGangsMax = 24;  // gang words live in the 256-byte misc block, from byte 64

bool gang_graph(const dfq_pool* p, int graph) {
    return !p->wide[graph] && p->n[graph] >= kGangMinVertices &&
           p->e[graph] < (int64_t)kGangMaxDegree * p->n[graph];
}

// (Re)allocate `gangs` gang workspaces for the largest gang graph.
int ensure_gangs(dfq_pool* p, int gangs, bool par) {
    long long nmax = 1, emax = 0;
    for (int i = 0; i < p->ngraphs; ++i)
        if (gang_graph(p, i)) { nmax = std::max<long long>(nmax, p->n[i]); emax = std::max<long long>(emax, p->e[i]); }
    if (p->gang_mem && p->gang_count >= gangs && (p->gang_par || !par)) return DFQ_OK;
    cudaFree(p->gang_mem);
    p->gang_mem = nullptr;
    p->gang_lay = ws_layout(nmax, emax, kMinLarge, kMinPiece, par);
    p->gang_stride = al256(p->gang_lay.total);
    p->gang_count = gangs;
    p->gang_par = par;
    return dmalloc(&p->gang_mem, p->gang_stride * (size_t)std::max(gangs, 1));
}

int ensure_tables(dfq_pool* p, int nq) {
    if (p->qcap >= nq) return DFQ_OK;
    cudaFree(p->d_queries); cudaFree(p->d_lists); cudaFree(p->d_ctls);
    if (p->h_queries) cudaFreeHost(p->h_queries);
    if (p->h_lists) cudaFreeHost(p->h_lists);
    if (p->h_ctls) cudaFreeHost(p->h_ctls);
    p->d_queries = nullptr; p->d_lists = nullptr; p->d_ctls = nullptr;
    p->h_queries = nullptr; p->h_lists = nullptr; p->h_ctls = nullptr;
    p->qcap = 0;
    int rc;
    if ((rc = dmalloc(&p->d_queries, sizeof(BatchQuery) * nq))) return rc;
    if ((rc = dmalloc(&p->d_lists, sizeof(int) * 2 * nq))) return rc;
    if ((rc = dmalloc(&p->d_ctls, sizeof(Control) * nq))) return rc;
    if (cudaMallocHost((void**)&p->h_queries, sizeof(BatchQuery) * nq) != cudaSuccess ||
        cudaMallocHost((void**)&p->h_lists, sizeof(int) * 2 * nq) != cudaSuccess ||
        cudaMallocHost((void**)&p->h_ctls, sizeof(Control) * nq) != cudaSuccess)
        return fail(DFQ_ENOMEM, "pinned host tables for %d queries", nq);
    p->qcap = nq;
    if (p->gexec) { cudaGraphExecDestroy(p->gexec); p->gexec = nullptr; p->g_nq = -1; }
    return DFQ_OK;
}

template <int B, bool PAR>
void* batch_fn() { return (void*)dfq_batch_kernel<B, PAR>; }

void* pick_batch(int B, bool par) {
    switch (B) {
        case 256: return par ? batch_fn<256, true>() : batch_fn<256, false>();
        case 512: return par ? batch_fn<512, true>() : batch_fn<512, false>();
        case 1024: return par ? batch_fn<1024, true>() : batch_fn<1024, false>();
        default: return nullptr;
    }
}
int launch_coop(const void* fn, int grid, int B, int smem, void* arg, cudaStream_t s) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(B);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {arg};
    cudaError_t err = cudaLaunchKernelExC(&cfg, fn, args);
    if (err != cudaSuccess) return fail(DFQ_ECUDA, "cooperative launch: %s", cudaGetErrorString(err));
    return DFQ_OK;
}

int map_status(int st) {
    switch (st) {
        case kErrNone: return DFQ_OK;
        case kErrBarrierTimeout:
        case kErrTmaTimeout: return DFQ_ETIMEOUT;
        default: return DFQ_EDEVICE;
    }
}

// block_threads = 0 for a pool or a server: 1,024-thread blocks (one per SM)
// where their shared-memory layout, with parents and the requested hot cache,
// fits; else 512.  Measured on the 42 GB serving pool at 1,000 and 2,000
// requests/s offered: p99 157 / 193 ms against 236 / 301 ms with 512, and
// 1,723 against 1,574 requests/s sustained; the pool autotuner also picks
// 1,024 on the 256-graph batch pool.
int pool_block_threads(const dfq_opts& o) {
    const SmemLayout L = smem_layout(1024, o.local_queue_cap ? o.local_queue_cap : 256, o.piece_edges, true);
    const int need = L.bytes + (o.hot_cache > 0 ? 4 * kHotWordsMax : 0);
    return need <= 227 * 1024 ? 1024 : 512;
}

}  // namespace

extern "C" {

int dfq_pool_create(const dfq_csr* graphs, int32_t ngraphs, const dfq_opts* opts, dfq_pool** out) {
    clear_error();
    if (!out || !graphs || ngraphs < 1) return fail(DFQ_EINVAL, "dfq_pool_create: need graphs");
    *out = nullptr;
    dfq_opts o;
    dfq_opts_default(&o);
    if (opts) o = *opts;
    if (o.wide_min_edges <= 0) o.wide_min_edges = 1 << 21;
    if (o.wide_min_degree <= 0) o.wide_min_degree = 8;
    if (o.block_threads == 0) o.block_threads = pool_block_threads(o);
    if (o.local_queue_cap == 0) o.local_queue_cap = 256;
    if (o.local_edge_budget == 0) o.local_edge_budget = 8192;
    if (o.timeout_ms == 0) o.timeout_ms = 5000;
    dfq_pool* p = new dfq_pool();
    p->opts = o;
    p->ngraphs = ngraphs;
    cudaGetDevice(&p->device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, p->device) != cudaSuccess) { pool_release(p); return fail(DFQ_ECUDA, "no CUDA device"); }
    p->sms = prop.multiProcessorCount;
    int64_t tot_n = 0, tot_e = 0;
    std::vector<int64_t> off_base(ngraphs), col_base(ngraphs);
    for (int i = 0; i < ngraphs; ++i) {
        const dfq_csr& g = graphs[i];
        if (g.n < 1 || g.e < 0 || !g.offsets || (g.e > 0 && !g.cols) || g.offsets[0] != 0 || g.offsets[g.n] != g.e) {
            pool_release(p);
            return fail(DFQ_EFORMAT, "pool graph %d is not a valid CSR", i);
        }
        for (int32_t u = 0; u < g.n; ++u)
            if (g.offsets[u + 1] < g.offsets[u]) { pool_release(p); return fail(DFQ_EFORMAT, "graph %d: offsets decrease", i); }
        for (int64_t k = 0; k < g.e; ++k)
            if ((uint32_t)g.cols[k] >= (uint32_t)g.n) { pool_release(p); return fail(DFQ_EFORMAT, "graph %d: column out of range", i); }
        p->n.push_back(g.n);
        p->e.push_back(g.e);
        const bool wide = g.e >= o.wide_min_edges && g.e >= (int64_t)o.wide_min_degree * g.n;
        p->wide.push_back(wide ? 1 : 0);
        // narrow cost estimate: edges plus levels times a per-level latency
        // in edge units; sparse graphs (average degree < 8) get ~2 sqrt(n) levels
        const double deg = (double)g.e / g.n;
        const double levels = deg < 8 ? 2.0 * std::sqrt((double)g.n) : std::log2((double)g.n + 2);
        p->cost.push_back((double)g.e + 4096.0 * levels);
        off_base[i] = tot_n;
        col_base[i] = tot_e;
        tot_n += (int64_t)g.n + 1;
        tot_e += ((g.e + 3) & ~(int64_t)3) + kColsPad;
    }
#define P_TRY(x) do { int rc_ = (x); if (rc_) { pool_release(p); return rc_; } } while (0)
#define P_CUDA(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { pool_release(p); return fail(DFQ_ECUDA, "%s: %s", #x, cudaGetErrorString(e_)); } } while (0)
    P_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    P_CUDA(cudaEventCreate(&p->ev0));
    P_CUDA(cudaEventCreate(&p->ev1));
    P_TRY(dmalloc(&p->offsets, sizeof(int32_t) * (size_t)tot_n));
    P_TRY(dmalloc(&p->cols, sizeof(int32_t) * (size_t)tot_e));
    P_CUDA(cudaMemsetAsync(p->cols, 0, sizeof(int32_t) * (size_t)tot_e, p->stream));
    for (int i = 0; i < ngraphs; ++i) {
        // wide graphs with skewed degrees are stored hub-first (as dfq_graph_create does)
        dfq_csr rg;
        memset(&rg, 0, sizeof rg);
        std::vector<int32_t> rank, order;
        int relabeled = 0;
        if (p->wide[i]) {
            relabeled = hub_first_csr(graphs[i], o.vertex_order, &rg, &rank, &order);
            if (relabeled < 0) { pool_release(p); return relabeled; }
        }
        const dfq_csr& g = relabeled ? rg : graphs[i];
        P_CUDA(cudaMemcpyAsync(p->offsets + off_base[i], g.offsets, sizeof(int32_t) * ((size_t)g.n + 1),
                               cudaMemcpyHostToDevice, p->stream));
        if (g.e) P_CUDA(cudaMemcpyAsync(p->cols + col_base[i], g.cols, sizeof(int32_t) * (size_t)g.e,
                                        cudaMemcpyHostToDevice, p->stream));
        const int32_t* d_rank = nullptr;
        const int32_t* d_order = nullptr;
        if (relabeled) {
            int32_t *a = nullptr, *b = nullptr;
            int rc = dmalloc(&a, sizeof(int32_t) * (size_t)g.n);
            if (rc == DFQ_OK) p->remap_arrays.push_back(a);
            if (rc == DFQ_OK) rc = dmalloc(&b, sizeof(int32_t) * (size_t)g.n);
            if (rc == DFQ_OK) p->remap_arrays.push_back(b);
            if (rc) { dfq_csr_free(&rg); pool_release(p); return rc; }
            cudaMemcpyAsync(a, rank.data(), sizeof(int32_t) * (size_t)g.n, cudaMemcpyHostToDevice, p->stream);
            cudaMemcpyAsync(b, order.data(), sizeof(int32_t) * (size_t)g.n, cudaMemcpyHostToDevice, p->stream);
            d_rank = a;
            d_order = b;
        }
        PoolGraph pg;
        pg.rank = d_rank;
        pg.order = d_order;
        pg.offsets = p->offsets + off_base[i];
        pg.cols = p->cols + col_base[i];
        pg.n = g.n;
        pg.wide = p->wide[i];
        pg.e = g.e;
        p->h_graphs.push_back(pg);
        const cudaError_t serr = cudaStreamSynchronize(p->stream);  // host arrays may be pageable / are freed now
        dfq_csr_free(&rg);
        P_CUDA(serr);
    }
    P_TRY(dmalloc(&p->d_graphs, sizeof(PoolGraph) * ngraphs));
    P_CUDA(cudaMemcpyAsync(p->d_graphs, p->h_graphs.data(), sizeof(PoolGraph) * ngraphs, cudaMemcpyHostToDevice,
                           p->stream));
    P_TRY(dmalloc(&p->d_misc, 256));
    P_TRY(dmalloc(&p->d_t0, 256));
    P_TRY(dmalloc(&p->d_ctl1, sizeof(Control)));
    P_CUDA(cudaMallocHost((void**)&p->h_t0, 64));
    P_CUDA(cudaMallocHost((void**)&p->h_ctl1, sizeof(Control)));
    P_CUDA(cudaStreamSynchronize(p->stream));
#undef P_TRY
#undef P_CUDA
    *out = p;
    return DFQ_OK;
}

int dfq_pool_destroy(dfq_pool* p) {
    clear_error();
    if (!p) return fail(DFQ_EINVAL, "dfq_pool_destroy: null pool");
    pool_release(p);
    return DFQ_OK;
}

int32_t dfq_pool_num_graphs(const dfq_pool* p) { return p ? p->ngraphs : -1; }

int dfq_pool_get_opts(const dfq_pool* p, dfq_opts* o) {
    clear_error();
    if (!p || !o) return fail(DFQ_EINVAL, "dfq_pool_get_opts: null argument");
    *o = p->opts;
    return DFQ_OK;
}

int dfq_pool_set_opts(dfq_pool* p, const dfq_opts* o) {
    clear_error();
    if (!p || !o) return fail(DFQ_EINVAL, "dfq_pool_set_opts: null argument");
    dfq_opts v = *o;
    if (v.wide_min_edges <= 0) v.wide_min_edges = 1 << 21;
    if (v.wide_min_degree <= 0) v.wide_min_degree = 8;
    if (v.block_threads == 0) v.block_threads = pool_block_threads(v);
    if (v.local_queue_cap == 0) v.local_queue_cap = 256;
    if (v.local_edge_budget == 0) v.local_edge_budget = 8192;
    if (v.timeout_ms == 0) v.timeout_ms = 5000;
    if (v.wide_min_edges != p->opts.wide_min_edges || v.wide_min_degree != p->opts.wide_min_degree ||
        v.vertex_order != p->opts.vertex_order)
        return fail(DFQ_EINVAL, "dfq_pool_set_opts: wide_min_edges, wide_min_degree and vertex_order are fixed at "
                    "pool creation (they decided how the graphs were stored)");
    if (v.direction != 0 || v.stall_test_level != 0)
        return fail(DFQ_EINVAL, "dfq_pool_set_opts: pools run top-down levels without test hooks");
    if (int rc = check_opts(v)) return rc;
    cudaSetDevice(p->device);
    cudaStreamSynchronize(p->stream);
    p->opts = v;
    if (p->gexec) {  // the captured launch baked in the old options
        cudaGraphExecDestroy(p->gexec);
        p->gexec = nullptr;
        p->g_nq = -1;
    }
    return DFQ_OK;
}

int dfq_pool_autotune(dfq_pool* p, const dfq_query* q, int32_t nq, dfq_opts* best) {
    clear_error();
    if (!p || !q || nq < 1 || !best) return fail(DFQ_EINVAL, "dfq_pool_autotune: bad arguments");
    dfq_opts cur = p->opts;
    const dfq_opts start = cur;
    // median of three timed batches (after one untimed) with options o; < 0 on failure
    auto time_batch = [&](const dfq_opts& o) -> double {
        if (dfq_pool_set_opts(p, &o) != DFQ_OK) return -1;
        float ms = 0;
        if (dfq_pool_batch(p, q, nq, 0, nullptr, &ms) != DFQ_OK) return -1;
        float t[3];
        for (float& x : t)
            if (dfq_pool_batch(p, q, nq, 0, nullptr, &x) != DFQ_OK) return -1;
        std::sort(t, t + 3);
        return t[1];
    };
    double best_t = time_batch(cur);
    if (best_t < 0) {
        dfq_pool_set_opts(p, &start);
        return fail(DFQ_ECUDA, "dfq_pool_autotune: baseline batch failed");
    }
    struct Axis { int32_t dfq_opts::*field; std::vector<int32_t> values; };
    // kernel options only: the wide split and the vertex order are the pool's
    const std::vector<Axis> axes = {
        {&dfq_opts::block_threads, {512, 1024}},
        {&dfq_opts::medium_min_degree, {16, 32, 64, 128}},
        {&dfq_opts::large_min_degree, {128, 256, 512, 1024}},
        {&dfq_opts::piece_edges, {256, 512}},
        {&dfq_opts::local_queue_cap, {256, 512}},
        {&dfq_opts::probe_first, {1, 2}},
        {&dfq_opts::use_tma, {0, 1}},
    };
    for (int pass = 0; pass < 2; ++pass) {
        bool improved = false;
        for (const Axis& ax : axes)
            for (int32_t v : ax.values) {
                if (cur.*ax.field == v) continue;
                dfq_opts t = cur;
                t.*ax.field = v;
                if (t.medium_min_degree > t.large_min_degree) t.medium_min_degree = t.large_min_degree;
                const double ms = time_batch(t);
                if (ms > 0 && ms < best_t * 0.98) { best_t = ms; cur = t; improved = true; }
            }
        if (!improved) break;
    }
    int rc = dfq_pool_set_opts(p, &cur);
    if (rc) return rc;
    *best = cur;
    return DFQ_OK;
}

int dfq_pool_graph_info(const dfq_pool* p, int32_t graph, int32_t* n, int64_t* e, int32_t* wide) {
    clear_error();
    if (!p || graph < 0 || graph >= p->ngraphs) return fail(DFQ_EINVAL, "dfq_pool_graph_info: bad graph");
    if (n) *n = p->n[graph];
    if (e) *e = p->e[graph];
    if (wide) *wide = p->wide[graph];
    return DFQ_OK;
}

int dfq_pool_bfs(dfq_pool* p, int32_t graph, int32_t src, int32_t* levels, int32_t* parents, dfq_stats* stats) {
    clear_error();
    if (!p || graph < 0 || graph >= p->ngraphs || !levels) return fail(DFQ_EINVAL, "dfq_pool_bfs: bad arguments");
    if (src < 0 || src >= p->n[graph]) return fail(DFQ_EINVAL, "source %d outside [0,%d)", src, p->n[graph]);
    cudaSetDevice(p->device);
    const bool par = parents != nullptr;
    int rc = ensure_wide(p, par);
    if (rc) return rc;
    const dfq_opts& o = p->opts;
    const void* fn = single_source_kernel(o.block_threads, par);
    if (!fn) return fail(DFQ_EINVAL, "block_threads %d", o.block_threads);
    const SmemLayout lay = smem_layout(o.block_threads, o.local_queue_cap, o.piece_edges, par);
    const int hot = hot_limit_words(o.hot_cache) > 0 ? hot_words_of(hot_limit_words(o.hot_cache), p->n[graph]) : 0;
    const int smem = lay.bytes + 4 * hot;
    int grid = 0;
    if ((rc = grid_for(p, fn, o.block_threads, smem, &grid))) return rc;
    const Workspace w = ws_from(p->wide_mem, p->wide_lay);
    Params prm;
    memset(&prm, 0, sizeof prm);
    prm.offsets = p->h_graphs[graph].offsets;
    prm.cols = p->h_graphs[graph].cols;
    prm.n = p->n[graph];
    prm.src = src;
    prm.levels = levels;
    prm.parents = parents;
    prm.bitmap = w.bitmap;
    prm.bitmap_words = (p->n[graph] + 31) / 32;
    for (int i = 0; i < 2; ++i) {
        prm.ovf[i] = w.ovf[i];
        prm.ovfv[i] = w.ovfv[i];
        prm.piece[i] = w.piece[i];
        prm.piece_v[i] = w.piece_v[i];
    }
    prm.piece_cap = w.piece_cap;
    prm.ovf_cap = p->n[graph];
    prm.ctl = p->d_ctl1;
    prm.medium_min = o.medium_min_degree;
    prm.large_min = o.large_min_degree;
    prm.piece_edges = o.piece_edges;
    prm.local_cap = o.local_queue_cap;
    prm.local_budget = o.local_edge_budget;
    prm.probe_first = o.probe_first;
    prm.use_tma = o.use_tma;
    prm.timeout_ns = (long long)o.timeout_ms * 1000000LL;
    prm.hot_words = hot;
    prm.tally_bar = grid < 1024 ? tally_bar_for(p->n[graph], p->e[graph]) : 0;
    remap_params(prm, p->h_graphs[graph], w);
    cudaEventRecord(p->ev0, p->stream);
    cudaMemsetAsync(p->d_ctl1, 0, sizeof(Control), p->stream);
    if ((rc = launch_coop(fn, grid, o.block_threads, smem, &prm, p->stream))) return rc;
    cudaEventRecord(p->ev1, p->stream);
    cudaMemcpyAsync(p->h_ctl1, p->d_ctl1, sizeof(Control), cudaMemcpyDeviceToHost, p->stream);
    cudaError_t err = cudaStreamSynchronize(p->stream);
    if (err != cudaSuccess) return fail(DFQ_ECUDA, "dfq_pool_bfs: %s", cudaGetErrorString(err));
    const Control& c = *p->h_ctl1;
    if (stats) {
        memset(stats, 0, sizeof *stats);
        float ms = 0;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        stats->kernel_ms = ms;
        stats->depth = c.stats.depth;
        stats->levels = c.stats.levels;
        stats->reached = (int64_t)c.stats.claims + 1;
        stats->edges = (int64_t)c.stats.edges;
        stats->overflow = (int64_t)c.stats.overflow;
        stats->large = (int64_t)c.stats.large;
    }
    return c.status ? fail(map_status(c.status), "dfq_pool_bfs: device status %d", c.status) : DFQ_OK;
}

int dfq_pool_batch(dfq_pool* p, const dfq_query* q, int32_t nq, int32_t flags, dfq_query_result* results,
                   float* total_ms) {
    clear_error();
    if (!p || (nq > 0 && !q) || nq < 0) return fail(DFQ_EINVAL, "dfq_pool_batch: bad arguments");
    if (nq == 0) { if (total_ms) *total_ms = 0; return DFQ_OK; }
    cudaSetDevice(p->device);
    const bool par = q[0].parents != nullptr;
    for (int i = 0; i < nq; ++i) {
        if (q[i].graph < 0 || q[i].graph >= p->ngraphs) return fail(DFQ_EINVAL, "query %d: graph %d", i, q[i].graph);
        if (q[i].source < 0 || q[i].source >= p->n[q[i].graph]) return fail(DFQ_EINVAL, "query %d: source", i);
        if (!q[i].levels) return fail(DFQ_EINVAL, "query %d: levels is null", i);
        if ((q[i].parents != nullptr) != par) return fail(DFQ_EINVAL, "parents must be given for all queries or none");
    }
    const dfq_opts& o = p->opts;
    const void* fn = pick_batch(o.block_threads, par);
    if (!fn) return fail(DFQ_EINVAL, "block_threads %d", o.block_threads);
    const SmemLayout lay = smem_layout(o.block_threads, o.local_queue_cap, o.piece_edges, par);
    // one cache size per pool (the largest graph's), so a captured launch
    // stays valid for any batch of the same shape
    int hot = 0;
    if (hot_limit_words(o.hot_cache) > 0)  // the cache only on request
        for (int i = 0; i < p->ngraphs; ++i) hot = std::max(hot, hot_words_of(hot_limit_words(o.hot_cache), p->n[i]));
    const int smem = lay.bytes + 4 * hot;
    int grid = 0, rc;
    if ((rc = grid_for(p, fn, o.block_threads, smem, &grid))) return rc;
    if ((rc = ensure_wide(p, par))) return rc;
    if ((rc = ensure_blocks(p, grid, par))) return rc;
    if ((rc = ensure_tables(p, nq))) return rc;
    // query table and lists (pinned staging, copied inside the launch sequence)
    int nw = 0, nn = 0;
    std::vector<int> narrow, ganged;
    for (int i = 0; i < nq; ++i) {
        BatchQuery& b = p->h_queries[i];
        b.graph = q[i].graph;
        b.source = q[i].source;
        b.levels = q[i].levels;
        b.parents = q[i].parents;
        b.t_start = b.t_end = 0;
        if (p->wide[q[i].graph]) p->h_lists[nw++] = i;
        else if (gang_graph(p, q[i].graph)) ganged.push_back(i);
        else narrow.push_back(i);
    }
    // gang size: the gang budget (half the grid) shared by the gang queries;
    // below 2 blocks per query they run narrow like the rest
    int gang_size = 0, n_gangs = 0;
    if (!ganged.empty()) {
        gang_size = std::min(kGangMax, (grid / 2) / (int)ganged.size());
        if (gang_size >= 2) {
            n_gangs = std::min<int>({(int)ganged.size(), (grid / 2) / gang_size, kGangsMax});
        } else {
            narrow.insert(narrow.end(), ganged.begin(), ganged.end());
            ganged.clear();
            gang_size = 0;
        }
    }
    auto by_cost = [&](int a, int b) { return p->cost[q[a].graph] > p->cost[q[b].graph]; };
    std::stable_sort(narrow.begin(), narrow.end(), by_cost);
    std::stable_sort(ganged.begin(), ganged.end(), by_cost);
    nn = (int)narrow.size();
    const int ng = (int)ganged.size();
    for (int k = 0; k < nn; ++k) p->h_lists[nq + k] = narrow[k];
    for (int k = 0; k < ng; ++k) p->h_lists[nq + nn + k] = ganged[k];
    if (n_gangs > 0 && (rc = ensure_gangs(p, n_gangs, par))) return rc;

    BatchParams bp;
    memset(&bp, 0, sizeof bp);
    bp.graphs = p->d_graphs;
    bp.queries = p->d_queries;
    bp.ctls = p->d_ctls;
    bp.wide_list = p->d_lists;
    bp.n_wide = nw;
    bp.narrow_list = p->d_lists + nq;
    bp.n_narrow = nn;
    bp.narrow_next = p->d_misc;
    bp.t0 = p->d_t0;
    bp.wide_ws = ws_from(p->wide_mem, p->wide_lay);
    bp.block_ws = p->block_mem;
    bp.block_ws_stride = p->block_stride;
    bp.block_lay = p->block_lay;
    bp.medium_min = o.medium_min_degree;
    bp.large_min = o.large_min_degree;
    bp.piece_edges = o.piece_edges;
    bp.local_cap = o.local_queue_cap;
    bp.local_budget = o.local_edge_budget;
    bp.probe_first = o.probe_first;
    bp.use_tma = o.use_tma;
    bp.timeout_ns = (long long)o.timeout_ms * 1000000LL;
    bp.hot_words = hot;
    // gangs: the last n_gangs * gang_size blocks
    bp.gang_list = p->d_lists + nq + nn;
    bp.n_gang = ng;
    bp.gang_next = p->d_misc + 1;
    bp.gang_word = reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(p->d_misc) + 64);
    bp.n_gangs = n_gangs;
    bp.gang_size = n_gangs > 0 ? gang_size : 1;
    bp.gang_ws = p->gang_mem;
    bp.gang_ws_stride = p->gang_stride;
    bp.gang_lay = p->gang_lay;
    // a sixth of the rest starts the narrow queries while the others run the
    // wide ones (when there are both; measured on the 256-graph pool: 1/16
    // 16.1k, 1/8 17.0-18.0k, 1/6 18.1k, 1/4 17.1k queries/s)
    const int gang_blocks = n_gangs * gang_size;
    const int rest = grid - gang_blocks;
    bp.reserve = gang_blocks + ((nw > 0 && nn > 0) ? std::min(nn, std::max(1, rest / 6)) : 0);

    auto enqueue = [&]() -> int {
        cudaError_t e1 = cudaMemcpyAsync(p->d_queries, p->h_queries, sizeof(BatchQuery) * nq, cudaMemcpyHostToDevice, p->stream);
        cudaError_t e2 = cudaMemcpyAsync(p->d_lists, p->h_lists, sizeof(int) * 2 * nq, cudaMemcpyHostToDevice, p->stream);
        cudaError_t e3 = cudaMemsetAsync(p->d_ctls, 0, sizeof(Control) * nq, p->stream);
        cudaError_t e4 = cudaMemsetAsync(p->d_misc, 0, 256, p->stream);
        if (e1 || e2 || e3 || e4) return fail(DFQ_ECUDA, "batch upload failed");
        return launch_coop(fn, grid, o.block_threads, smem, &bp, p->stream);
    };
    cudaEventRecord(p->ev0, p->stream);
    if (flags & DFQ_BATCH_GRAPH) {
        // the captured graph bakes in the kernel arguments: rebuild it when
        // the batch's shape changes, else replay it with new table contents
        if (!p->gexec || p->g_nq != nq || p->g_nwide != nw || p->g_par != (int)par || p->g_nnarrow != nn ||
            p->g_gangs != n_gangs || p->g_gang_size != gang_size) {
            if (p->gexec) { cudaGraphExecDestroy(p->gexec); p->gexec = nullptr; }
            cudaGraph_t graph = nullptr;
            cudaError_t err = cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal);
            if (err != cudaSuccess) return fail(DFQ_ECUDA, "begin capture: %s", cudaGetErrorString(err));
            int erc = enqueue();
            err = cudaStreamEndCapture(p->stream, &graph);
            if (erc) { if (graph) cudaGraphDestroy(graph); return erc; }
            if (err != cudaSuccess) return fail(DFQ_ECUDA, "end capture: %s", cudaGetErrorString(err));
            err = cudaGraphInstantiate(&p->gexec, graph, 0);
            cudaGraphDestroy(graph);
            if (err != cudaSuccess) { p->gexec = nullptr; return fail(DFQ_ECUDA, "instantiate: %s", cudaGetErrorString(err)); }
            p->g_nq = nq;
            p->g_nwide = nw;
            p->g_par = par;
            p->g_nnarrow = nn;
            p->g_gangs = n_gangs;
            p->g_gang_size = gang_size;
        }
        cudaError_t err = cudaGraphLaunch(p->gexec, p->stream);
        if (err != cudaSuccess) return fail(DFQ_ECUDA, "graph launch: %s", cudaGetErrorString(err));
    } else {
        if ((rc = enqueue())) return rc;
    }
    cudaEventRecord(p->ev1, p->stream);
    cudaMemcpyAsync(p->h_ctls, p->d_ctls, sizeof(Control) * nq, cudaMemcpyDeviceToHost, p->stream);
    cudaMemcpyAsync(p->h_queries, p->d_queries, sizeof(BatchQuery) * nq, cudaMemcpyDeviceToHost, p->stream);
    cudaMemcpyAsync(p->h_t0, p->d_t0, sizeof(long long), cudaMemcpyDeviceToHost, p->stream);
    cudaError_t err = cudaStreamSynchronize(p->stream);
    if (err != cudaSuccess) return fail(DFQ_ECUDA, "dfq_pool_batch: %s", cudaGetErrorString(err));
    if (total_ms) cudaEventElapsedTime(total_ms, p->ev0, p->ev1);
    int worst = DFQ_OK;
    for (int i = 0; i < nq; ++i) {
        const Control& c = p->h_ctls[i];
        const int st = map_status(c.status);
        if (st != DFQ_OK && worst == DFQ_OK) worst = st;
        if (results) {
            dfq_query_result& r = results[i];
            r.status = st;
            r.wide = p->wide[q[i].graph];
            r.depth = c.stats.depth;
            r.levels = c.stats.levels;
            r.reached = (int64_t)c.stats.claims + 1;
            r.edges = (int64_t)c.stats.edges;
            r.start_us = (double)(p->h_queries[i].t_start - *p->h_t0) * 1e-3;
            r.end_us = (double)(p->h_queries[i].t_end - *p->h_t0) * 1e-3;
        }
    }
    return worst == DFQ_OK ? DFQ_OK : fail(worst, "dfq_pool_batch: at least one query failed on the device");
}

}  // extern "C"
