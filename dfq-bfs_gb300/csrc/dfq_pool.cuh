// Device-resident graph pools: types and host helpers shared by the batch
// (dfq_batch.cu) and serving (dfq_serve.cu) layers.
#pragma once
#include "common.hpp"
#include "dfq_kernel.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

namespace dfqk {

struct PoolGraph {
    const int* offsets;
    const int* cols;
    int n;
    int wide;
    long long e;
    const int* rank;   // hub-first renumbered graph: new id of each input id (else null)
    const int* order;  //   and input id of each new id
};

// One query as the device sees it; start/end written by the kernel.
struct BatchQuery {
    int graph;
    int source;
    int* levels;
    int* parents;
    long long t_start;
    long long t_end;
};

// BFS workspace: queues, bitmap and capacities for graphs up to n vertices.
struct Workspace {
    unsigned* bitmap;
    int2* ovf[2];
    int* ovfv[2];
    int2* piece[2];
    int* piece_v[2];
    int piece_cap;
    int* levels_int;      // renumbered graphs: levels / parents by new id (else null)
    int* parents_int;
    unsigned* hub_claim;  //   and the hubs' claim words
};

// Byte layout of one workspace for graphs up to n vertices and e edges.
struct WsLayout {
    size_t bitmap, ovf[2], ovfv[2], piece[2], piece_v[2], levels_int, parents_int, hub_claim, total;
    int piece_cap;
    bool remap;
};

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }
// remap: room for a renumbered graph's levels / parents by new id and hub claim words
inline WsLayout ws_layout(long long n, long long e, int min_large, int min_piece, bool par, bool remap = false) {
    WsLayout w;
    size_t o = 0;
    w.remap = remap;
    w.bitmap = o;  o = al256(o + 4 * (size_t)(((n + 31) / 32 + 31) & ~31LL));
    w.piece_cap = piece_capacity(n, e, min_large, min_piece);
    for (int i = 0; i < 2; ++i) { w.ovf[i] = o;   o = al256(o + 8 * (size_t)std::max<long long>(n, 1)); }
    for (int i = 0; i < 2; ++i) { w.ovfv[i] = o;  o = al256(o + (par ? 4 * (size_t)std::max<long long>(n, 1) : 256)); }
    for (int i = 0; i < 2; ++i) { w.piece[i] = o;   o = al256(o + 8 * (size_t)w.piece_cap); }
    for (int i = 0; i < 2; ++i) { w.piece_v[i] = o; o = al256(o + (par ? 4 * (size_t)w.piece_cap : 256)); }
    w.levels_int = o; o = al256(o + (remap ? 4 * (size_t)std::max<long long>(n, 1) : 256));
    w.parents_int = o; o = al256(o + (remap && par ? 4 * (size_t)std::max<long long>(n, 1) : 256));
    w.hub_claim = o;  o = al256(o + (remap ? 4 * (size_t)kHubStride * kHubIds : 256));
    w.total = o;
    return w;
}

// A query on a renumbered graph (g.rank != null) in a workspace with room for
// it: the kernel runs on new ids into the workspace's arrays and writes the
// caller's levels / parents in input ids at the end.
__host__ __device__ inline void remap_params(Params& sp, const PoolGraph& g, const Workspace& ws) {
    if (!g.rank || !ws.levels_int) return;
    sp.levels_out = sp.levels;
    sp.parents_out = sp.parents;
    sp.levels = ws.levels_int;
    sp.parents = sp.parents ? ws.parents_int : nullptr;
    sp.rank = g.rank;
    sp.order = g.order;
    sp.map_src = 1;
    sp.hub_claim = ws.hub_claim;
    sp.hub_n = hub_count(g.n);
}

}  // namespace dfqk

// The pool handle of include/dfq.h.
struct dfq_pool {
    using Control = dfqk::Control;
    using BatchQuery = dfqk::BatchQuery;
    using WsLayout = dfqk::WsLayout;
    using PoolGraph = dfqk::PoolGraph;
    int device = 0;
    int sms = 0;
    dfq_opts opts{};
    int32_t ngraphs = 0;
    std::vector<int32_t> n;
    std::vector<int64_t> e;
    std::vector<int32_t> wide;
    std::vector<double> cost;
    int32_t* offsets = nullptr;  // packed
    int32_t* cols = nullptr;     // packed, each graph 16-byte aligned and padded
    PoolGraph* d_graphs = nullptr;
    std::vector<PoolGraph> h_graphs;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // whole-grid workspace (largest graph) and per-block workspaces (largest narrow graph)
    unsigned char* wide_mem = nullptr;
    WsLayout wide_lay{};
    bool wide_par = false;
    unsigned char* block_mem = nullptr;
    size_t block_stride = 0;
    WsLayout block_lay{};
    int block_grid = 0;
    int block_n = 0;
    bool block_par = false;
    // batch tables
    BatchQuery* d_queries = nullptr;
    BatchQuery* h_queries = nullptr;  // pinned
    int* d_lists = nullptr;
    int* h_lists = nullptr;           // pinned: wide list then narrow list
    Control* d_ctls = nullptr;
    Control* h_ctls = nullptr;        // pinned
    int* d_misc = nullptr;            // narrow cursor
    long long* d_t0 = nullptr;
    long long* h_t0 = nullptr;
    int qcap = 0;
    // captured batch
    cudaGraphExec_t gexec = nullptr;
    int g_nq = -1, g_nwide = -1, g_par = -1, g_nnarrow = -1, g_gangs = -1, g_gang_size = -1;
    // gang workspaces (largest gang graph), gang_count of them
    unsigned char* gang_mem = nullptr;
    size_t gang_stride = 0;
    WsLayout gang_lay{};
    int gang_count = 0;
    bool gang_par = false;
    // single-query launches
    Control* d_ctl1 = nullptr;
    Control* h_ctl1 = nullptr;
    std::vector<int32_t*> remap_arrays;  // rank / order of the renumbered graphs
};

namespace dfqpool {

using namespace dfq;
using namespace dfqk;

constexpr int kMinLarge = 32, kMinPiece = 64, kColsPad = 32;

template <class T>
inline int dmalloc(T** p, size_t bytes) {
    *p = nullptr;
    cudaError_t err = cudaMalloc((void**)p, bytes ? bytes : 16);
    if (err != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(err == cudaErrorMemoryAllocation ? DFQ_ENOMEM : DFQ_ECUDA, "cudaMalloc(%zu): %s", bytes,
                    cudaGetErrorString(err));
    }
    return DFQ_OK;
}

inline void pool_release(dfq_pool* p) {
    if (!p) return;
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    cudaFree(p->offsets);
    cudaFree(p->cols);
    cudaFree(p->d_graphs);
    cudaFree(p->wide_mem);
    cudaFree(p->block_mem);
    cudaFree(p->gang_mem);
    cudaFree(p->d_queries);
    cudaFree(p->d_lists);
    cudaFree(p->d_ctls);
    cudaFree(p->d_misc);
    cudaFree(p->d_t0);
    cudaFree(p->d_ctl1);
    for (int32_t* a : p->remap_arrays) cudaFree(a);
    if (p->h_queries) cudaFreeHost(p->h_queries);
    if (p->h_lists) cudaFreeHost(p->h_lists);
    if (p->h_ctls) cudaFreeHost(p->h_ctls);
    if (p->h_t0) cudaFreeHost(p->h_t0);
    if (p->h_ctl1) cudaFreeHost(p->h_ctl1);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

inline Workspace ws_from(unsigned char* base, const WsLayout& l) {
    Workspace w;
    w.bitmap = (unsigned*)(base + l.bitmap);
    for (int i = 0; i < 2; ++i) {
        w.ovf[i] = (int2*)(base + l.ovf[i]);
        w.ovfv[i] = (int*)(base + l.ovfv[i]);
        w.piece[i] = (int2*)(base + l.piece[i]);
        w.piece_v[i] = (int*)(base + l.piece_v[i]);
    }
    w.piece_cap = l.piece_cap;
    w.levels_int = l.remap ? (int*)(base + l.levels_int) : nullptr;
    w.parents_int = l.remap ? (int*)(base + l.parents_int) : nullptr;
    w.hub_claim = l.remap ? (unsigned*)(base + l.hub_claim) : nullptr;
    return w;
}

// (Re)allocate the whole-grid workspace for the largest graph, with parent
// ids if asked.
inline int ensure_wide(dfq_pool* p, bool par) {
    if (p->wide_mem && (p->wide_par || !par)) return DFQ_OK;
    cudaFree(p->wide_mem);
    p->wide_mem = nullptr;
    long long nmax = 1, emax = 0;
    for (int i = 0; i < p->ngraphs; ++i) { nmax = std::max<long long>(nmax, p->n[i]); emax = std::max<long long>(emax, p->e[i]); }
    bool remap = false;
    for (const PoolGraph& g : p->h_graphs) remap = remap || g.rank != nullptr;
    p->wide_lay = ws_layout(nmax, emax, kMinLarge, kMinPiece, par, remap);
    p->wide_par = par;
    return dmalloc(&p->wide_mem, p->wide_lay.total);
}

inline int grid_for(dfq_pool* p, const void* fn, int B, int smem, int* grid) {
    if (int rc = allow_dyn_smem(fn, smem)) return rc;
    int per_sm = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, B, smem);
    if (err != cudaSuccess || per_sm < 1)
        return fail(DFQ_ECUDA, "kernel does not fit: %s", cudaGetErrorString(err));
    if (p->opts.blocks_per_sm > 0) per_sm = std::min(per_sm, p->opts.blocks_per_sm);
    *grid = p->sms * per_sm;
    return DFQ_OK;
}

}  // namespace dfqpool
