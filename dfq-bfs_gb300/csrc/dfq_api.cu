// Host side of the libdfq C ABI: device-resident graphs, per-graph workspace,
// cooperative launch of the persistent DFQ kernel, statistics and errors.
//
// Replaces the reference host path of
// design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu:
//   :194-199,273-277  managed allocation + prefetch   -> dfq_graph_create
//   :255-268,283      occupancy-sized cooperative launch -> launch_bfs
//   :279-288          events around launch + sync      -> dfq_bfs (kernel_ms)
//   :290-300          Dist / Touch / Error             -> dfq_stats
#include "common.hpp"
#include "dfq_kernel.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

using namespace dfq;

#define CUDA_TRY(call)                                                                           \
    do {                                                                                         \
        cudaError_t err_ = (call);                                                               \
        if (err_ != cudaSuccess)                                                                 \
            return fail(DFQ_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(err_),    \
                        __FILE__, __LINE__);                                                     \
    } while (0)

struct dfq_graph {
    int device = 0;
    int sms = 0;
    int32_t n = 0;
    int64_t e = 0;
    dfq_opts opts{};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int32_t* offsets = nullptr;
    int32_t* cols = nullptr;
    // workspace
    int32_t* levels_tmp = nullptr;
    int32_t* parents_tmp = nullptr;
    unsigned* bitmap = nullptr;
    int bitmap_words = 0;
    int2* ovf[2] = {nullptr, nullptr};
    int32_t* ovfv[2] = {nullptr, nullptr};
    int2* piece[2] = {nullptr, nullptr};
    int32_t* piece_v[2] = {nullptr, nullptr};
    int piece_cap = 0;
    dfqk::Control* ctl = nullptr;
    dfqk::Control* ctl_host = nullptr;  // pinned copy for status / stats
    bool persist_set = false;
    // hub-first vertex order (when chosen at create): the device CSR uses new
    // ids, new id rank[v] for input id v, input id order[i] for new id i
    bool symmetric = false;  // checked at create when direction = 1 was asked for
    bool relabeled = false;
    std::vector<int32_t> rank_host;
    int32_t* rank = nullptr;
    int32_t* order = nullptr;
    int32_t* levels_int = nullptr;   // levels / parents by new id
    int32_t* parents_int = nullptr;
    unsigned* hub_claim = nullptr;   // claim words of the first hub_n (new) ids
    int hub_n = 0;
    // launch shape of the last launch (kernel, dynamic shared memory, blocks
    // per SM cap) and the occupancy grid it gave: recomputed only when one
    // changes (the kernel's shared-memory limit is still set every launch)
    const void* cfg_kernel = nullptr;
    int cfg_smem = -1, cfg_bps = -1, cfg_grid = 0;
    int cfg_cluster = 0;  // cluster size whose fit was checked for cfg_kernel / cfg_smem
};

namespace {

constexpr int kMinLargeDegree = 32;
constexpr int kMinPiece = 64;
constexpr int kColsPad = 32;

using KernelFn = void (*)(dfqk::Params);

KernelFn pick_kernel(int B, bool par) {
    switch (B) {
        case 256: return par ? dfqk::dfq_bfs_kernel<256, true> : dfqk::dfq_bfs_kernel<256, false>;
        case 512: return par ? dfqk::dfq_bfs_kernel<512, true> : dfqk::dfq_bfs_kernel<512, false>;
        case 1024: return par ? dfqk::dfq_bfs_kernel<1024, true> : dfqk::dfq_bfs_kernel<1024, false>;
        default: return nullptr;
    }
}

// block_threads = 0: 1024 for graphs of average degree below 8 (grids,
// meshes: thousands of small levels, where 152 blocks of 32 warps finish a
// level 5-7 % sooner than 304 blocks of 16, measured on the 4096^2 grid);
// 512 otherwise (equal on R-MAT, and smaller per-block layouts).
// The larger blocks only where their shared-memory layout (with parents and
// the requested hot cache) fits; else 512.
int auto_block_threads(int32_t n, int64_t e, const dfq_opts& o) {
    if (e >= 8 * (int64_t)n) return 512;
    const dfqk::SmemLayout L = dfqk::smem_layout(1024, o.local_queue_cap ? o.local_queue_cap : 256, o.piece_edges, true);
    const int need = L.bytes + (o.hot_cache > 0 ? 4 * dfqk::kHotWordsMax : 0);
    return need <= 227 * 1024 ? 1024 : 512;
}

int validate_opts(const dfq_opts& o) {
    if (o.block_threads != 256 && o.block_threads != 512 && o.block_threads != 1024)
        return fail(DFQ_EINVAL, "block_threads must be 256, 512 or 1024 (got %d)", o.block_threads);
    if (o.blocks_per_sm < 0 || o.blocks_per_sm > 8) return fail(DFQ_EINVAL, "blocks_per_sm must be in [0,8]");
    if (o.large_min_degree < kMinLargeDegree)
        return fail(DFQ_EINVAL, "large_min_degree must be >= %d", kMinLargeDegree);
    if (o.medium_min_degree < 1) return fail(DFQ_EINVAL, "medium_min_degree must be >= 1");
    if (o.piece_edges < kMinPiece || o.piece_edges % 64 || o.piece_edges > 16384)
        return fail(DFQ_EINVAL, "piece_edges must be a multiple of 64 in [64,16384]");
    if (o.local_queue_cap < 1 || o.local_queue_cap > 8192)
        return fail(DFQ_EINVAL, "local_queue_cap must be in [1,8192]");
    if (o.local_edge_budget < 0) return fail(DFQ_EINVAL, "local_edge_budget must be >= 0");
    if (o.timeout_ms < 1) return fail(DFQ_EINVAL, "timeout_ms must be >= 1");
    if (o.probe_first < 0 || o.probe_first > 2) return fail(DFQ_EINVAL, "probe_first must be 0, 1 or 2");
    if (o.hot_cache < -1 || o.hot_cache > 32) return fail(DFQ_EINVAL, "hot_cache must be -1, 0 or 1..32 (KB)");
    if (o.profile < 0) return fail(DFQ_EINVAL, "profile must be >= 0");
    if (o.direction != 0 && o.direction != 1) return fail(DFQ_EINVAL, "direction must be 0 or 1");
    if (o.stall_test_level < 0) return fail(DFQ_EINVAL, "stall_test_level must be >= 0");
    if (o.vertex_order < 0 || o.vertex_order > 2) return fail(DFQ_EINVAL, "vertex_order must be 0, 1 or 2");
    if (o.cluster_blocks != 0 && o.cluster_blocks != 2 && o.cluster_blocks != 4 && o.cluster_blocks != 8 &&
        o.cluster_blocks != 16)
        return fail(DFQ_EINVAL, "cluster_blocks must be 0, 2, 4, 8 or 16 (got %d)", o.cluster_blocks);
    const dfqk::SmemLayout L = dfqk::smem_layout(o.block_threads, o.local_queue_cap, o.piece_edges, true);
    const int need = L.bytes + (o.hot_cache > 0 ? 4 * dfqk::kHotWordsMax : 0);
    if (need > 227 * 1024)
        return fail(DFQ_EINVAL, "options need %d bytes of shared memory per block (max 232448)", need);
    return DFQ_OK;
}

template <class T>
int dev_alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t err = cudaMalloc((void**)p, sizeof(T) * count);
    if (err != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(err == cudaErrorMemoryAllocation ? DFQ_ENOMEM : DFQ_ECUDA,
                    "cudaMalloc of %zu bytes failed: %s", sizeof(T) * count, cudaGetErrorString(err));
    }
    return DFQ_OK;
}

bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device address of page-locked host memory mapped into device dev's address
// space (cudaHostAlloc / cudaHostRegister on that device, e.g. a pinned torch
// tensor), else null.  The kernel writes such output directly, so no separate
// copy follows; memory pinned through another device is copied instead.
int32_t* host_mapped(int32_t* p, int dev) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    if (a.type != cudaMemoryTypeHost || a.device != dev) return nullptr;
    return static_cast<int32_t*>(a.devicePointer);
}

__global__ void validate_csr_kernel(const int32_t* off, const int32_t* cols, int32_t n, int64_t e,
                                    int* bad) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < n; i += nth)
        if (off[i + 1] < off[i]) atomicCAS(bad, 0, 1);
    if (tid == 0 && (off[0] != 0 || (int64_t)off[n] != e)) atomicCAS(bad, 0, 2);
    for (int64_t k = tid; k < e; k += nth)
        if ((uint32_t)cols[k] >= (uint32_t)n) atomicCAS(bad, 0, 3);
}

// In-degree of every vertex (appearances in cols).
__global__ void indegree_kernel(const int32_t* __restrict__ cols, int64_t e, int32_t* __restrict__ indeg) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < e; k += nth) atomicAdd(&indeg[cols[k]], 1);
}

// Rows of the relabelled graph: new vertex i is input vertex order[i]; its
// neighbours are that row's, renamed through rank.  One warp per row.
__global__ void relabel_rows_kernel(const int32_t* __restrict__ off_in, const int32_t* __restrict__ cols_in,
                                    const int32_t* __restrict__ off_new, const int32_t* __restrict__ order,
                                    const int32_t* __restrict__ rank, int32_t n, int32_t* __restrict__ cols_new) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nw) {
        const int32_t o = order[i];
        const int32_t s0 = off_in[o], d = off_in[o + 1] - s0, t = off_new[i];
        int32_t best = INT32_MAX, at = -1;
        for (int32_t k = lane; k < d; k += 32) {
            const int32_t c = rank[cols_in[s0 + k]];
            cols_new[t + k] = c;
            if (c < best) { best = c; at = k; }
        }
        // the row's hub (smallest new id) first: a bottom-up search tries it first
        for (int off = 16; off > 0; off >>= 1) {
            const int32_t ob = __shfl_xor_sync(0xffffffffu, best, off);
            const int32_t oa = __shfl_xor_sync(0xffffffffu, at, off);
            if (ob < best || (ob == best && oa < at)) { best = ob; at = oa; }
        }
        __syncwarp();
        if (lane == 0 && at > 0) {
            cols_new[t + at] = cols_new[t];
            cols_new[t] = best;
        }
    }
}

// Undirected-graph check for direction-optimising BFS: every row sorted
// (flag bit 2 otherwise) and every edge u->v matched by v->u (bit 1
// otherwise, found by binary search in row v).  One warp per row.
__global__ void symmetric_check_kernel(const int32_t* __restrict__ off, const int32_t* __restrict__ cols, int32_t n,
                                       int* __restrict__ flag) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += nw) {
        const int32_t s0 = off[u], e0 = off[u + 1];
        for (int32_t k = s0 + lane; k < e0; k += 32) {
            const int32_t v = cols[k];
            if (k + 1 < e0 && cols[k + 1] < v) atomicOr(flag, 2);
            int32_t lo = off[v], hi = off[v + 1];
            const int32_t end = hi;
            while (lo < hi) {
                const int32_t mid = lo + ((hi - lo) >> 1);
                if (cols[mid] < (int32_t)u) lo = mid + 1;
                else hi = mid;
            }
            if (lo >= end || cols[lo] != (int32_t)u) atomicOr(flag, 1);
        }
    }
}

int map_device_status(const dfqk::Control& c) {
    switch (c.status) {
        case dfqk::kErrNone: return DFQ_OK;
        case dfqk::kErrBarrierTimeout:
            return fail(DFQ_ETIMEOUT, "grid barrier wait timed out (block %d, target %u)", c.err_info[0],
                        (unsigned)c.err_info[1]);
        case dfqk::kErrTmaTimeout:
            return fail(DFQ_ETIMEOUT, "bulk-copy wait timed out (block %d, edge %d)", c.err_info[0],
                        c.err_info[1]);
        case dfqk::kErrQueueCap:
            return fail(DFQ_EDEVICE, "queue capacity exceeded (index %d, capacity %d)", c.err_info[0],
                        c.err_info[1]);
        default: return fail(DFQ_EDEVICE, "device reported status %d", c.status);
    }
}

void release(dfq_graph* g) {
    if (!g) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    cudaFree(g->offsets);
    cudaFree(g->cols);
    cudaFree(g->levels_tmp);
    cudaFree(g->parents_tmp);
    cudaFree(g->bitmap);
    for (int i = 0; i < 2; ++i) {
        cudaFree(g->ovf[i]);
        cudaFree(g->ovfv[i]);
        cudaFree(g->piece[i]);
        cudaFree(g->piece_v[i]);
    }
    cudaFree(g->ctl);
    cudaFree(g->rank);
    cudaFree(g->order);
    cudaFree(g->levels_int);
    cudaFree(g->parents_int);
    cudaFree(g->hub_claim);
    if (g->ctl_host) cudaFreeHost(g->ctl_host);
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    if (g->stream) cudaStreamDestroy(g->stream);
    cudaSetDevice(prev);
    delete g;
}

int apply_persist(dfq_graph* g) {
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, g->device));
    cudaStreamAttrValue attr;
    memset(&attr, 0, sizeof attr);
    if (g->opts.l2_persist && prop.persistingL2CacheMaxSize > 0 && prop.accessPolicyMaxWindowSize > 0) {
        size_t bytes = sizeof(unsigned) * (size_t)g->bitmap_words;
        bytes = std::min(bytes, (size_t)prop.accessPolicyMaxWindowSize);
        size_t limit = std::min(bytes, (size_t)prop.persistingL2CacheMaxSize);
        CUDA_TRY(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, limit));
        attr.accessPolicyWindow.base_ptr = g->bitmap;
        attr.accessPolicyWindow.num_bytes = bytes;
        attr.accessPolicyWindow.hitRatio = 1.0f;
        attr.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        CUDA_TRY(cudaStreamSetAttribute(g->stream, cudaStreamAttributeAccessPolicyWindow, &attr));
        g->persist_set = true;
    } else if (g->persist_set) {
        attr.accessPolicyWindow.num_bytes = 0;
        CUDA_TRY(cudaStreamSetAttribute(g->stream, cudaStreamAttributeAccessPolicyWindow, &attr));
        g->persist_set = false;
    }
    return DFQ_OK;
}

// Hub-first order: input ids sorted by descending in-degree, ties by id
// (a stable counting sort), so the most-probed vertices get the smallest
// ids.  Chosen automatically when the graph has at least 2^16 vertices and
// its largest in-degree is at least 64 times the average.
bool want_hub_first(const std::vector<int32_t>& indeg, int32_t n, int64_t e, int mode) {
    if (mode == 1) return false;
    if (mode == 2) return true;
    if (n < (1 << 16)) return false;
    const int32_t mx = *std::max_element(indeg.begin(), indeg.end());
    return (double)mx >= 64.0 * ((double)e / (double)n);
}

void hub_first_order(const std::vector<int32_t>& indeg, int32_t n, std::vector<int32_t>& order) {
    const int32_t mx = *std::max_element(indeg.begin(), indeg.end());
    order.resize(n);
    if ((int64_t)mx <= 4 * (int64_t)n + 1024) {
        std::vector<int64_t> at((size_t)mx + 2, 0);  // at[k]: first slot of in-degree mx - k
        for (int32_t v = 0; v < n; ++v) at[(size_t)(mx - indeg[v]) + 1]++;
        for (size_t k = 1; k < at.size(); ++k) at[k] += at[k - 1];
        for (int32_t v = 0; v < n; ++v) order[at[(size_t)(mx - indeg[v])]++] = v;
    } else {
        for (int32_t v = 0; v < n; ++v) order[v] = v;
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return indeg[a] > indeg[b]; });
    }
}

// Rewrite g's device CSR in hub-first ids if the options and the graph call
// for it (g->offsets / g->cols hold the input CSR, validated).
int maybe_relabel(dfq_graph* g) {
    const int32_t n = g->n;
    const int64_t e = g->e;
    if (g->opts.vertex_order == 1 || e == 0) return DFQ_OK;
    int32_t* indeg_d = nullptr;
    int rc = dev_alloc(&indeg_d, (size_t)n);
    if (rc) return rc;
    std::vector<int32_t> indeg((size_t)n);
    cudaMemsetAsync(indeg_d, 0, sizeof(int32_t) * (size_t)n, g->stream);
    indegree_kernel<<<g->sms * 8, 256, 0, g->stream>>>(g->cols, e, indeg_d);
    cudaMemcpyAsync(indeg.data(), indeg_d, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, g->stream);
    cudaError_t err = cudaStreamSynchronize(g->stream);
    cudaFree(indeg_d);
    if (err != cudaSuccess) return fail(DFQ_ECUDA, "in-degree count: %s", cudaGetErrorString(err));
    if (!want_hub_first(indeg, n, e, g->opts.vertex_order)) return DFQ_OK;

    std::vector<int32_t> order, off_in((size_t)n + 1), off_new((size_t)n + 1);
    hub_first_order(indeg, n, order);
    std::vector<int32_t> rank((size_t)n);
    for (int32_t i = 0; i < n; ++i) rank[order[i]] = i;
    CUDA_TRY(cudaMemcpyAsync(off_in.data(), g->offsets, sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost,
                             g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    off_new[0] = 0;
    for (int32_t i = 0; i < n; ++i) off_new[i + 1] = off_new[i] + (off_in[order[i] + 1] - off_in[order[i]]);

    int32_t *off_d = nullptr, *cols_d = nullptr;
    if ((rc = dev_alloc(&g->rank, (size_t)n)) || (rc = dev_alloc(&g->order, (size_t)n)) ||
        (rc = dev_alloc(&g->levels_int, (size_t)n)) || (rc = dev_alloc(&off_d, (size_t)n + 1)) ||
        (rc = dev_alloc(&cols_d, (size_t)e + kColsPad))) {
        cudaFree(off_d);
        cudaFree(cols_d);
        return rc;
    }
    CUDA_TRY(cudaMemcpyAsync(g->rank, rank.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, g->stream));
    CUDA_TRY(cudaMemcpyAsync(g->order, order.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, g->stream));
    CUDA_TRY(cudaMemcpyAsync(off_d, off_new.data(), sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyHostToDevice,
                             g->stream));
    CUDA_TRY(cudaMemsetAsync(cols_d + e, 0, sizeof(int32_t) * kColsPad, g->stream));
    relabel_rows_kernel<<<g->sms * 8, 256, 0, g->stream>>>(g->offsets, g->cols, off_d, g->order, g->rank, n, cols_d);
    err = cudaStreamSynchronize(g->stream);
    if (err != cudaSuccess) {
        cudaFree(off_d);
        cudaFree(cols_d);
        return fail(DFQ_ECUDA, "relabel: %s", cudaGetErrorString(err));
    }
    cudaFree(g->offsets);
    cudaFree(g->cols);
    g->offsets = off_d;
    g->cols = cols_d;
    g->rank_host = std::move(rank);
    g->relabeled = true;
    // hubs (now the smallest ids) get claim words of their own
    g->hub_n = dfqk::hub_count(n);
    if ((rc = dev_alloc(&g->hub_claim, (size_t)g->hub_n * dfqk::kHubStride))) return rc;
    return DFQ_OK;
}

// direction = 1 at create: the input CSR must be undirected with sorted rows.
int check_symmetric(dfq_graph* g) {
    int* flag = nullptr;
    int rc = dev_alloc(&flag, 1);
    if (rc) return rc;
    int h = 0;
    cudaMemsetAsync(flag, 0, sizeof(int), g->stream);
    symmetric_check_kernel<<<g->sms * 8, 256, 0, g->stream>>>(g->offsets, g->cols, g->n, flag);
    cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, g->stream);
    cudaError_t err = cudaStreamSynchronize(g->stream);
    cudaFree(flag);
    if (err != cudaSuccess) return fail(DFQ_ECUDA, "symmetry check: %s", cudaGetErrorString(err));
    if (h & 2) return fail(DFQ_EINVAL, "direction = 1 needs sorted rows (sort and de-duplicate them, DFQ_CSR_DEDUP)");
    if (h & 1) return fail(DFQ_EINVAL, "direction = 1 needs an undirected graph: an edge u->v has no v->u");
    g->symmetric = true;
    return DFQ_OK;
}

// Shared-memory words of the hot-vertex cache for a graph of bitmap_words.
// hot_cache = K > 0: a cache of K KB (rounded down to 4 KB, at most 32 KB)
int hot_words_for(const dfq_opts& o, int n) {
    const int words = dfqk::hot_limit_words(o.hot_cache);
    return words > 0 ? dfqk::hot_words_of(words, n) : 0;
}

// Queue control-block reset + the cooperative kernel on g->stream.  The
// kernel computes into levels / parents (device); lv_host / pa_host, when
// given, are mapped host buffers that its last pass writes the results to.
int launch_bfs(dfq_graph* g, int32_t src, int32_t* levels, int32_t* parents, int32_t* lv_host = nullptr,
               int32_t* pa_host = nullptr) {
    const dfq_opts& o = g->opts;
    const bool par = parents != nullptr;
    KernelFn k = o.cluster_blocks > 1 ? (KernelFn)cluster_kernel(o.block_threads, par) : pick_kernel(o.block_threads, par);
    if (!k)
        return fail(DFQ_EINVAL, "no kernel for block_threads=%d%s", o.block_threads,
                    o.cluster_blocks > 1 ? " in a cluster (512 or 1024)" : "");
    const dfqk::SmemLayout lay = dfqk::smem_layout(o.block_threads, o.local_queue_cap, o.piece_edges, par);
    const int hot_words = hot_words_for(o, g->n);
    const int smem = lay.bytes + 4 * hot_words;
    // the limit is shared with every other caller of this kernel
    if (int rc = allow_dyn_smem((const void*)k, smem)) return rc;
    if ((const void*)k != g->cfg_kernel || smem != g->cfg_smem || o.blocks_per_sm != g->cfg_bps) {
        int per_sm = 0;
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k, o.block_threads, smem));
        if (per_sm < 1) return fail(DFQ_EINVAL, "kernel does not fit on an SM with these options");
        if (o.blocks_per_sm > 0) per_sm = std::min(per_sm, o.blocks_per_sm);
        g->cfg_kernel = (const void*)k;
        g->cfg_smem = smem;
        g->cfg_bps = o.blocks_per_sm;
        g->cfg_grid = g->sms * per_sm;
        g->cfg_cluster = 0;
    }
    const int grid = g->cfg_grid;

    dfqk::Params p;
    memset(&p, 0, sizeof p);
    p.offsets = g->offsets;
    p.cols = g->cols;
    p.n = g->n;
    p.src = src;
    p.levels = levels;
    p.parents = parents;
    p.bitmap = g->bitmap;
    p.bitmap_words = g->bitmap_words;
    for (int i = 0; i < 2; ++i) {
        p.ovf[i] = g->ovf[i];
        p.ovfv[i] = g->ovfv[i];
        p.piece[i] = g->piece[i];
        p.piece_v[i] = g->piece_v[i];
    }
    p.piece_cap = g->piece_cap;
    p.ovf_cap = g->n;
    p.ctl = g->ctl;
    p.medium_min = o.medium_min_degree;
    p.large_min = o.large_min_degree;
    p.piece_edges = o.piece_edges;
    p.local_cap = o.local_queue_cap;
    p.local_budget = o.local_edge_budget;
    p.probe_first = o.probe_first;
    p.use_tma = o.use_tma;
    p.timeout_ns = (long long)o.timeout_ms * 1000000LL;
    p.hot_words = hot_words;
    p.profile = o.profile ? 1 : 0;
    p.trace_from = (DFQ_CLAIM_PROBES && o.profile > 1) ? o.profile : 0;
    if (o.direction == 1 && !g->symmetric)
        return fail(DFQ_EINVAL, "direction = 1 needs a graph created with direction = 1 (checked undirected)");
    p.direction = o.direction;
    p.stall_level = o.stall_test_level;
    // levels end on the tally barrier when its 27-bit fields hold this graph's
    // totals exactly (fewer than 2^27 vertices and edges) and the grid's
    // arrivals fit its 10-bit count
    p.tally_bar = grid < 1024 ? dfqk::tally_bar_for(g->n, g->e) : 0;
    p.e = (int)g->e;
    if (g->relabeled) {
        if (par && !g->parents_int) {
            int rc = dev_alloc(&g->parents_int, (size_t)g->n);
            if (rc) return rc;
        }
        p.src = g->rank_host[src];
        p.levels = g->levels_int;
        p.parents = par ? g->parents_int : nullptr;
        p.levels_out = lv_host ? lv_host : levels;
        p.parents_out = pa_host ? pa_host : parents;
        p.rank = g->rank;
        p.order = g->order;
        p.hub_claim = g->hub_claim;
        p.hub_n = g->hub_n;
    } else {
        p.levels_out = lv_host;
        p.parents_out = pa_host;
    }

    CUDA_TRY(cudaMemsetAsync(g->ctl, 0, sizeof(dfqk::Control), g->stream));
    if (o.cluster_blocks > 1) {
        // one thread-block cluster runs the BFS (its blocks are co-scheduled
        // by the hardware, so no cooperative launch is needed)
        const int C = o.cluster_blocks;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)C;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3((unsigned)C);
        cfg.blockDim = dim3((unsigned)o.block_threads);
        cfg.dynamicSmemBytes = (size_t)smem;
        cfg.stream = g->stream;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (g->cfg_cluster != C) {
            if (C > 8) CUDA_TRY(cudaFuncSetAttribute((const void*)k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
            int fits = 0;
            CUDA_TRY(cudaOccupancyMaxActiveClusters(&fits, (const void*)k, &cfg));
            if (fits < 1)
                return fail(DFQ_EINVAL, "a cluster of %d blocks of %d threads with %d bytes of shared memory does not fit",
                            C, o.block_threads, smem);
            g->cfg_cluster = C;
        }
        CUDA_TRY(cudaLaunchKernelEx(&cfg, k, p));
        return DFQ_OK;
    }
    void* args[] = {&p};
    CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k, dim3(grid), dim3(o.block_threads), args, smem, g->stream));
    return DFQ_OK;
}

// Status and statistics of the last launch (full: the per-level traces too).
int fill_stats(dfq_graph* g, dfq_stats* st, bool full = false) {
    const size_t bytes = full ? sizeof(dfqk::Control) : offsetof(dfqk::Control, trace_ns);
    CUDA_TRY(cudaMemcpyAsync(g->ctl_host, g->ctl, bytes, cudaMemcpyDeviceToHost, g->stream));
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    const dfqk::Control& c = *g->ctl_host;
    if (st) {
        st->depth = c.stats.depth;
        st->levels = c.stats.levels;
        st->reached = (int64_t)c.stats.claims + 1;
        st->edges = (int64_t)c.stats.edges;
        st->overflow = (int64_t)c.stats.overflow;
        st->large = (int64_t)c.stats.large;
    }
    return map_device_status(c);
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

namespace dfq {
int allow_dyn_smem(const void* fn, int smem_needed) {
    // The limit only ever rises (per kernel and device, under one lock): a
    // limit above what a launch uses costs nothing, while lowering it could
    // fail another host thread's launch that set a larger value just before.
    static std::mutex mu;
    static std::vector<std::pair<std::pair<const void*, int>, int>> set_to;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    for (auto& kv : set_to)
        if (kv.first.first == fn && kv.first.second == dev) {
            if (kv.second >= smem_needed) return DFQ_OK;
            cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_needed);
            if (err != cudaSuccess) return fail(DFQ_ECUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(err));
            kv.second = smem_needed;
            return DFQ_OK;
        }
    cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_needed);
    if (err != cudaSuccess) return fail(DFQ_ECUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(err));
    set_to.push_back({{fn, dev}, smem_needed});
    return DFQ_OK;
}

int device_status(const dfqk::Control& c) { return map_device_status(c); }

int check_opts(const dfq_opts& o) { return validate_opts(o); }

const void* single_source_kernel(int block_threads, bool par) {
    return (const void*)pick_kernel(block_threads, par);
}
}  // namespace dfq

extern "C" {

void dfq_opts_default(dfq_opts* o) {
    if (!o) return;
    o->block_threads = 0;  // chosen per graph at create (auto_block_threads)
    o->blocks_per_sm = 0;
    o->medium_min_degree = 64;
    o->large_min_degree = 256;
    o->local_queue_cap = 256;
    o->local_edge_budget = 8192;
    o->piece_edges = 256;
    o->probe_first = 2;
    o->l2_persist = 0;
    o->use_tma = 1;
    o->timeout_ms = 5000;
    o->wide_min_edges = 1 << 21;
    o->wide_min_degree = 8;
    o->hot_cache = 0;
    o->vertex_order = 0;
    o->profile = 0;
    o->direction = 0;
    o->stall_test_level = 0;
    o->cluster_blocks = 0;
}

int dfq_graph_create(const int32_t* offsets, const int32_t* cols, int32_t n, int64_t e, const dfq_opts* opts,
                     dfq_graph** out) {
    clear_error();
    if (!out) return fail(DFQ_EINVAL, "dfq_graph_create: out is null");
    *out = nullptr;
    if (!offsets || (e > 0 && !cols) || n < 1 || e < 0 || e >= ((int64_t)1 << 31))
        return fail(DFQ_EINVAL, "dfq_graph_create: need offsets, cols, 1 <= n, 0 <= e < 2^31");
    dfq_opts o;
    dfq_opts_default(&o);
    if (opts) o = *opts;
    if (o.block_threads == 0) o.block_threads = auto_block_threads(n, e, o);
    if (o.local_queue_cap == 0) o.local_queue_cap = 256;
    if (o.local_edge_budget == 0) o.local_edge_budget = 8192;
    if (o.timeout_ms == 0) o.timeout_ms = 5000;
    int rc = validate_opts(o);
    if (rc) return rc;

    const bool dev_in = is_device_ptr(offsets);
    if (!dev_in) {  // host input: validate here (the reference validates nothing)
        if (offsets[0] != 0 || (int64_t)offsets[n] != e)
            return fail(DFQ_EFORMAT, "offsets[0] must be 0 and offsets[n] must equal e");
        for (int32_t u = 0; u < n; ++u)
            if (offsets[u + 1] < offsets[u]) return fail(DFQ_EFORMAT, "offsets decrease at vertex %d", u);
        for (int64_t k = 0; k < e; ++k)
            if ((uint32_t)cols[k] >= (uint32_t)n)
                return fail(DFQ_EFORMAT, "cols[%lld] = %d outside [0,%d)", (long long)k, cols[k], n);
    }

    dfq_graph* g = new dfq_graph();
    g->n = n;
    g->e = e;
    g->opts = o;
    cudaGetDevice(&g->device);
    cudaDeviceProp prop;
    cudaError_t err = cudaGetDeviceProperties(&prop, g->device);
    if (err != cudaSuccess) { release(g); return fail(DFQ_ECUDA, "no CUDA device: %s", cudaGetErrorString(err)); }
    if (!prop.cooperativeLaunch) { release(g); return fail(DFQ_ECUDA, "device does not support cooperative launch"); }
    g->sms = prop.multiProcessorCount;
#define G_TRY(x) do { int rc_ = (x); if (rc_) { release(g); return rc_; } } while (0)
#define G_CUDA(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { release(g); return fail(DFQ_ECUDA, "%s: %s", #x, cudaGetErrorString(e_)); } } while (0)
    G_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    G_CUDA(cudaEventCreate(&g->ev0));
    G_CUDA(cudaEventCreate(&g->ev1));
    G_TRY(dev_alloc(&g->offsets, (size_t)n + 1));
    G_TRY(dev_alloc(&g->cols, (size_t)e + kColsPad));
    const cudaMemcpyKind kind = dev_in ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    G_CUDA(cudaMemcpyAsync(g->offsets, offsets, sizeof(int32_t) * ((size_t)n + 1), kind, g->stream));
    if (e > 0) G_CUDA(cudaMemcpyAsync(g->cols, cols, sizeof(int32_t) * (size_t)e, kind, g->stream));
    G_CUDA(cudaMemsetAsync(g->cols + e, 0, sizeof(int32_t) * kColsPad, g->stream));

    g->bitmap_words = (int)(((int64_t)n + 31) / 32);
    G_TRY(dev_alloc(&g->bitmap, ((size_t)g->bitmap_words + 31) & ~(size_t)31));
    G_TRY(dev_alloc(&g->levels_tmp, (size_t)n));
    g->piece_cap = dfqk::piece_capacity(n, e, kMinLargeDegree, kMinPiece);
    for (int i = 0; i < 2; ++i) {
        G_TRY(dev_alloc(&g->ovf[i], (size_t)n));
        G_TRY(dev_alloc(&g->ovfv[i], (size_t)n));
        G_TRY(dev_alloc(&g->piece[i], (size_t)g->piece_cap));
        G_TRY(dev_alloc(&g->piece_v[i], (size_t)g->piece_cap));
    }
    G_TRY(dev_alloc(&g->ctl, 1));
    G_CUDA(cudaMallocHost((void**)&g->ctl_host, sizeof(dfqk::Control)));
    memset(g->ctl_host, 0, sizeof(dfqk::Control));

    if (dev_in) {
        int* bad = nullptr;
        G_TRY(dev_alloc(&bad, 1));
        cudaMemsetAsync(bad, 0, sizeof(int), g->stream);
        validate_csr_kernel<<<g->sms * 4, 256, 0, g->stream>>>(g->offsets, g->cols, n, e, bad);
        int hbad = 0;
        cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, g->stream);
        cudaError_t e2 = cudaStreamSynchronize(g->stream);
        cudaFree(bad);
        if (e2 != cudaSuccess) { release(g); return fail(DFQ_ECUDA, "CSR validation: %s", cudaGetErrorString(e2)); }
        if (hbad) {
            release(g);
            return fail(DFQ_EFORMAT, hbad == 1 ? "offsets decrease" : hbad == 2 ? "offsets[0] != 0 or offsets[n] != e"
                                                                                  : "a column index is outside [0,n)");
        }
    }
    if (o.direction == 1) G_TRY(check_symmetric(g));
    G_TRY(maybe_relabel(g));
    G_TRY(apply_persist(g));
    G_CUDA(cudaStreamSynchronize(g->stream));
#undef G_TRY
#undef G_CUDA
    *out = g;
    return DFQ_OK;
}

int dfq_graph_destroy(dfq_graph* g) {
    clear_error();
    if (!g) return fail(DFQ_EINVAL, "dfq_graph_destroy: null graph");
    release(g);
    return DFQ_OK;
}

int dfq_graph_get_opts(const dfq_graph* g, dfq_opts* o) {
    clear_error();
    if (!g || !o) return fail(DFQ_EINVAL, "dfq_graph_get_opts: null argument");
    *o = g->opts;
    return DFQ_OK;
}

int dfq_graph_set_opts(dfq_graph* g, const dfq_opts* o) {
    clear_error();
    if (!g || !o) return fail(DFQ_EINVAL, "dfq_graph_set_opts: null argument");
    dfq_opts v = *o;
    if (v.block_threads == 0) v.block_threads = auto_block_threads(g->n, g->e, v);
    if (v.local_queue_cap == 0) v.local_queue_cap = 256;
    if (v.local_edge_budget == 0) v.local_edge_budget = 8192;
    if (v.timeout_ms == 0) v.timeout_ms = 5000;
    int rc = validate_opts(v);
    if (rc) return rc;
    DeviceGuard dg(g->device);
    g->opts = v;
    return apply_persist(g);
}

void* dfq_graph_stream(dfq_graph* g) { return g ? (void*)g->stream : nullptr; }

int32_t dfq_graph_num_vertices(const dfq_graph* g) { return g ? g->n : -1; }
int32_t dfq_graph_is_hub_first(const dfq_graph* g) { return g ? (g->relabeled ? 1 : 0) : -1; }
int64_t dfq_graph_num_edges(const dfq_graph* g) { return g ? g->e : -1; }

int dfq_bfs_launch(dfq_graph* g, int32_t src, int32_t* levels_dev, int32_t* parents_dev) {
    clear_error();
    if (!g || !levels_dev) return fail(DFQ_EINVAL, "dfq_bfs_launch: null argument");
    if (src < 0 || src >= g->n) return fail(DFQ_EINVAL, "source %d outside [0,%d)", src, g->n);
    DeviceGuard dg(g->device);
    return launch_bfs(g, src, levels_dev, parents_dev);
}

int dfq_graph_sync(dfq_graph* g) {
    clear_error();
    if (!g) return fail(DFQ_EINVAL, "dfq_graph_sync: null graph");
    DeviceGuard dg(g->device);
    return fill_stats(g, nullptr);
}

int dfq_bfs_last_stats(dfq_graph* g, dfq_stats* st) {
    clear_error();
    if (!g || !st) return fail(DFQ_EINVAL, "dfq_bfs_last_stats: null argument");
    DeviceGuard dg(g->device);
    memset(st, 0, sizeof *st);
    return fill_stats(g, st);
}

int dfq_bfs_last_trace(dfq_graph* g, int64_t* start_ns, int32_t* frontier, int32_t max_levels) {
    clear_error();
    if (!g || max_levels < 0 || (max_levels > 0 && (!start_ns || !frontier)))
        return fail(DFQ_EINVAL, "dfq_bfs_last_trace: bad arguments");
    DeviceGuard dg(g->device);
    int rc = fill_stats(g, nullptr, true);
    if (rc) return rc;
    const dfqk::Control& c = *g->ctl_host;
    const int from = (DFQ_CLAIM_PROBES && g->opts.profile > 1) ? g->opts.profile : 0;
    int n = std::min(std::min(max_levels, dfqk::kTraceLevels), std::max(c.stats.levels + 1 - from, 0));
    for (int i = 0; i < n; ++i) {
        start_ns[i] = c.trace_ns[i];
        frontier[i] = c.trace_frontier[i];
    }
    return n;
}

int dfq_bfs_last_levels(dfq_graph* g, dfq_level_info* out, int32_t max_levels) {
    clear_error();
    if (!g || max_levels < 0 || (max_levels > 0 && !out))
        return fail(DFQ_EINVAL, "dfq_bfs_last_levels: bad arguments");
    DeviceGuard dg(g->device);
    int rc = fill_stats(g, nullptr, true);
    if (rc) return rc;
    const dfqk::Control& c = *g->ctl_host;
    const int from = (DFQ_CLAIM_PROBES && g->opts.profile > 1) ? g->opts.profile : 0;
    int n = std::min(std::min(max_levels, dfqk::kTraceLevels), std::max(c.stats.levels + 1 - from, 0));
    for (int i = 0; i < n; ++i) {
        dfq_level_info& o = out[i];
        memset(&o, 0, sizeof o);
        o.level = from + i;
        for (int k = 0; k < 4; ++k) o.claim_ns[k] = (int32_t)c.trace_claim[i][k];
        for (int k = 0; k < 4; ++k) o.piece_stats[k] = (int64_t)c.trace_piece[i][k];
        o.start_ns = c.trace_ns[i];
        o.frontier = c.trace_frontier[i];
        o.edges = c.trace_edges[i];
        o.overflow = c.trace_ovf[i];
        o.pieces = c.trace_pieces[i];
        o.probe = c.trace_probe[i];
        o.last_done_ns = (int64_t)c.trace_done_last[i];
        o.first_done_ns = c.trace_done_first[i] ? (int64_t)~c.trace_done_first[i] : 0;
        for (int k = 0; k < 4; ++k) o.phase_ns[k] = (int32_t)c.trace_phase[i][k];
    }
    return n;
}

int dfq_bfs(dfq_graph* g, int32_t src, int32_t* levels, int32_t* parents, dfq_stats* stats) {
    clear_error();
    if (!g || !levels) return fail(DFQ_EINVAL, "dfq_bfs: graph and levels are required");
    if (src < 0 || src >= g->n) return fail(DFQ_EINVAL, "source %d outside [0,%d)", src, g->n);
    DeviceGuard dg(g->device);
    const bool lv_dev = is_device_ptr(levels);
    const bool pa_dev = parents && is_device_ptr(parents);
    // pinned host outputs are written by the kernel itself; other host
    // outputs are copied from device scratch after it
    int32_t* lv_map = lv_dev ? nullptr : host_mapped(levels, g->device);
    int32_t* pa_map = (parents && !pa_dev) ? host_mapped(parents, g->device) : nullptr;
    int32_t* dl = lv_dev ? levels : g->levels_tmp;
    int32_t* dp = nullptr;
    if (parents) {
        if (pa_dev) dp = parents;
        else {
            if (!g->parents_tmp) {
                int rc = dev_alloc(&g->parents_tmp, (size_t)g->n);
                if (rc) return rc;
            }
            dp = g->parents_tmp;
        }
    }
    CUDA_TRY(cudaEventRecord(g->ev0, g->stream));
    int rc = launch_bfs(g, src, dl, dp, lv_map, pa_map);
    if (rc) return rc;
    CUDA_TRY(cudaEventRecord(g->ev1, g->stream));
    if (!lv_dev && !lv_map)
        CUDA_TRY(cudaMemcpyAsync(levels, dl, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToHost, g->stream));
    if (parents && !pa_dev && !pa_map)
        CUDA_TRY(cudaMemcpyAsync(parents, dp, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToHost, g->stream));
    dfq_stats st;
    memset(&st, 0, sizeof st);
    rc = fill_stats(g, &st);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, g->ev0, g->ev1);
    st.kernel_ms = ms;
    if (stats) *stats = st;
    return rc;
}

}  // extern "C"
