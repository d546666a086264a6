// dfq_bfs_noalloc: single-source BFS that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host framework that owns all of the
// GPU's memory through its own pool (an allocation from a plug-in would fail
// against that pool or fragment it), a serving process that reserves its HBM
// budget at start-up and allows no allocation afterwards, or a caller that
// cannot accept cudaMalloc/cudaFree stalling every stream on the device.
// dfq_graph_create allocates a per-graph workspace, so those callers get this
// entry point instead: they pass the CSR and the output arrays (device
// memory they already own) and the kernel's scratch - visited bitmap,
// frontier queues, control block - comes from one fixed array in this file.
//
// The scratch array is a file-scope static __device__ array of
// DFQ_NOALLOC_SCRATCH_BYTES: every GPU that loads libdfq holds it until the
// process exits.  Graphs whose scratch would exceed it are rejected with
// DFQ_ENOMEM before anything is launched.  All calls on a device share the one
// array and it keeps the previous call's contents; each call clears the
// control block and the kernel re-initialises the bitmap and levels, and queue
// slots are written before they are read.  Calls whose work overlaps on the
// GPU (different streams or host threads without ordering) race on the array.
//
// No cudaMalloc, cudaFree or allocating library routine is called on this
// path.  The first call on each device looks up the array's device address
// with cudaGetSymbolAddress (host code cannot use the array's name as a device
// pointer) and caches it with the kernel's launch shape; make that first call
// before any stream capture.
//
// Cost: every call first checks the caller's CSR on the device (one pass over
// the n + 1 offsets and the e columns, about 4 bytes per edge) and waits for
// that check before the traversal, whose algorithmic traffic is also about 4
// bytes per edge, so a call moves up to twice the bytes of dfq_bfs on a graph
// handle (which checks its CSR once, at creation).
#include "common.hpp"
#include "dfq_kernel.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

static __device__ __align__(256) unsigned char g_noalloc_scratch[DFQ_NOALLOC_SCRATCH_BYTES];

using namespace dfq;

namespace {

constexpr int kBlock = 512;
constexpr int kMaxDevices = 64;

struct DeviceSetup {
    bool ready = false;
    unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
    int sms = 0;
    int grid[2] = {0, 0};  // without / with parents
    int smem[2] = {0, 0};  // without / with parents
};

std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

// Byte layout of the scratch array for one graph (256-byte aligned pieces).
struct ScratchLayout {
    size_t ctl, bitmap, ovf[2], ovfv[2], piece[2], piece_v[2], total;
    int bitmap_words, piece_cap;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

ScratchLayout scratch_layout(int32_t n, int64_t e, const dfq_opts& o, bool par) {
    ScratchLayout s;
    size_t p = 0;
    s.ctl = p;            p = align256(p + sizeof(dfqk::Control));
    s.bitmap_words = (int)(((int64_t)n + 31) / 32);
    s.bitmap = p;         p = align256(p + 4 * (((size_t)s.bitmap_words + 31) & ~(size_t)31));
    s.piece_cap = dfqk::piece_capacity(n, e, o.large_min_degree, o.piece_edges);
    for (int i = 0; i < 2; ++i) { s.ovf[i] = p;   p = align256(p + 8 * (size_t)n); }
    for (int i = 0; i < 2; ++i) { s.ovfv[i] = p;  p = align256(p + 4 * (size_t)n); }
    for (int i = 0; i < 2; ++i) { s.piece[i] = p;   p = align256(p + 8 * (size_t)s.piece_cap); }
    for (int i = 0; i < 2; ++i) { s.piece_v[i] = p; p = align256(p + (par ? 4 * (size_t)s.piece_cap : 256)); }
    s.total = p;
    return s;
}

// Written into the scratch control block's status word by the CSR check.
__global__ void noalloc_validate_kernel(const int32_t* off, const int32_t* cols, int32_t n, int64_t e,
                                        dfqk::Control* ctl) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < n; i += nth)
        if (off[i + 1] < off[i]) atomicCAS(&ctl->status, 0, 1);
    if (tid == 0 && (off[0] != 0 || (int64_t)off[n] != e)) atomicCAS(&ctl->status, 0, 2);
    for (int64_t k = tid; k < e; k += nth)
        if ((uint32_t)cols[k] >= (uint32_t)n) atomicCAS(&ctl->status, 0, 3);
}

int setup_device(int dev, const dfq_opts& o, DeviceSetup** out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(DFQ_ECUDA, "dfq_bfs_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_setup_mu);
    DeviceSetup& d = g_setup[dev];
    if (!d.ready) {
        void* addr = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
        if (err != cudaSuccess || !addr)
            return fail(DFQ_ECUDA, "dfq_bfs_noalloc: cudaGetSymbolAddress of the scratch array failed: %s",
                        cudaGetErrorString(err));
        cudaDeviceProp prop;
        err = cudaGetDeviceProperties(&prop, dev);
        if (err != cudaSuccess) return fail(DFQ_ECUDA, "dfq_bfs_noalloc: %s", cudaGetErrorString(err));
        if (!prop.cooperativeLaunch) return fail(DFQ_ECUDA, "dfq_bfs_noalloc: no cooperative launch on device %d", dev);
        const void* fns[2] = {single_source_kernel(kBlock, false), single_source_kernel(kBlock, true)};
        for (int i = 0; i < 2; ++i) {
            // input ids are kept here, so the hot-vertex cache stays off (as
            // hot_cache = 0 leaves it for graphs not given hub-first ids)
            const dfqk::SmemLayout lay = dfqk::smem_layout(kBlock, o.local_queue_cap, o.piece_edges, i == 1);
            d.smem[i] = lay.bytes;
            if (int rc = allow_dyn_smem(fns[i], d.smem[i])) return rc;
            int per_sm = 0;
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fns[i], kBlock, d.smem[i]);
            if (err != cudaSuccess || per_sm < 1)
                return fail(DFQ_ECUDA, "dfq_bfs_noalloc: kernel setup failed: %s", cudaGetErrorString(err));
            d.grid[i] = prop.multiProcessorCount * per_sm;
        }
        d.sms = prop.multiProcessorCount;
        d.scratch = (unsigned char*)addr;
        d.ready = true;
    }
    *out = &d;
    return DFQ_OK;
}

}  // namespace

extern "C" int dfq_bfs_noalloc(const int32_t* offsets, const int32_t* cols, int32_t n, int64_t e, int32_t src,
                               int32_t* levels, int32_t* parents, void* stream, dfq_stats* stats) {
    clear_error();
    if (!offsets || !levels || (e > 0 && !cols) || n < 1 || e < 0 || e >= ((int64_t)1 << 31))
        return fail(DFQ_EINVAL, "dfq_bfs_noalloc: need device offsets, cols, levels, 1 <= n, 0 <= e < 2^31");
    if (src < 0 || src >= n) return fail(DFQ_EINVAL, "dfq_bfs_noalloc: source %d outside [0,%d)", src, n);
    if (((uintptr_t)cols & 15) || ((uintptr_t)offsets & 3) || ((uintptr_t)levels & 3) || ((uintptr_t)parents & 3))
        return fail(DFQ_EINVAL, "dfq_bfs_noalloc: cols must be 16-byte aligned and offsets/levels/parents 4-byte aligned");
    dfq_opts o;
    dfq_opts_default(&o);
    const ScratchLayout sl = scratch_layout(n, e, o, parents != nullptr);
    if (sl.total > (size_t)DFQ_NOALLOC_SCRATCH_BYTES)
        return fail(DFQ_ENOMEM, "dfq_bfs_noalloc: a graph with n=%d, e=%lld needs %zu bytes of scratch; the fixed "
                    "scratch array holds %zu (24 bytes per vertex + 0.2 per edge); use dfq_graph_create for larger graphs",
                    n, (long long)e, sl.total, (size_t)DFQ_NOALLOC_SCRATCH_BYTES);
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return fail(DFQ_ECUDA, "dfq_bfs_noalloc: %s", cudaGetErrorString(err));
    DeviceSetup* ds = nullptr;
    int rc = setup_device(dev, o, &ds);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* base = ds->scratch;
    dfqk::Control* ctl = (dfqk::Control*)(base + sl.ctl);
    dfqk::Control host_ctl;

    // CSR check first: a malformed graph would send the kernel out of bounds
    if ((err = cudaMemsetAsync(ctl, 0, sizeof(dfqk::Control), s)) != cudaSuccess)
        return fail(DFQ_ECUDA, "dfq_bfs_noalloc: %s", cudaGetErrorString(err));
    noalloc_validate_kernel<<<ds->sms * 4, 256, 0, s>>>(offsets, cols, n, e, ctl);
    if ((err = cudaMemcpyAsync(&host_ctl, ctl, sizeof(host_ctl), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (err = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(DFQ_ECUDA, "dfq_bfs_noalloc: CSR check: %s", cudaGetErrorString(err));
    if (host_ctl.status)
        return fail(DFQ_EFORMAT, "dfq_bfs_noalloc: %s", host_ctl.status == 1 ? "offsets decrease"
                    : host_ctl.status == 2 ? "offsets[0] != 0 or offsets[n] != e" : "a column index is outside [0,n)");

    dfqk::Params p;
    memset(&p, 0, sizeof p);
    p.offsets = offsets;
    p.cols = cols;
    p.n = n;
    p.src = src;
    p.levels = levels;
    p.parents = parents;
    p.bitmap = (unsigned*)(base + sl.bitmap);
    p.bitmap_words = sl.bitmap_words;
    for (int i = 0; i < 2; ++i) {
        p.ovf[i] = (int2*)(base + sl.ovf[i]);
        p.ovfv[i] = (int*)(base + sl.ovfv[i]);
        p.piece[i] = (int2*)(base + sl.piece[i]);
        p.piece_v[i] = (int*)(base + sl.piece_v[i]);
    }
    p.piece_cap = sl.piece_cap;
    p.ovf_cap = n;
    p.ctl = ctl;
    p.medium_min = o.medium_min_degree;
    p.large_min = o.large_min_degree;
    p.piece_edges = o.piece_edges;
    p.local_cap = o.local_queue_cap;
    p.local_budget = o.local_edge_budget;
    p.probe_first = o.probe_first;
    p.use_tma = o.use_tma;
    p.timeout_ns = (long long)o.timeout_ms * 1000000LL;
    const bool par = parents != nullptr;
    const void* fn = single_source_kernel(kBlock, par);
    // the kernel is shared with the graph handles, which set its limit too
    if (int rc = allow_dyn_smem(fn, ds->smem[par ? 1 : 0])) return rc;
    void* args[] = {&p};
    if ((err = cudaMemsetAsync(ctl, 0, sizeof(dfqk::Control), s)) != cudaSuccess ||
        (err = cudaLaunchCooperativeKernel(fn, dim3(ds->grid[par ? 1 : 0]), dim3(kBlock), args, ds->smem[par ? 1 : 0], s)) !=
            cudaSuccess ||
        (err = cudaMemcpyAsync(&host_ctl, ctl, sizeof(host_ctl), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (err = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(DFQ_ECUDA, "dfq_bfs_noalloc: %s", cudaGetErrorString(err));
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->depth = host_ctl.stats.depth;
        stats->levels = host_ctl.stats.levels;
        stats->reached = (int64_t)host_ctl.stats.claims + 1;
        stats->edges = (int64_t)host_ctl.stats.edges;
        stats->overflow = (int64_t)host_ctl.stats.overflow;
        stats->large = (int64_t)host_ctl.stats.large;
    }
    return device_status(host_ctl);
}
