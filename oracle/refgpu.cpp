// refgpu.cpp - runs the reference's own BFS kernel.  TEST/BENCH INFRASTRUCTURE:
// used to pin the CPU oracle against the reference itself and as the
// reference GPU baseline; the product never links it.
//
// The kernel comes from a cubin that oracle/build.py compiles from the
// reference sources (device code only).  This file reproduces the reference
// host path around it (design/shared-q/atomic-sa/our-sep/upper-bound/bfs.cu,
// "DFQ"): cost[] = -1 except the source (DFQ:216), done = false (DFQ:259),
// grid = SMs x occupancy(1024 threads) (DFQ:255-268), one cooperative launch
// timed with events around launch + synchronize (DFQ:279-288).  Device memory
// replaces the reference's managed memory + prefetch (DFQ:194-197,273-277).
//
// Guards (the reference kernel has no bounds checks):
//   * the edge array is padded by 16 zero entries, because VISIT_tiled reads
//     edge[start + lane] for all 8 lanes before testing the list end
//     (DFQ:49-51); padding keeps those reads inside the allocation and the
//     vertex ids they produce valid;
//   * the caller passes per-level bin populations computed from oracle levels
//     (refgpu_check_bins) and the run is refused when a level would exceed a
//     static global queue (ftr_EQ[131072], ftr_FQ[16384], DFQ:31-36,96; the
//     global-queue baseline's ftr_SQ/MQ/LQ, design/global-q/stripe-sa/gun-sep/
//     lower-bound/bfs.cu:16-18,77) or the depth would overflow the kernel's
//     short levels (DFQ:105,192).
#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {
thread_local std::string g_err;
int fail(const char* what, CUresult r) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "unknown CUDA error");
    return -1;
}
int fail(const std::string& what) { g_err = what; return -1; }
}  // namespace

struct refgpu {
    CUdevice dev = 0;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction fn = nullptr;
    CUstream stream = nullptr;
    CUevent ev0 = nullptr, ev1 = nullptr;
    CUdeviceptr node = 0, edge = 0, cost = 0, done = 0, num = 0;
    int32_t n = 0;
    int64_t e = 0;
    int grid = 0;
    int kind = 0;  // 0 = shared-q DFQ, 1 = global-q gun-sep
};

extern "C" {

const char* refgpu_error(void) { return g_err.c_str(); }

// kind: 0 = the canonical DFQ kernel, 1 = the global-queue gun-sep baseline.
int refgpu_open(const char* cubin, int kind, refgpu** out) {
    *out = nullptr;
    CUresult r = cuInit(0);
    if (r) return fail("cuInit", r);
    refgpu* h = new refgpu();
    h->kind = kind;
    if ((r = cuDeviceGet(&h->dev, 0))) { delete h; return fail("cuDeviceGet", r); }
    if ((r = cuDevicePrimaryCtxRetain(&h->ctx, h->dev))) { delete h; return fail("cuDevicePrimaryCtxRetain", r); }
    cuCtxSetCurrent(h->ctx);
    if ((r = cuModuleLoad(&h->mod, cubin))) { cuDevicePrimaryCtxRelease(h->dev); delete h; return fail("cuModuleLoad", r); }
    // CUDA_BFS_KERNEL_CG_NEW(Node*, int*, short*, bool*, int*) with C++ linkage
    if ((r = cuModuleGetFunction(&h->fn, h->mod, "_Z22CUDA_BFS_KERNEL_CG_NEWP4NodePiPsPbS1_"))) {
        cuModuleUnload(h->mod); cuDevicePrimaryCtxRelease(h->dev); delete h;
        return fail("cuModuleGetFunction", r);
    }
    int sms = 0, per_sm = 0;
    cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, h->dev);
    cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, h->fn, 1024, 0);
    if (per_sm < 1) per_sm = 1;
    h->grid = sms * per_sm;
    cuStreamCreate(&h->stream, CU_STREAM_NON_BLOCKING);
    cuEventCreate(&h->ev0, CU_EVENT_DEFAULT);
    cuEventCreate(&h->ev1, CU_EVENT_DEFAULT);
    *out = h;
    return 0;
}

int refgpu_grid(refgpu* h) { return h ? h->grid : -1; }

int refgpu_load_graph(refgpu* h, int32_t n, int64_t e, const int32_t* offsets, const int32_t* cols) {
    cuCtxSetCurrent(h->ctx);
    std::vector<int32_t> node(2 * (size_t)n);
    for (int32_t i = 0; i < n; ++i) { node[2 * i] = offsets[i]; node[2 * i + 1] = offsets[i + 1] - offsets[i]; }
    CUresult r;
    if ((r = cuMemAlloc(&h->node, 8 * (size_t)n))) return fail("cuMemAlloc(node)", r);
    if ((r = cuMemAlloc(&h->edge, 4 * ((size_t)e + 16)))) return fail("cuMemAlloc(edge)", r);
    if ((r = cuMemAlloc(&h->cost, 2 * (size_t)n + 16))) return fail("cuMemAlloc(cost)", r);
    if ((r = cuMemAlloc(&h->done, 16))) return fail("cuMemAlloc(done)", r);
    if ((r = cuMemAlloc(&h->num, 16))) return fail("cuMemAlloc(num)", r);
    cuMemcpyHtoD(h->node, node.data(), 8 * (size_t)n);
    if (e) cuMemcpyHtoD(h->edge, cols, 4 * (size_t)e);
    cuMemsetD32(h->edge + 4 * (size_t)e, 0, 16);
    cuMemcpyHtoD(h->num, &n, 4);
    h->n = n;
    h->e = e;
    return 0;
}

// Bin populations per level for the reference kernel `kind`, from oracle
// levels; returns 0 when every static queue is large enough, else -1.
int refgpu_check_bins(int kind, int32_t n, const int32_t* offsets, const int32_t* levels) {
    int32_t depth = -1;
    for (int32_t v = 0; v < n; ++v) if (levels[v] > depth) depth = levels[v];
    if (depth >= 32000) return fail("depth " + std::to_string(depth) + " overflows the kernel's short levels");
    std::vector<int64_t> a((size_t)depth + 2, 0), b((size_t)depth + 2, 0), c((size_t)depth + 2, 0);
    for (int32_t v = 0; v < n; ++v) {
        const int32_t l = levels[v];
        if (l < 0) continue;
        const int32_t d = offsets[v + 1] - offsets[v];
        if (d == 0) continue;
        if (kind == 0) {
            if (d > 16384) a[l]++;          // ftr_FQ
            else if (d > 1024) b[l]++;      // ftr_EQ
        } else {
            if (d <= 32) a[l]++;            // ftr_SQ
            else if (d <= 256) b[l]++;      // ftr_MQ
            else c[l]++;                    // ftr_LQ
        }
    }
    for (int32_t l = 0; l <= depth; ++l) {
        if (kind == 0 && (a[l] > 16384 || b[l] > 131072))
            return fail("level " + std::to_string(l) + " exceeds the DFQ kernel's global queues");
        if (kind == 1 && (a[l] > 33554432 || b[l] > 16777216 || c[l] > 8388608))
            return fail("level " + std::to_string(l) + " exceeds the global-queue kernel's queues");
    }
    return 0;
}

// One BFS from src; levels_out[n] (int32, -1 unreached) and the reference's
// "- Time" in *ms.
int refgpu_bfs(refgpu* h, int32_t src, int32_t* levels_out, float* ms) {
    if (!h || src < 0 || src >= h->n) return fail("refgpu_bfs: bad arguments");
    cuCtxSetCurrent(h->ctx);
    CUresult r;
    cuMemsetD16Async(h->cost, 0xffff, (size_t)h->n, h->stream);
    const int16_t zero = 0;
    cuMemcpyHtoDAsync(h->cost + 2 * (size_t)src, &zero, 2, h->stream);
    cuMemsetD8Async(h->done, 0, 16, h->stream);
    void* args[] = {&h->node, &h->edge, &h->cost, &h->done, &h->num};
    cuEventRecord(h->ev0, h->stream);
    if ((r = cuLaunchCooperativeKernel(h->fn, h->grid, 1, 1, 1024, 1, 1, 0, h->stream, args)))
        return fail("cuLaunchCooperativeKernel", r);
    if ((r = cuStreamSynchronize(h->stream))) return fail("kernel", r);
    cuEventRecord(h->ev1, h->stream);
    if ((r = cuEventSynchronize(h->ev1))) return fail("event", r);
    float t = 0;
    cuEventElapsedTime(&t, h->ev0, h->ev1);
    if (ms) *ms = t;
    std::vector<int16_t> c((size_t)h->n);
    if ((r = cuMemcpyDtoH(c.data(), h->cost, 2 * (size_t)h->n))) return fail("cuMemcpyDtoH", r);
    for (int32_t i = 0; i < h->n; ++i) levels_out[i] = c[i];
    return 0;
}

void refgpu_close(refgpu* h) {
    if (!h) return;
    cuCtxSetCurrent(h->ctx);
    if (h->stream) cuStreamSynchronize(h->stream);
    if (h->node) cuMemFree(h->node);
    if (h->edge) cuMemFree(h->edge);
    if (h->cost) cuMemFree(h->cost);
    if (h->done) cuMemFree(h->done);
    if (h->num) cuMemFree(h->num);
    if (h->ev0) cuEventDestroy(h->ev0);
    if (h->ev1) cuEventDestroy(h->ev1);
    if (h->stream) cuStreamDestroy(h->stream);
    if (h->mod) cuModuleUnload(h->mod);
    cuDevicePrimaryCtxRelease(h->dev);
    delete h;
}

}  // extern "C"
