// The single-source kernel in its cluster form: one thread-block cluster of
// 2-16 blocks runs the whole BFS and ends each level on a cluster barrier in
// distributed shared memory (dfqk::cluster_barrier) instead of the grid
// barrier in global memory.  A translation unit of its own, so the build
// compiles it beside the other kernels.
#include "dfq_kernel.cuh"
#include "common.hpp"

namespace dfq {

const void* cluster_kernel(int block_threads, bool par) {
    switch (block_threads) {
        case 512: return par ? (const void*)dfqk::dfq_cluster_kernel<512, true> : (const void*)dfqk::dfq_cluster_kernel<512, false>;
        case 1024: return par ? (const void*)dfqk::dfq_cluster_kernel<1024, true> : (const void*)dfqk::dfq_cluster_kernel<1024, false>;
        default: return nullptr;
    }
}

}  // namespace dfq
