// hrw_batch_dev.cuh - device helpers shared by the batched kernels (batch.cu, batch_f32c.cu).
#pragma once
#include <cuda_runtime.h>

namespace hrw {

constexpr int kBatchThreads = 256;  // threads per block; a block holds kBatchThreads / G groups

// barrier of one group of G threads (whole warps) within the block
template <int G>
__device__ __forceinline__ void group_sync(int gid) {
  if constexpr (G == 32) {
    __syncwarp();
  } else if constexpr (G == kBatchThreads) {
    __syncthreads();
  } else {
    // named barrier gid + 1 (barrier 0 is __syncthreads), G threads of whole warps
    asm volatile("bar.sync %0, %1;" ::"r"(gid + 1), "r"(G) : "memory");
  }
}

}  // namespace hrw
