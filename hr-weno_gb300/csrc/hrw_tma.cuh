// hrw_tma.cuh - TMA tile copies for the 2D stage kernels (stage2d.cu, stage2d_f32c.cu): one
// thread issues cp.async.bulk.tensor.2d copies that complete on a block mbarrier, which the
// block waits on with a bounded poll.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace hrw {

static __device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

static __device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                                   uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

static __device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

static __device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Wait for phase `parity` of the block's mbarrier, at most `limit` polls; true when it
// completed.
static __device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit) {
  const uint32_t a = smem_u32(bar);
  for (int it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// A row-major array of n2 rows of n1 elements of `elem_bytes` (4: float, 8: double; row pitch
// n1 elements) as a 2D tensor with a box_x x box_y box, cached by array; false when it cannot
// be described (pitch or address not 16-byte aligned, or no driver entry point).
bool tile_map_2d(const void* p, int elem_bytes, int n1, int n2, int box_x, int box_y, CUtensorMap* out);

}  // namespace hrw
