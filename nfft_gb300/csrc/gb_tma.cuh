// gb_tma.cuh -- tensor-memory-accelerator (TMA) copies of padded grid tiles and
// the shared-memory barrier that waits for them (sm_90 and later PTX).
//
// The oversampled grid is viewed as a 3-D tensor of floats [n_0][n_1][2 n_2]
// (complex values interleaved along the last dimension; encode_grid_map in
// gb_col3_setup.cu), one box being a padded tile: ext x ext x 2 zb floats;
// a 2-D grid as [n_0][2 n_1] with boxes of ext x 2 zb floats
// (encode_grid_map_2d).
//  * tma_load_3d copies a box into shared memory and signals an mbarrier with
//    the byte count (B's subgrid staging);
//  * tma_reduce_add_3d adds a box from shared memory into the grid (B^T's
//    write-back), element by element at L2, as one bulk operation.
// Coordinates are {float index along z, y, x}; the z coordinate must be a
// multiple of 4 floats (16 bytes) and a reduce must not start at a negative
// coordinate.  Waits are bounded: a copy that does not arrive within the
// limit makes the kernel record a time-out and give up on its tile.
#pragma once

#include <cuda.h>

namespace gb {

// polls of an mbarrier before a wait gives up (each poll suspends the thread
// for at most a short, system-defined time)
static constexpr unsigned TMA_WAIT_POLLS = 1u << 22;

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            unsigned long long *bar)
{
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_reduce_add_3d(const CUtensorMap *map, const void *src, int c0, int c1, int c2)
{
  asm volatile("cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                   map),
               "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(src))
               : "memory");
}

// the same for 2-D views (the 2-D column kernels: f32 [n_0][2 n_1])
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            unsigned long long *bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap *map, const void *src, int c0, int c1)
{
  asm volatile("cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(map),
               "r"(c0), "r"(c1), "r"(smem_u32(src))
               : "memory");
}

__device__ __forceinline__ void bulk_commit()
{
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// returns once every committed bulk operation has finished reading shared memory
__device__ __forceinline__ void bulk_wait_read_all()
{
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// orders this thread's earlier shared-memory writes before later bulk (async
// proxy) operations on the same memory
__device__ __forceinline__ void fence_proxy_async_smem()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// waits for phase `parity` of the barrier to complete; false after `polls`
// unsuccessful polls
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, unsigned polls)
{
  for (unsigned i = 0; i < polls; ++i) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace gb
