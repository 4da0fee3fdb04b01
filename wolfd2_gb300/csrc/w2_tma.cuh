// w2_tma.cuh -- tensor-memory-accelerator (TMA) loads of whole tile boxes.
//
// The mixed Poisson kernel's multi-tile mode restages each tile's box (two
// colour planes of e, two of r) from the colour-split global buffers every
// group of sweeps.  Those boxes are exactly 3-D tiles of the buffers --
// {box columns, box rows, 2 colours} -- so one thread issues one
// cp.async.bulk.tensor per buffer and the copy engine fills the shared
// planes while the block waits on an mbarrier, instead of every thread
// moving 16-byte vectors.  Only this GPU's own memory is read; no cluster
// multicast.
//
// Alignment (checked on the host when the maps are made, else the kernel
// keeps its vector loads): buffer base and row/plane strides multiples of 16
// bytes, box x offsets (tile column origins, multiples of 4 floats) and box
// widths multiples of 16 bytes, box extents at most 256, shared destinations
// aligned to 128 bytes.
#pragma once
#include <cuda.h>

#include "w2_common.cuh"

namespace w2 {

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arrive (the one arrival a phase needs) and announce the bytes the phase's
// copies will deliver.
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// Order this thread's earlier generic-proxy accesses to shared memory (made
// visible to it by a block barrier) before async-proxy writes it issues next.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 3-D tile {x, y, z} of the tensor map into shared memory at dst, completing
// on bar.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_test(unsigned long long *bar, unsigned phase) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return done != 0;
}

// Wait for phase `phase` of bar to complete, at most kWaitLimitNs.  On
// timeout it sets W2_E_TIMEOUT, then waits once more within the same limit
// so that no copy is still writing this block's shared memory when the
// caller leaves, and returns false.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned phase, Sync *sy) {
  unsigned long long t0 = gtime_ns();
  for (unsigned spins = 0;; ++spins) {
    if (mbar_test(bar, phase)) return true;
    if ((spins & 63u) == 63u && gtime_ns() - t0 > kWaitLimitNs) break;
  }
  set_error(sy, W2_E_TIMEOUT);
  t0 = gtime_ns();
  for (unsigned spins = 0;; ++spins) {
    if (mbar_test(bar, phase)) break;
    if ((spins & 63u) == 63u && gtime_ns() - t0 > kWaitLimitNs) break;
  }
  return false;
}

}  // namespace w2

// ---- host: tensor maps of the colour-split buffers -------------------------

// Map of a buffer of 2 colour planes of gh rows x gw floats, read in boxes
// of {hw, bh, 2}.  Returns false where the TMA rules do not hold (then the
// caller keeps the vector loads).
bool w2_encode_plane_map(CUtensorMap *map, const float *base, int gw, int gh, int hw, int bh);
