// Tensor-memory-accelerator (TMA) staging of frame tiles: a 2-D tensor map
// per frame (host), and the per-warp mbarrier protocol that one lane drives
// (device). Only this GPU's own frames are mapped, and no load is
// multicast: every tile goes to the shared memory of the warp that asked.
//
// The protocol for one buffer of one warp: lane 0 fences the warp's earlier
// generic accesses to the buffer against the async proxy, arms the buffer's
// mbarrier with the box's byte count and issues the 2-D box load; every lane
// then waits on the mbarrier's phase. Waits are bounded: a wait that runs out
// returns false, and the caller records a fault and stops instead of
// spinning on.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sf {

// try_wait rounds before a wait gives up. Each round may suspend the thread
// for a hardware-chosen time (microseconds), so the bound is about a second
// or more, far beyond a tile load's microseconds.
constexpr uint32_t kTmaWaitRounds = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Makes mbarrier initialisation visible to the async proxy (the TMA unit).
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Orders this thread's (and, after a warp sync, its warp's) generic-proxy
// accesses to shared memory before later async-proxy ones.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// One 2-D box of `map` at element coordinates (x, y) into shared memory at
// dst (128-byte aligned), completing on bar. x * element size must be a
// multiple of 16 bytes; x and y may lie before the tensor (out-of-bounds
// elements are filled with zeros).
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// Waits for phase `parity` of bar to complete; false if it did not within
// kTmaWaitRounds rounds.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t i = 0; i < kTmaWaitRounds; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done)
      return true;
  }
  return false;
}

// Host: a 2-D tensor map over a row-major frame of h rows x w pixels of
// `bytes_per_pixel` (2 or 4) at `base`, boxes of box_w x box_h pixels.
// False when the frame cannot be mapped (base not 16-byte aligned, a row
// pitch that is not a multiple of 16 bytes, no driver entry point) -- the
// caller then stages with per-lane copies.
bool encode_frame_map(CUtensorMap *map, const void *base, int h, int w, int bytes_per_pixel,
                      int box_w, int box_h);

} // namespace sf
