// TMA (cp.async.bulk.tensor) + mbarrier helpers in inline PTX for sm_103a.
//
// The face kernel stages one z-plane of the primitive field per step: a
// 4-D box {tx+6, ty+2H, 1, NQ} of the tensor (x, y, z, component) of one
// box's scratch array.  Every wait is bounded: after MBAR_SPIN_LIMIT polls
// it gives up and reports failure to the caller, which raises an error flag
// the host reads, instead of hanging the GPU.
#pragma once
#include <cstdint>
#include <cuda.h>

namespace amrs {

constexpr long long MBAR_SPIN_LIMIT = 1ll << 26;

// Per-launch TMA descriptor table: maps[b] is the tensor map of box b's
// primitive scratch (64-byte aligned CUtensorMap objects in global memory).
struct TmaDesc {
  const CUtensorMap* maps;
  int enabled;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Returns false if the phase did not complete within `limit` polls.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity,
                                          long long limit = MBAR_SPIN_LIMIT) {
  const uint32_t a = smem_u32(bar);
  for (long long it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Issue one 4-D tiled TMA load of box b's plane into shared memory and
// arm the barrier with the expected byte count.  Coordinates are element
// offsets into the scratch array (x must be even: 16-byte aligned start).
__device__ __forceinline__ void tma_load_plane(const TmaDesc& t, int b, unsigned long long* bar, void* dst, int x,
                                               int y, int z, int bytes) {
  const uint32_t ab = smem_u32(bar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ab), "r"(bytes) : "memory");
  const CUtensorMap* m = t.maps + b;
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(m)), "r"(x), "r"(y), "r"(z), "r"(0), "r"(ab)
      : "memory");
}

}  // namespace amrs
