// Tensor-memory-access (TMA) tile loads and the mbarrier they complete on,
// as inline PTX for sm_103a.  One elected thread arms the barrier with the
// byte count it expects and issues the bulk tensor copies; every thread then
// waits on the barrier's phase.  Every wait is bounded.
#pragma once

#include <cuda.h>  // CUtensorMap (the type only; maps are encoded on the host)

namespace wenofd {
namespace dev {

// Polls of a TMA completion wait before it gives up (a copy completes in
// microseconds).
constexpr unsigned kTmaWaitLimit = 1u << 20;

__device__ __forceinline__ unsigned tma_smem_addr(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void tma_bar_init(unsigned bar, unsigned arrivals) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(arrivals) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that also announces `bytes` of copies still to complete.
__device__ __forceinline__ void tma_bar_expect(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// Waits for phase `parity` of the barrier to complete; false if it did not
// within `limit` polls.
__device__ __forceinline__ bool tma_bar_wait(unsigned bar, unsigned parity, unsigned limit) {
  for (unsigned it = 0; it < limit; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred P1;\n mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
        " selp.b32 %0, 1, 0, P1;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before later async-proxy (TMA) writes to it.
__device__ __forceinline__ void tma_fence_proxy() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Box of a 3-D / 2-D tiled tensor map at element coordinates (x innermost)
// into shared memory at dst; completes `bar`'s transaction bytes.  The
// innermost coordinate times the element size must be a multiple of 16
// bytes; other coordinates may lie outside the tensor (zero fill).
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap *map, int x, int y, int z, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap *map, int x, int y, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

}  // namespace dev
}  // namespace wenofd
