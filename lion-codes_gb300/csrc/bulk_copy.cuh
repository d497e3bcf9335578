// Copy-engine staging of matrices into shared memory: 1-D bulk copies
// (cp.async.bulk, global -> this CTA's shared memory) that complete on an
// mbarrier, and bulk prefetches into L2. Everything here reads this GPU's own
// memory; nothing is multicast.
//
// A warp stages one n x n complex128 matrix (row stride lda in global memory,
// lds in shared memory) with one bulk copy per row, issued by lanes 0..n-1:
// each row is 16 n bytes, and both row starts are 16-byte aligned because
// complex128 entries are 16 bytes, so the padded shared-memory row stride
// (n + 1 entries, against bank conflicts) needs no second pass. The warp then
// waits on its mbarrier for the n rows' bytes. Every wait is bounded: a wait
// that runs out reports failure, and the caller stops using bulk copies for
// the rest of the kernel after a second bounded wait for the copies in flight.
#pragma once

#include <stdint.h>

#include "lufqhe_internal.cuh"

namespace lufqhe {

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
// make an initialised mbarrier visible to the copy engine
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// order this thread's earlier generic-proxy accesses to shared memory before
// later async-proxy (bulk copy) writes to it
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// bytes (a multiple of 16) from 16-byte aligned global src to 16-byte aligned
// shared dst, completing `bytes` transactions on bar
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded: false if the phase did not complete within `tries` polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, unsigned tries) {
  for (unsigned t = 0; t < tries; ++t)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// bytes (a multiple of 16) from 16-byte aligned global memory into L2
__device__ __forceinline__ void prefetch_l2_bulk(const void *src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Polls of one wait before it is given up (each poll may suspend the thread
// for a while; this is far above any real copy's time).
constexpr unsigned kBulkWaitTries = 1u << 22;

// One warp's bulk-copy state: its mbarrier (8 bytes of shared memory) and the
// phase it waits for next.
struct WarpBulk {
  uint64_t *bar = nullptr;
  unsigned phase = 0;
  bool broken = false;  // a wait ran out: per-lane loads from then on

  __device__ __forceinline__ void init(uint64_t *b, int lane) {
    bar = b;
    phase = 0;
    if (lane == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    __syncwarp();
  }
  // Stage matrix A (n x n complex128, row stride lda) into M (row stride lds).
  // Warp-uniform result: false if the wait ran out (M is then not valid).
  __device__ bool load(const double2 *A, int n, int lda, double2 *M, int lds, int lane) {
    __syncwarp();
    fence_proxy_async_smem();
    if (lane == 0) mbar_arrive_expect_tx(bar, (unsigned)(n * n * 16));
    __syncwarp();
    for (int i = lane; i < n; i += 32)
      bulk_g2s(M + i * lds, A + (size_t)i * lda, (unsigned)(n * 16), bar);
    bool ok = mbar_wait(bar, phase, kBulkWaitTries);
    ok = __all_sync(kFull, ok);
    if (!ok) {
      // give the copies in flight a second bounded wait, then stop using them
      mbar_wait(bar, phase, kBulkWaitTries);
      broken = true;
    }
    phase ^= 1u;
    return ok;
  }
};

// L2 prefetch of an n x n complex128 matrix with row stride lda (the span
// from its first entry to the end of its last row).
__device__ __forceinline__ void prefetch_matrix_l2(const double2 *A, int n, int lda) {
  prefetch_l2_bulk(A, (unsigned)(((size_t)(n - 1) * lda + n) * 16));
}

}  // namespace lufqhe
