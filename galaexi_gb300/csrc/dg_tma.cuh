// One-dimensional bulk copies global -> shared memory by the tensor memory accelerator
// (cp.async.bulk), completing on an mbarrier in shared memory, and a bounded wait for them; bulk
// prefetches global -> L2.
//
// A copy needs a 16-byte aligned source and destination and a size that is a multiple of 16 bytes;
// bulk_ok() checks that.  One thread arms the barrier with the total byte count of its copies and
// issues them; every thread then waits for the barrier's phase with a limit on its polls.  A wait that
// runs out of polls records kTmaTimeout in *err (read back by the host, which reports
// DG_ERR_TIMEOUT), waits once more with a limit for the copies still in flight (so that they do not
// land in shared memory the block no longer owns) and reports failure; the caller returns.
#pragma once
#include <cstdint>

namespace gx {

constexpr int kTmaTimeout = 1;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool bulk_ok(const void* src, const void* dst, unsigned bytes) {
  return ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst) | bytes) & 15u) == 0;
}

// initialise a barrier for one arrival (the thread that issues the copies); call from one thread,
// then __syncthreads() before any thread waits on it
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// the issuing thread's arrival, announcing the bytes the copies will deliver
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// start pulling `bytes` (16-byte aligned address and size) from global memory into L2; no completion
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned phase) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return done != 0;
}

// wait for the barrier's phase; false (and *err set) if the copies did not complete within `limit`
// polls.  try_wait suspends the thread between polls until the phase completes or a time limit of
// the hardware passes (7.5 us per poll measured on GB300 for a phase that never completes), so the
// default limit gives up after about a second, far beyond the microseconds the copies take
constexpr long long kTmaWaitLimit = 1ll << 17;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned phase, int* err, long long limit = kTmaWaitLimit) {
  for (long long it = 0; it < limit; ++it)
    if (mbar_test(bar, phase)) return true;
  if (err) atomicExch(err, kTmaTimeout);
  for (long long it = 0; it < limit; ++it)
    if (mbar_test(bar, phase)) break;
  return false;
}

}  // namespace gx
