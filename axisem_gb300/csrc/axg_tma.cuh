// axg_tma.cuh -- bulk (TMA) copies global -> shared with mbarrier completion.
//
// Element blocks of metric terms are contiguous, 16-byte aligned and a
// multiple of 16 bytes long, so they are moved with the 1-D form
// cp.async.bulk (no tensor map).  Every wait on an mbarrier is bounded in
// time, measured on the GPU's global nanosecond timer: after kWaitNs the
// waiter records AXG_ERR_TIMEOUT in the kernel's error word and gives up, so a
// lost copy cannot hang the GPU.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace axg {

constexpr uint64_t kWaitNs = 1000000000ull;  // a wait gives up after 1 s
// a wait still pending after this long first checks whether another wait of
// the kernel already gave up; if so it returns at once, so that a kernel whose
// copies were lost ends within about kWaitNs instead of kWaitNs per wait
constexpr uint64_t kWaitCheckNs = 20000ull;
constexpr int kPollsPerTimerRead = 16;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization may start before the kernel ahead of it in the stream has
// finished: pdl_wait() returns once that kernel has completed and its
// writes are visible (a no-op for an ordinary launch), so every kernel of a
// time step calls it before its first read of data the step writes.
// pdl_trigger() lets the next kernel's CTAs be scheduled once every CTA of
// this one has called it (or exited); they run up to their own pdl_wait().
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// make the initialised barriers visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one thread: arm the barrier for `bytes` and start the bulk copy
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar,
                                         uint64_t policy) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
      : "memory");
}

// arm the barrier once for several copies that complete on it
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// bulk copy completing on a barrier that mbar_expect_tx already armed
__device__ __forceinline__ void bulk_g2s_tx(void *dst, const void *src, uint32_t bytes, uint64_t *bar,
                                            uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
      : "memory");
}

// plain arrival (release semantics at CTA scope) of the calling thread
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// 4-byte asynchronous global -> shared copy (no register staging), and the
// wait for all of the thread's outstanding ones
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// L2 policy for data read once per step (the metric terms)
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for the phase of `bar` with `parity`; returns false when it
// gave up, after recording AXG_ERR_TIMEOUT in *err.  The first poll is the
// fast path; the timer is read only once the wait is pending.
__device__ __noinline__ bool mbar_wait_slow(uint64_t *bar, uint32_t parity, int32_t *err) {
  const uint64_t t0 = globaltimer_ns();
  bool checked = false;
  for (;;) {
    for (int k = 0; k < kPollsPerTimerRead; ++k)
      if (mbar_try_wait(bar, parity)) return true;
    const uint64_t dt = globaltimer_ns() - t0;
    if (!checked && dt > kWaitCheckNs) {
      checked = true;
      if (err && *reinterpret_cast<volatile int32_t *>(err) != 0) return false;  // a wait already gave up
    }
    if (dt > kWaitNs) break;
  }
  if (err) atomicCAS(err, 0, 5 /* AXG_ERR_TIMEOUT */);
  return false;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int32_t *err) {
  if (mbar_try_wait(bar, parity)) return true;
  return mbar_wait_slow(bar, parity, err);
}

// After a timeout, copies issued by this CTA may still be in flight into its
// shared memory: wait (bounded again) for the last phase issued on `bar`
// before the CTA exits.  A phase that never completes gives up after kWaitNs.
__device__ __forceinline__ void mbar_drain(uint64_t *bar, uint32_t parity) {
  const uint64_t t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity))
    if (globaltimer_ns() - t0 > kWaitNs) break;
}

}  // namespace axg
