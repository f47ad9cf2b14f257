// pt_tma.cuh -- bulk copies from global into shared memory with the Tensor
// Memory Accelerator (cp.async.bulk, completing on an mbarrier), and
// waits on the mbarrier bounded by %globaltimer.
#pragma once
#include <cstdint>

namespace pt {

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// One thread: an mbarrier with one arrival, made visible to the async proxy.
__device__ __forceinline__ void mbar_init(uint32_t bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// The arrival, expecting `bytes` from the bulk copies of this phase.
__device__ __forceinline__ void mbar_arrive_expect(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// Waits for the phase with `parity` to complete; false after bound_ns.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long bound_ns) {
  const unsigned long long t0 = global_ns();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (global_ns() - t0 > bound_ns) return false;
  }
}

// A block copies n doubles src[0, n) into shared memory (`raw`: n + 2
// doubles, 16-byte aligned) and returns where they start: raw + 1 when src
// sits 8 bytes past a 16-byte boundary, so that source and destination
// share their alignment.  The aligned interior goes by one bulk copy on
// `bar`; the head and tail (at most one double each) by plain loads.  Call
// with every thread of the block; false (after a second bounded wait for
// the copy in flight) when the copy did not land within bound_ns.  The copy
// may then still be in flight into this block's shared memory, where a later
// block on the same SM could find its bytes: the caller records PT_TIMEOUT,
// and the device's results after it are suspect (the host discards the
// handle whose run reported it).
__device__ __forceinline__ bool stage_doubles(double* raw, const double* src, int n, uint64_t* bar_word,
                                              unsigned long long bound_ns, double** out) {
  const int off = ((uintptr_t)src & 15u) ? 1 : 0;
  double* dst = raw + off;
  const int head = off, ni = ((n - head) / 2) * 2;
  const uint32_t bar = smem_addr(bar_word);
  if (threadIdx.x == 0) {
    mbar_init(bar);
    mbar_arrive_expect(bar, (uint32_t)ni * 8u);
    if (ni > 0) bulk_g2s(dst + head, src + head, (uint32_t)ni * 8u, bar);
  }
  if (threadIdx.x == 1 && head) dst[0] = __ldg(src);
  if (threadIdx.x == 2 && head + ni < n) dst[n - 1] = __ldg(src + n - 1);
  __syncthreads();                                  // the barrier is initialised before any wait
  const bool landed = __syncthreads_and(mbar_wait(bar, 0, bound_ns));
  if (!landed) {
    if (threadIdx.x == 0) mbar_wait(bar, 0, bound_ns);
    __syncthreads();
  }
  *out = dst;
  return landed;
}

}  // namespace pt
