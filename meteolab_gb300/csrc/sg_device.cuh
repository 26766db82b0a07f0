// Device helpers shared by the kernel translation units: the work-item loop and asynchronous copies.
#pragma once
#include <cuda_runtime.h>

namespace sg {

#define FOR_ITEMS for (int it = blockIdx.x; it < nitems; it += gridDim.x)

// 4-byte asynchronous copy global -> shared (lands without passing through registers), and the wait for all of
// this thread's copies; other threads see the data after the next barrier.
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
// 16-byte asynchronous copy (both addresses 16-byte aligned), not cached in L1
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---- TMA bulk copies (cp.async.bulk, global -> shared, completing on an mbarrier's transaction count) and the
// mbarrier operations around them. Addresses of both sides 16-byte aligned, sizes multiples of 16 bytes.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// One arrival that also raises the barrier's expected transaction bytes of its current phase.
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Waits for the phase of `parity` to complete, at most MBAR_WAIT_NS of the global timer (and at most 2^24 rounds of
// polls, should the timer not advance); false when it did not complete in that time.
constexpr unsigned long long MBAR_WAIT_NS = 200000000ull;
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (int round = 0; round < (1 << 24); round++) {
    for (int i = 0; i < 32; i++)
      if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > MBAR_WAIT_NS) return false;
  }
  return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
// Orders this thread's earlier shared-memory accesses (and, after a block barrier, the block's) before its later
// bulk copies into shared memory.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// Makes freshly initialised mbarriers visible to the copies that complete on them.
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

// Levels a run may have (per-level tables and column arrays in shared memory or registers are sized for it).
constexpr int MAXNZ = 128;

// Blocks of a launch over n work items: n, at most cap.
#define GRID(n, cap) dim3(max(1, min((n), (cap))))

// Opt every kernel with dynamic shared memory in to the device's per-block maximum, less its static shared memory.
template <class K>
cudaError_t smem_limit(K kernel, int bytes) {
  cudaFuncAttributes attr;
  cudaError_t e = cudaFuncGetAttributes(&attr, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes - (int)attr.sharedSizeBytes);
}

}  // namespace sg
