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
