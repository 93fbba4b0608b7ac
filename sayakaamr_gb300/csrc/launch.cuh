// Kernel launch helper with optional Programmatic Dependent Launch (PDL):
// the launch may start while the previous kernel in the stream is draining;
// every kernel launched this way calls pdl_enter() first, which releases its
// own dependents early and then waits until the previous grid has completed
// and its memory is visible.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <utility>

namespace sayaka_gb300 {

__device__ __forceinline__ void pdl_enter() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  cudaTriggerProgrammaticLaunchCompletion();
  cudaGridDependencySynchronize();
#endif
}

// The dynamic shared-memory limit of kernel fn raised to at least `bytes`
// on the current device, thread-safe and only when it grows: the attribute
// is per device, so a process with handles on several GPUs sets it on each.
// A refusal is not left pending as the thread's CUDA error: the launch that
// needs the memory reports it.
inline void ensure_max_smem(const void *fn, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, int> set_to;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  std::lock_guard<std::mutex> lk(mu);
  int &cur = set_to[{fn, dev}];
  if (cur >= bytes) return;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess)
    cur = bytes;
  else
    cudaGetLastError();
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                            Args... args) {
  if (!pdl) {
    kern<<<grid, block, smem, s>>>(args...);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute a[1];
  a[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  a[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = a;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

}  // namespace sayaka_gb300
