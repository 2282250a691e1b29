// Programmatic dependent launch for the kernels of the Krylov loops.  A kernel launched with
// launch_pdl may be scheduled while the kernel before it in the stream drains its last wave; it
// calls pdl_wait() before its first access to memory (which returns once that kernel has
// completed and its writes are visible; at once in a kernel launched the ordinary way) and
// pdl_launch_dependents() to let the next such kernel be scheduled.
#pragma once
#include <cuda_runtime.h>

#include <utility>

namespace sfem {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace sfem

namespace sfem {

// CTAs of `kernel` resident on the whole device at once (SMs x CTAs per SM at this block size);
// a grid of at most this many runs as one wave, with no partly filled last wave.
template <typename... KArgs>
inline int resident_ctas(void (*kernel)(KArgs...), int threads, size_t smem) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
  return (per > 0 ? per : 1) * (sms > 0 ? sms : 1);
}

}  // namespace sfem
