// Dot product of two device vectors that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the point where they need a reduction:
// code running inside a CUDA stream capture (cudaMalloc is not a capturable
// operation and synchronises the device), real-time control loops that forbid
// allocation after start-up, and host applications that plan all device memory
// themselves and hand the library nothing but their own buffers.  For them this
// file keeps the reduction's scratch -- one partial sum per 2048-element tile and
// a completion counter -- in a file-scope static device array of fixed size.
//
// Limits and sharing rules (also stated in include/sfem.h):
//  * at most kNoAllocMaxTiles tiles, i.e. n <= 65536 * 2048 = 134,217,728 entries;
//  * the array is loaded with the library and held by every GPU that loads it
//    until the process exits (512 KiB + 256 B per device);
//  * every call shares it and it keeps the last call's contents: each call clears
//    the completion counter before launching, so calls that overlap on the GPU
//    (concurrent streams) race and must be serialised by the caller;
//  * the first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call before
//    any stream capture begins.  The address is cached for the life of the process:
//    after cudaDeviceReset, or after the device's primary context is released, the
//    cached address is stale and the entry point must not be called on that device;
//  * the summation order (fixed tiles, partials in index order) is deterministic but
//    not sfem_dot's, so the two results can differ in the last bits.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "sfem.h"
#include "sfem_internal.h"

namespace {

constexpr int kTile = 2048;        // entries per block
constexpr int kThreadsNA = 256;    // 8 entries per thread
constexpr int64_t kNoAllocMaxTiles = 65536;
constexpr int kMaxDevices = 64;

// partials[0 .. tiles) followed by the completion counter (as the last 32 bytes)
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxTiles + 32];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum_na(double v) {
  __shared__ double sm[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sm[lane] : 0.0;
  if (w == 0) v = warp_sum(v);
  __syncthreads();
  return v;
}

// One 2048-entry tile per block; the last block to finish sums the tile partials in
// index order, so the result does not depend on block scheduling.
__global__ void __launch_bounds__(kThreadsNA) k_dot_noalloc(const double* __restrict__ a,
                                                            const double* __restrict__ b, int64_t n,
                                                            double* __restrict__ scratch, double* __restrict__ out) {
  const int64_t base = (int64_t)blockIdx.x * kTile;
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < kTile / kThreadsNA; k++) {
    const int64_t i = base + k * kThreadsNA + threadIdx.x;
    if (i < n) acc += a[i] * b[i];
  }
  acc = block_sum_na(acc);
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + kNoAllocMaxTiles);
  __shared__ bool is_last;
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = acc;
    __threadfence();
    is_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < gridDim.x; i += blockDim.x) s += __ldcg(&scratch[i]);
  s = block_sum_na(s);
  if (threadIdx.x == 0) {
    *out = s;
    *counter = 0u;
  }
}

// errors are reported through the library's sfem_last_error()
int na_fail(int code, const std::string& msg) { return sfem::set_error(code, msg.c_str()); }

}  // namespace

extern "C" {

int sfem_dot_noalloc_dev(const double* a_dev, const double* b_dev, int64_t n, double* out_dev, void* stream) {
  if (!a_dev || !b_dev || !out_dev) return na_fail(SFEM_ERR_INVALID, "sfem_dot_noalloc_dev: null pointer");
  if (n < 0) return na_fail(SFEM_ERR_INVALID, "sfem_dot_noalloc_dev: negative length");
  const int64_t tiles = n > 0 ? (n + kTile - 1) / kTile : 1;
  if (tiles > kNoAllocMaxTiles)
    return na_fail(SFEM_ERR_INVALID, "sfem_dot_noalloc_dev: n = " + std::to_string(n) +
                                         " exceeds the maximum of 134217728 entries (65536 tiles of 2048)");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return na_fail(SFEM_ERR_NO_DEVICE, "sfem_dot_noalloc_dev: no current CUDA device");
  void* scratch = nullptr;
  {
    // one-time set-up per device (with that device current): the host-side name of a
    // __device__ array is not a device address, so ask the runtime for the address
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return na_fail(SFEM_ERR_CUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = p;
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  double* sc = static_cast<double*>(scratch);
  // the completion counter must start at zero; partials are overwritten by this call
  cudaError_t e = cudaMemsetAsync(sc + kNoAllocMaxTiles, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return na_fail(SFEM_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  k_dot_noalloc<<<(unsigned)tiles, kThreadsNA, 0, st>>>(a_dev, b_dev, n, sc, out_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(SFEM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return SFEM_OK;
}

}  // extern "C"
