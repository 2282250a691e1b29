// FP16 node rows of the learned preconditioner's polynomial passes (Row16, sfem_gnn.h): packing,
// unpacking and the power-of-two scale that keeps the rows inside FP16's range.
#pragma once
#include <cuda_fp16.h>

#include "sfem_gnn.h"

namespace sfem {
namespace gnn {

__device__ __forceinline__ Row16 pack16(float x, float y, float z) {
  const __half2 a = __floats2half2_rn(x, y), b = __floats2half2_rn(z, 0.f);
  Row16 v;
  v.xy = *reinterpret_cast<const uint32_t*>(&a);
  v.z0 = *reinterpret_cast<const uint32_t*>(&b);
  return v;
}

__device__ __forceinline__ float3 unpack16(const Row16& v) {
  const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&v.xy));
  const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&v.z0));
  return make_float3(a.x, a.y, b.x);
}

// sigma = 2^k with the rows' RMS sqrt(xx / n3) times sigma in [1/8, 1/4); 1 when xx is not a
// positive number.  Over a flexible-CG solve the rows' largest entry stays far below FP16's 65504
// at this RMS, and entries below FP16's normal range carry a negligible share of the sums.
__device__ __forceinline__ float row16_scale(float xx, int64_t n3) {
  if (!(xx > 0.f) || !isfinite(xx) || n3 <= 0) return 1.f;
  const float rms = sqrtf(xx / (float)n3);
  int k = -ilogbf(rms) - 3;
  k = k < -126 ? -126 : (k > 126 ? 126 : k);
  return ldexpf(1.f, k);
}

}  // namespace gnn
}  // namespace sfem
