// Fixed-order sums of per-block partials, read by the last block of a grid.
#pragma once
#include <cuda_runtime.h>

namespace sfem {

// s[k] += P[k * stride + i] for i = threadIdx.x, threadIdx.x + blockDim.x, ... < n, added in
// that order (the same result as the plain strided loop).  The partials are read with L2 loads,
// eight values (B terms of all K sums) before any of them is added, so one thread waits for
// about n / (B * blockDim.x) L2 round trips instead of K * n / blockDim.x.
template <typename A, typename P, int K>
__device__ __forceinline__ void strided_sums(const P* part, unsigned stride, unsigned n, A (&s)[K]) {
  constexpr int B = K >= 8 ? 1 : 8 / K;
  for (unsigned i0 = threadIdx.x; i0 < n; i0 += B * blockDim.x) {
    P q[K][B];
#pragma unroll
    for (int j = 0; j < B; j++) {
      const unsigned i = i0 + j * blockDim.x;
#pragma unroll
      for (int k = 0; k < K; k++) q[k][j] = i < n ? __ldcg(&part[k * stride + i]) : P(0);
    }
#pragma unroll
    for (int j = 0; j < B; j++) {
      if (i0 + j * blockDim.x < n) {
#pragma unroll
        for (int k = 0; k < K; k++) s[k] += (A)q[k][j];
      }
    }
  }
}

}  // namespace sfem
