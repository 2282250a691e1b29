// Device helpers of the coarse restriction shared by k_coarse_runs and the flexible-CG update that
// forms the run sums itself (two-level preconditioner; the layout is described at CoarseView).
#pragma once
#include <cuda_runtime.h>

#include "sfem_internal.h"

namespace sfem {

// free node f's restriction inputs, r and its offset d_f, into column f - base of sv
__device__ __forceinline__ void coarse_stage(const CoarseView& cv, int64_t f, int64_t base, float r0, float r1, float r2,
                                             float (*sv)[kCoarseSpan]) {
  const float4 di = cv.d[f];
  const int t = (int)(f - base);
  sv[0][t] = r0;
  sv[1][t] = r1;
  sv[2][t] = r2;
  sv[3][t] = di.x;
  sv[4][t] = di.y;
  sv[5][t] = di.z;
}

// the runs of restriction block b (first node base), each summed in node order by one thread from
// the staged inputs (after a barrier): the nm terms of B_i^T r per node (rigid: r, d x r; affine: r,
// r[k] d[l] at 3 + 3 k + l), to runpart[c * n_runs + k]
__device__ __forceinline__ void coarse_block_runs(const CoarseView& cv, int b, int64_t base,
                                                  const float (*sv)[kCoarseSpan]) {
  const int k1 = cv.blk_run[b + 1];
  for (int k = cv.blk_run[b] + (int)threadIdx.x; k < k1; k += (int)blockDim.x) {
    const int j0 = (int)(cv.run_start[k] - base), j1 = (int)(cv.run_start[k + 1] - base);
    float acc[12] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (cv.nm == 6) {
      for (int j = j0; j < j1; j++) {
        const float r0 = sv[0][j], r1 = sv[1][j], r2 = sv[2][j], dx = sv[3][j], dy = sv[4][j], dz = sv[5][j];
        acc[0] += r0;
        acc[1] += r1;
        acc[2] += r2;
        acc[3] += dy * r2 - dz * r1;
        acc[4] += dz * r0 - dx * r2;
        acc[5] += dx * r1 - dy * r0;
      }
    } else {
      for (int j = j0; j < j1; j++) {
        const float r[3] = {sv[0][j], sv[1][j], sv[2][j]}, dd[3] = {sv[3][j], sv[4][j], sv[5][j]};
#pragma unroll
        for (int c = 0; c < 3; c++) {
          acc[c] += r[c];
#pragma unroll
          for (int l = 0; l < 3; l++) acc[3 + 3 * c + l] += r[c] * dd[l];
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 12; c++)
      if (c < cv.nm) cv.runpart[(int64_t)c * cv.n_runs + k] = acc[c];
  }
}

// node i's coarse prolongation term B_i y_a: rigid u + w x d_i (y_a = (u, w)); affine u + A d_i (y_a = (u,
// A row-major))
__device__ __forceinline__ float3 coarse_prolong_term(const float* __restrict__ ya, const float4& di, int nm) {
  if (nm == 6)
    return make_float3(ya[0] + (ya[4] * di.z - ya[5] * di.y), ya[1] + (ya[5] * di.x - ya[3] * di.z),
                       ya[2] + (ya[3] * di.y - ya[4] * di.x));
  return make_float3(ya[0] + (ya[3] * di.x + ya[4] * di.y + ya[5] * di.z),
                     ya[1] + (ya[6] * di.x + ya[7] * di.y + ya[8] * di.z),
                     ya[2] + (ya[9] * di.x + ya[10] * di.y + ya[11] * di.z));
}

}  // namespace sfem
