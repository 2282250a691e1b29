// Device helpers of the coarse restriction shared by k_coarse_runs and the flexible-CG update that
// forms the run sums itself (two-level preconditioner; the layout is described at CoarseView).
#pragma once
#include <cuda_runtime.h>

#include "sfem_internal.h"

namespace sfem {

// free node f's six restriction terms (r, d_f x r) into column f - base of sv
__device__ __forceinline__ void coarse_stage(const CoarseView& cv, int64_t f, int64_t base, float r0, float r1, float r2,
                                             float (*sv)[kCoarseSpan]) {
  const float4 di = cv.d[f];
  const int t = (int)(f - base);
  sv[0][t] = r0;
  sv[1][t] = r1;
  sv[2][t] = r2;
  sv[3][t] = di.y * r2 - di.z * r1;
  sv[4][t] = di.z * r0 - di.x * r2;
  sv[5][t] = di.x * r1 - di.y * r0;
}

// the runs of restriction block b (first node base), each summed in node order by one thread from
// the staged terms (after a barrier), to runpart[c * n_runs + k]
__device__ __forceinline__ void coarse_block_runs(const CoarseView& cv, int b, int64_t base,
                                                  const float (*sv)[kCoarseSpan]) {
  const int k1 = cv.blk_run[b + 1];
  for (int k = cv.blk_run[b] + (int)threadIdx.x; k < k1; k += (int)blockDim.x) {
    const int j0 = (int)(cv.run_start[k] - base), j1 = (int)(cv.run_start[k + 1] - base);
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int j = j0; j < j1; j++)
#pragma unroll
      for (int c = 0; c < 6; c++) acc[c] += sv[c][j];
#pragma unroll
    for (int c = 0; c < 6; c++) cv.runpart[(int64_t)c * cv.n_runs + k] = acc[c];
  }
}

}  // namespace sfem
