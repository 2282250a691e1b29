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

// the polynomial modes' features of an offset (F = 4: 1, dx, dy, dz; F = 10: also dx^2, dy^2, dz^2,
// dx dy, dy dz, dz dx)
template <int F>
__device__ __forceinline__ void coarse_features(float dx, float dy, float dz, float (&f)[F]) {
  f[0] = 1.f;
  f[1] = dx;
  f[2] = dy;
  f[3] = dz;
  if constexpr (F == 10) {
    f[4] = dx * dx;
    f[5] = dy * dy;
    f[6] = dz * dz;
    f[7] = dx * dy;
    f[8] = dy * dz;
    f[9] = dz * dx;
  }
}

// one run's sums of B_i^T r over nodes j0 .. j1 - 1 of the staged inputs: F features per component
// (term F k + m = r[k] f_m(d))
template <int F>
__device__ __forceinline__ void coarse_run_poly(const float (*sv)[kCoarseSpan], int j0, int j1, float* acc) {
  for (int j = j0; j < j1; j++) {
    float f[F];
    coarse_features<F>(sv[3][j], sv[4][j], sv[5][j], f);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float rk = sv[k][j];
#pragma unroll
      for (int m = 0; m < F; m++) acc[F * k + m] += rk * f[m];
    }
  }
}

// the runs of restriction block b (first node base), each summed in node order by one thread from
// the staged inputs (after a barrier): the nm terms of B_i^T r per node (rigid: r, d x r; polynomial:
// r[k] f_m(d) at F k + m), to runpart[c * n_runs + k]
__device__ __forceinline__ void coarse_block_runs(const CoarseView& cv, int b, int64_t base,
                                                  const float (*sv)[kCoarseSpan]) {
  const int k1 = cv.blk_run[b + 1];
  for (int k = cv.blk_run[b] + (int)threadIdx.x; k < k1; k += (int)blockDim.x) {
    const int j0 = (int)(cv.run_start[k] - base), j1 = (int)(cv.run_start[k + 1] - base);
    float acc[30];
#pragma unroll
    for (int c = 0; c < 30; c++) acc[c] = 0.f;
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
    } else if (cv.nm == 12) {
      coarse_run_poly<4>(sv, j0, j1, acc);
    } else {
      coarse_run_poly<10>(sv, j0, j1, acc);
    }
#pragma unroll
    for (int c = 0; c < 30; c++)
      if (c < cv.nm) cv.runpart[(int64_t)c * cv.n_runs + k] = acc[c];
  }
}

template <int F>
__device__ __forceinline__ float3 coarse_prolong_poly(const float* __restrict__ ya, const float4& di) {
  float f[F];
  coarse_features<F>(di.x, di.y, di.z, f);
  float z[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float v = 0.f;
#pragma unroll
    for (int m = 0; m < F; m++) v += ya[F * k + m] * f[m];
    z[k] = v;
  }
  return make_float3(z[0], z[1], z[2]);
}

// node i's coarse prolongation term B_i y_a: rigid u + w x d_i (y_a = (u, w)); polynomial
// sum_m y_a[F k + m] f_m(d_i) per component k
__device__ __forceinline__ float3 coarse_prolong_term(const float* __restrict__ ya, const float4& di, int nm) {
  if (nm == 6)
    return make_float3(ya[0] + (ya[4] * di.z - ya[5] * di.y), ya[1] + (ya[5] * di.x - ya[3] * di.z),
                       ya[2] + (ya[3] * di.y - ya[4] * di.x));
  if (nm == 12) return coarse_prolong_poly<4>(ya, di);
  return coarse_prolong_poly<10>(ya, di);
}

}  // namespace sfem
