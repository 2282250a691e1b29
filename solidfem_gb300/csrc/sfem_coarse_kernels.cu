// Coarse-space correction of the two-level preconditioner inside the flexible-CG inner solves:
// z += P Kc^-1 P^T r with P the aggregates' rigid-body modes (an extension: the reference's
// SolveConjugateGradientMF, Math/IterativeSolvers.h:115-195, has no coarse space).
//
// In the modes' own basis B (node i's 3 x 6 block [I, -[d_i]x], d_i its offset from its aggregate's
// centroid) the correction is z_i += B_i y_a(i), y = W s with s_a = B_a^T r = (sum r_i, sum d_i x r_i)
// over the aggregate's nodes and W = R Kc^-1 R^T (6 n_agg square, formed once on the host; R the
// per-aggregate orthonormalisation with dropped modes).  Three launches per application:
//   k_coarse_restrict  one CTA per chunk of <= 256 nodes of an aggregate, fixed-order sums
//   k_coarse_gemv      one warp per row of W (the one dense contraction: a bandwidth-bound GEMV)
//   k_coarse_prolong   one thread per free node, z_i += u_a + w_a x d_i   ((u_a, w_a) = y_a); inside the
//                      flexible CG the learned preconditioner's last pass adds this term instead
// All sums run in a fixed order, so the correction is bit-identical run to run.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "sfem_internal.h"

namespace sfem {
namespace {

constexpr int kCT = 256;

__device__ __forceinline__ double warp_sum_c(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// s_a = (sum r_i, sum d_i x r_i) over aggregate a's nodes: one CTA per chunk of at most 256 nodes of
// one aggregate (one node per thread), the chunk's six sums to cpart; the aggregate's last chunk to
// finish adds its chunks' sums in chunk order (a fixed order, so s is the same on every run) and
// resets the aggregate's counter
__global__ void __launch_bounds__(kCT) k_coarse_restrict(CoarseView cv, const float* __restrict__ r) {
  // FP32 within a warp (GB300's FP64 rate is a small fraction of FP32), the eight warp sums in FP64
  const int c = blockIdx.x;
  const int a = cv.chunk_agg[c];
  float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if ((int)threadIdx.x < cv.chunk_cnt[c]) {
    const int i = cv.agg_node[cv.chunk_start[c] + threadIdx.x];
    const float4 di = cv.d[i];
    const float r0 = r[3 * (int64_t)i], r1 = r[3 * (int64_t)i + 1], r2 = r[3 * (int64_t)i + 2];
    acc[0] = r0;
    acc[1] = r1;
    acc[2] = r2;
    acc[3] = di.y * r2 - di.z * r1;
    acc[4] = di.z * r0 - di.x * r2;
    acc[5] = di.x * r1 - di.y * r0;
  }
  __shared__ float sm[6][kCT / 32];
  __shared__ bool is_last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    float v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sm[k][w] = v;
  }
  __syncthreads();
  if (w == 0) {
    if (lane < 6) {
      double v = 0.0;
#pragma unroll
      for (int q = 0; q < kCT / 32; q++) v += (double)sm[lane][q];
      cv.cpart[6 * (int64_t)c + lane] = v;
      __threadfence();  // each writer orders its own partial before the count below
    }
    __syncwarp();
    if (lane == 0) {
      const unsigned n = (unsigned)(cv.agg_chunk[a + 1] - cv.agg_chunk[a]);
      is_last = atomicAdd(cv.ccount + a, 1u) == n - 1;
    }
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (threadIdx.x < 6) {
    double v = 0.0;
    for (int k = cv.agg_chunk[a]; k < cv.agg_chunk[a + 1]; k++) v += __ldcg(cv.cpart + 6 * (int64_t)k + threadIdx.x);
    cv.s[6 * a + threadIdx.x] = (float)v;
  }
  if (threadIdx.x == 0) cv.ccount[a] = 0u;
}

// y = W s, W row-major nc x ld (FP32, ld a multiple of 4, zero beyond nc; s zero beyond nc), one warp
// per row reading 16-byte column groups
__global__ void __launch_bounds__(kCT) k_coarse_gemv(int nc, int ld, const float* __restrict__ W,
                                                     const float* __restrict__ s, float* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int row = (int)((blockIdx.x * (int64_t)kCT + threadIdx.x) >> 5);
  if (row >= nc) return;
  const float4* Wr = reinterpret_cast<const float4*>(W + (int64_t)row * ld);
  const float4* s4 = reinterpret_cast<const float4*>(s);
  double acc = 0.0;
  for (int c = lane; c < ld / 4; c += 32) {
    const float4 wv = Wr[c], sv = s4[c];
    acc += (double)(wv.x * sv.x + wv.y * sv.y + wv.z * sv.z + wv.w * sv.w);
  }
  acc = warp_sum_c(acc);
  if (lane == 0) y[row] = (float)acc;
}

// z_i += u_a + w_a x d_i over the free nodes
__global__ void __launch_bounds__(kCT) k_coarse_prolong(int64_t nf, const int32_t* __restrict__ aid,
                                                        const float4* __restrict__ d, const float* __restrict__ y,
                                                        float* __restrict__ z) {
  for (int64_t i = (int64_t)blockIdx.x * kCT + threadIdx.x; i < nf; i += (int64_t)gridDim.x * kCT) {
    const float* ya = y + 6 * (int64_t)aid[i];
    const float4 di = d[i];
    const float u0 = ya[0], u1 = ya[1], u2 = ya[2], w0 = ya[3], w1 = ya[4], w2 = ya[5];
    z[3 * i] += u0 + (w1 * di.z - w2 * di.y);
    z[3 * i + 1] += u1 + (w2 * di.x - w0 * di.z);
    z[3 * i + 2] += u2 + (w0 * di.y - w1 * di.x);
  }
}

}  // namespace

void launch_coarse_restrict_gemv(const CoarseView& cv, const float* r, cudaStream_t st) {
  count_launch();
  k_coarse_restrict<<<cv.n_chunks, kCT, 0, st>>>(cv, r);
  count_launch();
  const int nc = 6 * cv.n_agg;
  k_coarse_gemv<<<(unsigned)((nc * 32 + kCT - 1) / kCT), kCT, 0, st>>>(nc, cv.ld, cv.W, cv.s, cv.y);
}

void launch_coarse_apply(const CoarseView& cv, const float* r, float* z, cudaStream_t st) {
  launch_coarse_restrict_gemv(cv, r, st);
  count_launch();
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (cv.nf + kCT - 1) / kCT;
  const unsigned grid = (unsigned)std::min<int64_t>(want > 0 ? want : 1, (int64_t)sms * 8);
  k_coarse_prolong<<<grid, kCT, 0, st>>>(cv.nf, cv.aid, cv.d, cv.y, z);
}

}  // namespace sfem
