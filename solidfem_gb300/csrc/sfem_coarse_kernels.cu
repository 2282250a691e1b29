// Coarse-space correction of the two-level preconditioner inside the flexible-CG inner solves:
// z += P Kc^-1 P^T r with P the aggregates' rigid-body modes (an extension: the reference's
// SolveConjugateGradientMF, Math/IterativeSolvers.h:115-195, has no coarse space).
//
// In the modes' own basis B (node i's 3 x 6 block [I, -[d_i]x], d_i its offset from its aggregate's
// centroid) the correction is z_i += B_i y_a(i), y = W s with s_a = B_a^T r = (sum r_i, sum d_i x r_i)
// over the aggregate's nodes and W = R Kc^-1 R^T (6 n_agg square, formed once on the host in FP64 and
// stored in FP16 times a power of two; R the per-aggregate orthonormalisation with dropped modes).  Four launches per application:
//   k_coarse_runs      one CTA per block of 1024 consecutive free nodes (coalesced loads of r and d into
//                      shared memory), one thread per run of the block: the run's six sums
//   k_coarse_aggsum    one CTA per aggregate: the sums of its runs, s_a
//   k_coarse_gemv      one warp per row of W (the one dense contraction: a bandwidth-bound GEMV)
//   k_coarse_prolong   one thread per free node, z_i += u_a + w_a x d_i   ((u_a, w_a) = y_a); inside the
//                      flexible CG the learned preconditioner's last pass adds this term instead
// All sums run in a fixed order, so the correction is bit-identical run to run.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "sfem_coarse.cuh"
#include "sfem_internal.h"

namespace sfem {
namespace {

constexpr int kCT = 256;

// Run sums of s_a = B_a^T r: restriction block b (coarse_block_start, up to kCoarseSpan free nodes), its
// nodes' r and d staged in shared memory by coalesced loads; then each run of the block summed in node
// order by one thread (coarse_block_runs), to runpart[c * n_runs + k]
__global__ void __launch_bounds__(kCT) k_coarse_runs(CoarseView cv, const float* __restrict__ r) {
  __shared__ float sv[6][kCoarseSpan];
  const int64_t base = coarse_block_start(blockIdx.x, cv.n_blocks, cv.blk_off, cv.nf);
  const int cnt = (int)(coarse_block_start(blockIdx.x + 1, cv.n_blocks, cv.blk_off, cv.nf) - base);
  for (int t = threadIdx.x; t < cnt; t += kCT) {
    const int64_t i = base + t;
    coarse_stage(cv, i, base, r[3 * i], r[3 * i + 1], r[3 * i + 2], sv);
  }
  __syncthreads();
  coarse_block_runs(cv, blockIdx.x, base, sv);
}

// s_a from aggregate a's run sums (nm per run): one CTA per aggregate, thread t adding runs t, t + 256,
// ... of the aggregate's list in order (one run each for aggregates of up to 256 runs), then fixed
// butterflies within the warps and the eight warp sums in warp order (the same order on every run)
__global__ void __launch_bounds__(kCT) k_coarse_aggsum(CoarseView cv) {
  __shared__ float ws[30][kCT / 32];
  const int a = blockIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nm = cv.nm;
  float acc[30];
#pragma unroll
  for (int c = 0; c < 30; c++) acc[c] = 0.f;
  const int q1 = cv.agg_run_ptr[a + 1];
  for (int q = cv.agg_run_ptr[a] + threadIdx.x; q < q1; q += kCT) {
    const int k = cv.agg_run[q];
#pragma unroll
    for (int c = 0; c < 30; c++)
      if (c < nm) acc[c] += cv.runpart[(int64_t)c * cv.n_runs + k];
  }
#pragma unroll
  for (int c = 0; c < 30; c++) {
    if (c >= nm) break;
    float v = acc[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) ws[c][w] = v;
  }
  __syncthreads();
  if ((int)threadIdx.x < nm) {
    float v = 0.f;
#pragma unroll
    for (int k = 0; k < kCT / 32; k++) v += ws[threadIdx.x][k];
    cv.s[nm * a + threadIdx.x] = v;
  }
}

// y = W s: W row-major nc x ld FP16 (scaled by 1 / inv_scale; ld a multiple of 8, zero beyond nc), s FP32
// (zero beyond nc).  One warp per row, each lane eight columns per 16-byte load and eight loads in
// flight (a row of 5,184 columns is three rounds); FP32 sums in a fixed order (lane partials, then a
// butterfly)
__device__ __forceinline__ float dot8(const uint4& w, const float4& a, const float4& b) {
  const float2 w0 = __half22float2(*reinterpret_cast<const __half2*>(&w.x));
  const float2 w1 = __half22float2(*reinterpret_cast<const __half2*>(&w.y));
  const float2 w2 = __half22float2(*reinterpret_cast<const __half2*>(&w.z));
  const float2 w3 = __half22float2(*reinterpret_cast<const __half2*>(&w.w));
  return ((w0.x * a.x + w0.y * a.y) + (w1.x * a.z + w1.y * a.w)) + ((w2.x * b.x + w2.y * b.y) + (w3.x * b.z + w3.y * b.w));
}
__global__ void __launch_bounds__(kCT) k_coarse_gemv(int nc, int ld, const __half* __restrict__ W, float inv_scale,
                                                     const float* __restrict__ s, float* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int row = (int)((blockIdx.x * (int64_t)kCT + threadIdx.x) >> 5);
  if (row >= nc) return;
  const uint4* Wr = reinterpret_cast<const uint4*>(W + (int64_t)row * ld);
  const float4* s4 = reinterpret_cast<const float4*>(s);
  const int n8 = ld / 8;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  int c = lane;
  for (; c + 224 < n8; c += 256) {
    uint4 w[8];
#pragma unroll
    for (int u = 0; u < 8; u++) w[u] = __ldcs(Wr + c + 32 * u);
#pragma unroll
    for (int u = 0; u < 8; u++) acc[u & 3] += dot8(w[u], s4[2 * (c + 32 * u)], s4[2 * (c + 32 * u) + 1]);
  }
  for (; c + 96 < n8; c += 128) {
    uint4 w[4];
#pragma unroll
    for (int u = 0; u < 4; u++) w[u] = __ldcs(Wr + c + 32 * u);
#pragma unroll
    for (int u = 0; u < 4; u++) acc[u] += dot8(w[u], s4[2 * (c + 32 * u)], s4[2 * (c + 32 * u) + 1]);
  }
  for (; c < n8; c += 32) acc[0] += dot8(__ldcs(Wr + c), s4[2 * c], s4[2 * c + 1]);
  float v = (acc[0] + acc[1]) + (acc[2] + acc[3]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) y[row] = v * inv_scale;
}

// z_i += B_i y_a over the free nodes (coarse_prolong_term)
__global__ void __launch_bounds__(kCT) k_coarse_prolong(int64_t nf, int nm, const int32_t* __restrict__ aid,
                                                        const float4* __restrict__ d, const float* __restrict__ y,
                                                        float* __restrict__ z) {
  for (int64_t i = (int64_t)blockIdx.x * kCT + threadIdx.x; i < nf; i += (int64_t)gridDim.x * kCT) {
    const float3 t = coarse_prolong_term(y + (int64_t)nm * aid[i], d[i], nm);
    z[3 * i] += t.x;
    z[3 * i + 1] += t.y;
    z[3 * i + 2] += t.z;
  }
}

}  // namespace

void launch_coarse_restrict_gemv(const CoarseView& cv, const float* r, cudaStream_t st) {
  // ordinary launches: with programmatic dependent launch the next kernel's waiting CTAs took the
  // slots of these grids' later CTAs (measured: 73 us more per flexible-CG iteration at 6.3M tets)
  if (cv.n_blocks <= 0) return;
  count_launch();
  k_coarse_runs<<<(unsigned)cv.n_blocks, kCT, 0, st>>>(cv, r);
  launch_coarse_sum_gemv(cv, st);
}

void launch_coarse_sum_gemv(const CoarseView& cv, cudaStream_t st) {
  if (cv.n_blocks <= 0) return;
  count_launch();
  k_coarse_aggsum<<<(unsigned)cv.n_agg, kCT, 0, st>>>(cv);
  count_launch();
  const int nc = cv.nm * cv.n_agg;
  k_coarse_gemv<<<(unsigned)((nc * 32 + kCT - 1) / kCT), kCT, 0, st>>>(nc, cv.ld, cv.W, cv.w_inv_scale, cv.s, cv.y);
}

void launch_coarse_apply(const CoarseView& cv, const float* r, float* z, cudaStream_t st) {
  launch_coarse_restrict_gemv(cv, r, st);
  count_launch();
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (cv.nf + kCT - 1) / kCT;
  const unsigned grid = (unsigned)std::min<int64_t>(want > 0 ? want : 1, (int64_t)sms * 8);
  k_coarse_prolong<<<grid, kCT, 0, st>>>(cv.nf, cv.nm, cv.aid, cv.d, cv.y, z);
}

}  // namespace sfem
