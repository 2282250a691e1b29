// Device kernels of the learned graph-network preconditioner (included by sfem_gnn.cu).
//
// The preconditioner is symmetric positive definite by construction:
//   x      = D^-1/2 r                                        (per free DOF)
//   S x    : h0_i = We x_i;  h_i <- h_i + Wl [h_i ; mean_{j in N(i)} h_j]   l = 1..3
//   M(r)   = D^-1/2 (c x + S^T S x),   c = exp(log c) > 0
// S is a linear message-passing network of width H = 64 on the free-node mesh graph, so
// M is one fixed SPD operator per tangent (conjugate gradients keep their guarantees);
// S^T runs the same layers transposed (the input-gradient propagation of S).
// Activations of S are stored in BF16, GEMMs run on the tensor cores (mma.sync m16n8k16,
// BF16 inputs, FP32 accumulation), the transposed pass carries FP32 vectors.  Weight-gradient
// kernels write per-CTA partials that are summed in a fixed order (deterministic).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sfem_gnn.h"
#include "sfem_pdl.cuh"
#include "sfem_reduce.cuh"
#include "sfem_row16.cuh"
#include "sfem_coarse.cuh"

namespace sfem {
namespace gnn {

__device__ __forceinline__ void mma_bf16(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ float2 bf2f(uint32_t v) {
  __nv_bfloat162 b = *reinterpret_cast<__nv_bfloat162*>(&v);
  return __bfloat1622float2(b);
}
__device__ __forceinline__ uint32_t f2bf(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

// two consecutive features of row `node` (64 wide) as floats, from BF16 or FP32 storage
__device__ __forceinline__ float2 load2(const __nv_bfloat16* a, int64_t node, int col) {
  return bf2f(reinterpret_cast<const uint32_t*>(a)[(node * H + col) >> 1]);
}
__device__ __forceinline__ float2 load2(const float* a, int64_t node, int col) {
  return *reinterpret_cast<const float2*>(&a[node * H + col]);
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sumd(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sums of K values into partials[k * gridDim.x + blockIdx.x]; the last block to finish
// adds them in a fixed order (thread t takes blocks t, t + 256, ... in FP64, then a fixed
// shuffle tree) and returns true with tot[] valid in its thread 0.  256 threads per block.
template <int K>
__device__ __forceinline__ bool last_block_sums(float (&v)[K], float* partials, unsigned* counter, double (&tot)[K]) {
  __shared__ float sm[K][8];
  __shared__ double sd[K][8];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    const float a = warp_sumf(v[k]);
    if (lane == 0) sm[k][w] = a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      float b = 0.f;
      for (int q = 0; q < 8; q++) b += sm[k][q];
      partials[k * gridDim.x + blockIdx.x] = b;
    }
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double a[K];
#pragma unroll
  for (int k = 0; k < K; k++) a[k] = 0.0;
  strided_sums<double, float, K>(partials, gridDim.x, gridDim.x, a);
#pragma unroll
  for (int k = 0; k < K; k++) {
    const double b = warp_sumd(a[k]);
    if (lane == 0) sd[k][w] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      double a = 0.0;
      for (int q = 0; q < 8; q++) a += sd[k][q];
      tot[k] = a;
    }
    *counter = 0u;
  }
  return true;
}

// ---- encoder: x = v * D^-1/2, h0 = We x; one warp per node, lane l computes outputs 2l, 2l+1 ----
__global__ void __launch_bounds__(256) k_gnn_encode(int64_t n, const float* __restrict__ v,
                                                    const float* __restrict__ dinv,
                                                    const float* __restrict__ params,
                                                    __nv_bfloat16* __restrict__ h0, float* __restrict__ xout,
                                                    const int* done) {
  if (done && *done) return;
  const int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (node >= n) return;
  float x[FIN];
#pragma unroll
  for (int c = 0; c < FIN; c++) x[c] = v[FIN * node + c] * sqrtf(dinv[FIN * node + c]);
  if (xout && lane < FIN) xout[FIN * node + lane] = x[lane];
  float a[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int o = 2 * lane + k;
    float acc = 0.f;
#pragma unroll
    for (int f = 0; f < FIN; f++) acc += params[OFF_WE + o * FIN + f] * x[f];
    a[k] = acc;
  }
  reinterpret_cast<uint32_t*>(h0)[node * (H / 2) + lane] = f2bf(a[0], a[1]);
}

// ---- message-passing layer of S: h_out = h_in + Wl [h_in ; mean_j h_j] ----
// CTA: 64 nodes, 4 warps x 16 nodes.  Shared A tile [64 x (h ; mean h)] and Wl [64 x 128].
__global__ void __launch_bounds__(LT) k_gnn_layer_fwd(Graph g, const __nv_bfloat16* __restrict__ hin,
                                                      const __nv_bfloat16* __restrict__ W,  // [H][AIN]
                                                      __nv_bfloat16* __restrict__ hout, const int* done) {
  if (done && *done) return;
  __shared__ __align__(16) __nv_bfloat16 As[TILE * SROW];
  __shared__ __align__(16) __nv_bfloat16 Ws[H * SROW];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * TILE;
  // weights: 64 rows x 128 bf16 = 16 uint4 per row
  for (int i = tid; i < H * (AIN / 8); i += LT) {
    const int row = i / (AIN / 8), c8 = i % (AIN / 8);
    *reinterpret_cast<uint4*>(&Ws[row * SROW + 8 * c8]) = reinterpret_cast<const uint4*>(W)[row * (AIN / 8) + c8];
  }
  // gather [h_i ; mean_j h_j] for this warp's 16 nodes; lane handles features 2l, 2l+1
  const uint32_t* h32 = reinterpret_cast<const uint32_t*>(hin);
  for (int rr = 0; rr < 16; rr++) {
    const int row = 16 * w + rr;
    const int64_t node = base + row;
    uint32_t self = 0, msg = 0;
    if (node < g.n) {
      self = h32[node * (H / 2) + lane];
      float m0 = 0.f, m1 = 0.f;
      const int e1 = g.ptr[node + 1];
      for (int e = g.ptr[node]; e < e1; e++) {
        const float2 v = bf2f(h32[(int64_t)g.idx[e] * (H / 2) + lane]);
        m0 += v.x;
        m1 += v.y;
      }
      const float id = g.inv_deg[node];
      msg = f2bf(m0 * id, m1 * id);
    }
    *reinterpret_cast<uint32_t*>(&As[row * SROW + 2 * lane]) = self;
    *reinterpret_cast<uint32_t*>(&As[row * SROW + H + 2 * lane]) = msg;
  }
  __syncthreads();
  const int gq = lane >> 2, t4 = lane & 3;
  float acc[8][4];
#pragma unroll
  for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  const __nv_bfloat16* Ar0 = &As[(16 * w + gq) * SROW];
  const __nv_bfloat16* Ar1 = &As[(16 * w + gq + 8) * SROW];
#pragma unroll
  for (int kk = 0; kk < AIN / 16; kk++) {
    const int k0 = 16 * kk + 2 * t4;
    const uint32_t a0 = ld32(Ar0 + k0), a1 = ld32(Ar1 + k0), a2 = ld32(Ar0 + k0 + 8), a3 = ld32(Ar1 + k0 + 8);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const __nv_bfloat16* Wr = &Ws[(8 * j + gq) * SROW + k0];
      mma_bf16(acc[j], a0, a1, a2, a3, ld32(Wr), ld32(Wr + 8));
    }
  }
  // epilogue: rows gq and gq + 8 of this warp, cols 8j + 2 t4 + {0,1}
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int row = 16 * w + gq + 8 * half;
    const int64_t node = base + row;
    if (node >= g.n) continue;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int col = 8 * j + 2 * t4;
      const float2 hs = bf2f(ld32(&As[row * SROW + col]));
      reinterpret_cast<uint32_t*>(hout)[node * (H / 2) + col / 2] =
          f2bf(hs.x + acc[j][2 * half], hs.y + acc[j][2 * half + 1]);
    }
  }
}

// ---- transposed layer (and, with WGRAD, its weight gradient) ----
// For h_out = h_in + Wl a, a = [h_in ; mean h_in] and a cotangent G_out = dL/dh_out:
//   g_a = G_out Wl  ->  G_self = G_out + g_a[:, :H],  G_msg = g_a[:, H:] / deg
//   (dL/dh_in = G_self + mean-aggregation^T of G_msg, formed by k_gnn_msg_scatter)
//   WGRAD: partial dWl = G_out^T a over the tile's nodes.
// Wt is Wl transposed ([AIN][H], bf16).  Dynamic shared memory (layer_bwd_smem).
template <bool WGRAD, typename GT>
__global__ void __launch_bounds__(LT) k_gnn_layer_bwd(Graph g, const __nv_bfloat16* __restrict__ hin,
                                                      const GT* __restrict__ Gout,
                                                      const __nv_bfloat16* __restrict__ Wt,
                                                      float* __restrict__ Gself, float* __restrict__ Gmsg,
                                                      float* __restrict__ partial /* [grid][LPART] */,
                                                      const int* done) {
  if (done && *done) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  __nv_bfloat16* gu = reinterpret_cast<__nv_bfloat16*>(smraw);  // [TILE][SROW64]  node-major
  __nv_bfloat16* Ws = gu + TILE * SROW64;                        // [AIN][SROW64]   = Wt
  __nv_bfloat16* guT = Ws + AIN * SROW64;                        // [H][SROW64]     out-major (WGRAD)
  __nv_bfloat16* aT = guT + H * SROW64;                          // [AIN][SROW64]   in-major  (WGRAD)
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * TILE;
  for (int i = tid; i < AIN * (H / 8); i += LT) {
    const int row = i / (H / 8), c8 = i % (H / 8);
    *reinterpret_cast<uint4*>(&Ws[row * SROW64 + 8 * c8]) = reinterpret_cast<const uint4*>(Wt)[row * (H / 8) + c8];
  }
  const uint32_t* h32 = reinterpret_cast<const uint32_t*>(hin);
  for (int rr = 0; rr < 16; rr++) {
    const int row = 16 * w + rr;
    const int64_t node = base + row;
    float2 gv = make_float2(0.f, 0.f);
    if (node < g.n) gv = load2(Gout, node, 2 * lane);
    const uint32_t gb = f2bf(gv.x, gv.y);
    *reinterpret_cast<uint32_t*>(&gu[row * SROW64 + 2 * lane]) = gb;
    if (WGRAD) {
      uint32_t self = 0, msg = 0;
      if (node < g.n) {
        self = h32[node * (H / 2) + lane];
        float m0 = 0.f, m1 = 0.f;
        const int e1 = g.ptr[node + 1];
        for (int e = g.ptr[node]; e < e1; e++) {
          const float2 v = bf2f(h32[(int64_t)g.idx[e] * (H / 2) + lane]);
          m0 += v.x;
          m1 += v.y;
        }
        const float id = g.inv_deg[node];
        msg = f2bf(m0 * id, m1 * id);
      }
      const __nv_bfloat162 gbb = *reinterpret_cast<const __nv_bfloat162*>(&gb);
      guT[(2 * lane) * SROW64 + row] = gbb.x;
      guT[(2 * lane + 1) * SROW64 + row] = gbb.y;
      const __nv_bfloat162 sb = *reinterpret_cast<const __nv_bfloat162*>(&self);
      const __nv_bfloat162 mb = *reinterpret_cast<const __nv_bfloat162*>(&msg);
      aT[(2 * lane) * SROW64 + row] = sb.x;
      aT[(2 * lane + 1) * SROW64 + row] = sb.y;
      aT[(H + 2 * lane) * SROW64 + row] = mb.x;
      aT[(H + 2 * lane + 1) * SROW64 + row] = mb.y;
    }
  }
  __syncthreads();
  const int gq = lane >> 2, t4 = lane & 3;
  // ---- g_a [64 nodes x 128] = gu [64 x 64] . Wl [64 x 128]; B[k][n] = Wt[n][k] ----
  {
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const __nv_bfloat16* Ar0 = &gu[(16 * w + gq) * SROW64];
    const __nv_bfloat16* Ar1 = &gu[(16 * w + gq + 8) * SROW64];
#pragma unroll
    for (int kk = 0; kk < H / 16; kk++) {
      const int k0 = 16 * kk + 2 * t4;
      const uint32_t a0 = ld32(Ar0 + k0), a1 = ld32(Ar1 + k0), a2 = ld32(Ar0 + k0 + 8), a3 = ld32(Ar1 + k0 + 8);
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const __nv_bfloat16* Br = &Ws[(8 * j + gq) * SROW64 + k0];
        mma_bf16(acc[j], a0, a1, a2, a3, ld32(Br), ld32(Br + 8));
      }
    }
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int row = 16 * w + gq + 8 * half;
      const int64_t node = base + row;
      if (node >= g.n) continue;
      const float id = g.inv_deg[node];
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const int col = 8 * j + 2 * t4;
        const float v0 = acc[j][2 * half], v1 = acc[j][2 * half + 1];
        if (col < H) {
          const float2 go = load2(Gout, node, col);
          *reinterpret_cast<float2*>(&Gself[node * H + col]) = make_float2(go.x + v0, go.y + v1);
        } else {
          *reinterpret_cast<float2*>(&Gmsg[node * H + col - H]) = make_float2(v0 * id, v1 * id);
        }
      }
    }
  }
  if constexpr (WGRAD) {
  // ---- dWl partial [64 out x 128 in] = guT [64 x 64 nodes] . a [64 nodes x 128]; B[k][n] = aT[n][k] ----
  float acc[16][4];
#pragma unroll
  for (int j = 0; j < 16; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  const __nv_bfloat16* Ar0 = &guT[(16 * w + gq) * SROW64];
  const __nv_bfloat16* Ar1 = &guT[(16 * w + gq + 8) * SROW64];
#pragma unroll
  for (int kk = 0; kk < TILE / 16; kk++) {
    const int k0 = 16 * kk + 2 * t4;
    const uint32_t a0 = ld32(Ar0 + k0), a1 = ld32(Ar1 + k0), a2 = ld32(Ar0 + k0 + 8), a3 = ld32(Ar1 + k0 + 8);
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const __nv_bfloat16* Br = &aT[(8 * j + gq) * SROW64 + k0];
      mma_bf16(acc[j], a0, a1, a2, a3, ld32(Br), ld32(Br + 8));
    }
  }
  float* P = partial + (int64_t)blockIdx.x * LPART;
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int o = 16 * w + gq + 8 * half;
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int col = 8 * j + 2 * t4;
      *reinterpret_cast<float2*>(&P[o * AIN + col]) = make_float2(acc[j][2 * half], acc[j][2 * half + 1]);
    }
  }
  }
}
__host__ __device__ constexpr size_t layer_bwd_smem(bool wgrad) {
  return sizeof(__nv_bfloat16) * (TILE * SROW64 + AIN * SROW64 + (wgrad ? H * SROW64 + AIN * SROW64 : 0));
}

// G_in[j] = G_self[j] + sum_{i in N(j)} G_msg[i]   (mean aggregation transposed; symmetric graph)
__global__ void __launch_bounds__(256) k_gnn_msg_scatter(Graph g, const float* __restrict__ Gself,
                                                         const float* __restrict__ Gmsg, float* __restrict__ Gin,
                                                         const int* done) {
  if (done && *done) return;
  const int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (node >= g.n) return;
  float2 a = *reinterpret_cast<const float2*>(&Gself[node * H + 2 * lane]);
  const int e1 = g.ptr[node + 1];
  for (int e = g.ptr[node]; e < e1; e++) {
    const float2 v = *reinterpret_cast<const float2*>(&Gmsg[(int64_t)g.idx[e] * H + 2 * lane]);
    a.x += v.x;
    a.y += v.y;
  }
  *reinterpret_cast<float2*>(&Gin[node * H + 2 * lane]) = a;
}

// ---- output: M(r) = D^-1/2 (c x + We^T G0) with x = D^-1/2 r; one warp per node ----
__global__ void __launch_bounds__(256) k_gnn_decode(int64_t n, const float* __restrict__ G0,
                                                    const float* __restrict__ params, const float* __restrict__ r,
                                                    const float* __restrict__ dinv, float* __restrict__ out,
                                                    const int* done) {
  if (done && *done) return;
  const int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (node >= n) return;
  const float2 gv = *reinterpret_cast<const float2*>(&G0[node * H + 2 * lane]);
  float y[FIN];
#pragma unroll
  for (int c = 0; c < FIN; c++)
    y[c] = warp_sumf(gv.x * params[OFF_WE + (2 * lane) * FIN + c] + gv.y * params[OFF_WE + (2 * lane + 1) * FIN + c]);
  if (lane < FIN) {
    const int64_t i = FIN * node + lane;
    const float cc = expf(params[OFF_C]);
    const float d = dinv[i];
    out[i] = cc * d * r[i] + sqrtf(d) * (lane == 0 ? y[0] : lane == 1 ? y[1] : y[2]);
  }
}

// encoder weight gradient for one block of 64 nodes: partial dWe = G0^T x
__global__ void __launch_bounds__(256) k_gnn_encode_bwd(int64_t n, const float* __restrict__ Gin,
                                                        const float* __restrict__ x,
                                                        float* __restrict__ partial /* [grid][H*FIN] */) {
  __shared__ float gs[64 * H];
  __shared__ float xs[64 * FIN];
  const int64_t base = (int64_t)blockIdx.x * 64;
  for (int i = threadIdx.x; i < 64 * H; i += blockDim.x) {
    const int64_t node = base + i / H;
    gs[i] = node < n ? Gin[node * H + i % H] : 0.f;
  }
  for (int i = threadIdx.x; i < 64 * FIN; i += blockDim.x) {
    const int64_t node = base + i / FIN;
    xs[i] = node < n ? x[node * FIN + i % FIN] : 0.f;
  }
  __syncthreads();
  for (int v = threadIdx.x; v < H * FIN; v += blockDim.x) {
    const int o = v / FIN, f = v % FIN;
    float a = 0.f;
    for (int i = 0; i < 64; i++) a += gs[i * H + o] * xs[i * FIN + f];
    partial[(int64_t)blockIdx.x * (H * FIN) + v] = a;
  }
}

// out[p] (+)= sum_b partial[b * P + p], b in order
__global__ void k_gnn_reduce_cols(int64_t nb, int P, const float* __restrict__ partial, float* __restrict__ out,
                                  int accumulate) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    double a = 0.0;
    for (int64_t b = 0; b < nb; b++) a += (double)partial[b * P + p];
    out[p] = accumulate ? out[p] + (float)a : (float)a;
  }
}

// dL/d(log c) = c * sum_i Go_i dinv_i r_i  (the Jacobi term's share of dL/dM), fixed-order finish
__global__ void __launch_bounds__(256) k_gnn_cgrad(int64_t n3, const float* __restrict__ Go,
                                                   const float* __restrict__ r, const float* __restrict__ dinv,
                                                   const float* __restrict__ params, float* __restrict__ partials,
                                                   unsigned* counter, float* __restrict__ grad, int accumulate) {
  float acc[1] = {0.f};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x)
    acc[0] += Go[i] * dinv[i] * r[i];
  double t[1];
  if (!last_block_sums<1>(acc, partials, counter, t) || threadIdx.x != 0) return;
  const float v = (float)(t[0] * (double)expf(params[OFF_C]));
  grad[OFF_C] = accumulate ? grad[OFF_C] + v : v;
}

// loss of one sample in the energy norm:  d = M(r) - e,  q = K d,
//   L = d.q / c,  dL/dM(r) = 2 q / c   (c = e.r = e.K.e);  the last block writes L to *loss
__global__ void __launch_bounds__(256) k_gnn_loss(int64_t n3, const float* __restrict__ d, const float* __restrict__ q,
                                                  float inv_c, float* __restrict__ Go, float* __restrict__ partials,
                                                  unsigned* counter, float* loss) {
  float acc[1] = {0.f};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
    acc[0] += d[i] * q[i];
    Go[i] = 2.f * q[i] * inv_c;
  }
  double t[1];
  if (last_block_sums<1>(acc, partials, counter, t) && threadIdx.x == 0) *loss = (float)(t[0] * inv_c);
}

// Adam on the FP32 master parameters
__global__ void k_gnn_adam(int np, float* __restrict__ prm, const float* __restrict__ grad, float* __restrict__ m,
                           float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2,
                           float clip_scale) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const float gi = grad[i] * clip_scale;
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    prm[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// BF16 copies of the layer weights in one array of 3 NL H AIN values:
//   Wb  [l][o][a] = Wl[o][a]                    (forward layers, [H][AIN])
//   Wtb [l][a][o] = Wl[o][a]                    (weight-gradient kernels, [AIN][H])
//   Wsb [l]       = [Wa^T | Wb^T], Wl = [Wa | Wb] (transposed layers run as forward layers, [H][AIN])
__global__ void k_gnn_pack(const float* __restrict__ prm, __nv_bfloat16* __restrict__ Wb) {
  const int per = H * AIN;
  __nv_bfloat16* Wtb = Wb + NL * per;
  __nv_bfloat16* Wsb = Wtb + NL * per;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NL * per; i += gridDim.x * blockDim.x) {
    const int l = i / per, k = i % per, o = k / AIN, a = k % AIN;
    const __nv_bfloat16 v = __float2bfloat16(prm[OFF_L + l * L_STRIDE + k]);
    Wb[i] = v;
    Wtb[l * per + a * H + o] = v;
    Wsb[l * per + (a < H ? a * AIN + o : (a - H) * AIN + H + o)] = v;
  }
}

// ============================== inference ==============================
// One kernel per layer of S and of S^T.  A transposed layer
//   g_in = g + g Wa + A^T (g Wb)  =  g + [g ; A^T g] [Wa ; Wb]
// has the shape of a forward layer with the transposed aggregation (A^T g)_j =
// sum_{i in N(j)} g_i / deg_i and the weights [Wa^T | Wb^T], so S^T needs no scatter pass.
// FIRST fuses the encoder (h0 = We x, A h0 = We (A x)), LAST the output
// M(r) = D^-1/2 (c x + We^T g0).  Persistent CTAs of 64 nodes (4 warps x 16 rows); the
// neighbour indices of a row are loaded by the lanes in parallel and broadcast with
// shuffles, so up to 8 neighbour rows are in flight per warp.
template <bool FIRST, bool TRANS, bool LAST>
__global__ void __launch_bounds__(LT) k_gnn_layer_inf(Graph g, const __nv_bfloat16* __restrict__ hin,
                                                      const float* __restrict__ r, const float* __restrict__ dinv,
                                                      const float* __restrict__ params,
                                                      const __nv_bfloat16* __restrict__ W,  // [H][AIN]
                                                      __nv_bfloat16* __restrict__ hout, float* __restrict__ out,
                                                      const int* done) {
  if (done && *done) return;
  __shared__ __align__(16) __nv_bfloat16 As[TILE * SROW];
  __shared__ __align__(16) __nv_bfloat16 Ws[H * SROW];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int i = tid; i < H * (AIN / 8); i += LT) {
    const int row = i / (AIN / 8), c8 = i % (AIN / 8);
    *reinterpret_cast<uint4*>(&Ws[row * SROW + 8 * c8]) = reinterpret_cast<const uint4*>(W)[row * (AIN / 8) + c8];
  }
  // encoder weights of this lane's two features (FIRST) / the three output rows (LAST)
  float we[2][FIN];
  if (FIRST) {
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
      for (int f = 0; f < FIN; f++) we[k][f] = params[OFF_WE + (2 * lane + k) * FIN + f];
  }
  const uint32_t* h32 = reinterpret_cast<const uint32_t*>(hin);
  const int64_t ntiles = (g.n + TILE - 1) / TILE;
  const int gq = lane >> 2, t4 = lane & 3;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t base = tile * TILE;
    for (int rr = 0; rr < 16; rr++) {
      const int row = 16 * w + rr;
      const int64_t node = base + row;
      uint32_t self = 0, msg = 0;
      if (node < g.n) {
        const int p0 = g.ptr[node], deg = g.ptr[node + 1] - p0;
        if (FIRST) {
          // x = D^-1/2 r at the node and the mean over its neighbours (lanes load neighbours)
          float xs[FIN], xm[FIN] = {0.f, 0.f, 0.f};
#pragma unroll
          for (int c = 0; c < FIN; c++) xs[c] = r[FIN * node + c] * sqrtf(dinv[FIN * node + c]);
          for (int e0 = 0; e0 < deg; e0 += 32) {
            if (e0 + lane < deg) {
              const int64_t j = g.idx[p0 + e0 + lane];
#pragma unroll
              for (int c = 0; c < FIN; c++) xm[c] += r[FIN * j + c] * sqrtf(dinv[FIN * j + c]);
            }
          }
          const float id = g.inv_deg[node];
#pragma unroll
          for (int c = 0; c < FIN; c++) xm[c] = warp_sumf(xm[c]) * id;
          float a0 = 0.f, a1 = 0.f, m0 = 0.f, m1 = 0.f;
#pragma unroll
          for (int f = 0; f < FIN; f++) {
            a0 += we[0][f] * xs[f];
            a1 += we[1][f] * xs[f];
            m0 += we[0][f] * xm[f];
            m1 += we[1][f] * xm[f];
          }
          self = f2bf(a0, a1);
          msg = f2bf(m0, m1);
        } else {
          self = h32[node * (H / 2) + lane];
          float m0 = 0.f, m1 = 0.f;
          for (int e0 = 0; e0 < deg; e0 += 32) {
            const int cnt = min(32, deg - e0);
            int jl = 0;
            float wl = 1.f;
            if (lane < cnt) {
              jl = g.idx[p0 + e0 + lane];
              if (TRANS) wl = g.inv_deg[jl];
            }
            for (int e = 0; e < cnt; e += 8) {
              float2 v[8];
#pragma unroll
              for (int u = 0; u < 8; u++) {
                const int j = __shfl_sync(0xffffffffu, jl, (e + u) & 31);
                v[u] = (e + u < cnt) ? bf2f(h32[(int64_t)j * (H / 2) + lane]) : make_float2(0.f, 0.f);
              }
#pragma unroll
              for (int u = 0; u < 8; u++) {
                const float wu = TRANS ? __shfl_sync(0xffffffffu, wl, (e + u) & 31) : 1.f;
                m0 += wu * v[u].x;
                m1 += wu * v[u].y;
              }
            }
          }
          const float id = TRANS ? 1.f : g.inv_deg[node];
          msg = f2bf(m0 * id, m1 * id);
        }
      }
      *reinterpret_cast<uint32_t*>(&As[row * SROW + 2 * lane]) = self;
      *reinterpret_cast<uint32_t*>(&As[row * SROW + H + 2 * lane]) = msg;
    }
    __syncthreads();
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const __nv_bfloat16* Ar0 = &As[(16 * w + gq) * SROW];
    const __nv_bfloat16* Ar1 = &As[(16 * w + gq + 8) * SROW];
#pragma unroll
    for (int kk = 0; kk < AIN / 16; kk++) {
      const int k0 = 16 * kk + 2 * t4;
      const uint32_t a0 = ld32(Ar0 + k0), a1 = ld32(Ar1 + k0), a2 = ld32(Ar0 + k0 + 8), a3 = ld32(Ar1 + k0 + 8);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const __nv_bfloat16* Wr = &Ws[(8 * j + gq) * SROW + k0];
        mma_bf16(acc[j], a0, a1, a2, a3, ld32(Wr), ld32(Wr + 8));
      }
    }
    // epilogue: rows gq and gq + 8 of this warp, cols 8j + 2 t4 + {0,1}
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int row = 16 * w + gq + 8 * half;
      const int64_t node = base + row;
      if (!LAST) {
        if (node < g.n) {
#pragma unroll
          for (int j = 0; j < 8; j++) {
            const int col = 8 * j + 2 * t4;
            const float2 hs = bf2f(ld32(&As[row * SROW + col]));
            reinterpret_cast<uint32_t*>(hout)[node * (H / 2) + col / 2] =
                f2bf(hs.x + acc[j][2 * half], hs.y + acc[j][2 * half + 1]);
          }
        }
      } else {
        // y = We^T g0 over this thread's 16 columns, then across the 4 lanes of the quad
        float y[FIN] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int col = 8 * j + 2 * t4;
          const float2 hs = bf2f(ld32(&As[row * SROW + col]));
          const float g0 = hs.x + acc[j][2 * half], g1 = hs.y + acc[j][2 * half + 1];
#pragma unroll
          for (int c = 0; c < FIN; c++)
            y[c] += g0 * params[OFF_WE + col * FIN + c] + g1 * params[OFF_WE + (col + 1) * FIN + c];
        }
#pragma unroll
        for (int c = 0; c < FIN; c++) {
          y[c] += __shfl_xor_sync(0xffffffffu, y[c], 1);
          y[c] += __shfl_xor_sync(0xffffffffu, y[c], 2);
        }
        if (t4 < FIN && node < g.n) {
          const int64_t i = FIN * node + t4;
          const float cc = expf(params[OFF_C]);
          const float d = dinv[i];
          out[i] = cc * d * r[i] + sqrtf(d) * (t4 == 0 ? y[0] : t4 == 1 ? y[1] : y[2]);
        }
      }
    }
    __syncthreads();  // As is refilled by the next tile
  }
}

// ======================= inference through the folded polynomial =======================
// y_{k+1} = A y_k (mean over neighbours), y_0 = x = D^-1/2 r; then w_j = sum_k y_k G[k][j]
// and M(r) = D^-1/2 (c x + w_0 + A^T (w_1 + A^T (w_2 + A^T w_3)))   (Horner in A^T).
// Six passes, one thread per node, over FP16 node rows of 8 bytes (Row16: x, y, z, 0, scaled by
// sigma) so that one neighbour costs one 8-byte load; sums and products in FP32.
// A^T u = sum_j u_j / deg_j: the pass that writes a Horner operand stores u_i / deg_i, so every
// gather is a plain neighbour sum.  The neighbour loop is unrolled by four (four loads in
// flight) and adds in neighbour order (deterministic).

// sum over the neighbours j of node i of v_j.  The neighbours come from the pattern table when
// there is one (a 2-byte id per node; the table's few hundred deltas stay in L1 and a warp of
// interior nodes reads one address), else from the 16-bit deltas or the 32-bit CSR; the three
// list the same neighbours in the same order.
__device__ __forceinline__ float3 node_gather16(const Graph& g, int64_t i, const Row16* __restrict__ v) {
  float3 a = make_float3(0.f, 0.f, 0.f);
  int e, p1;
  const int16_t* dl = g.d16;
  if (g.pid) {
    const int pat = g.pid[i];
    e = __ldg(&g.pptr[pat]);
    p1 = __ldg(&g.pptr[pat + 1]);
    dl = g.ptab;
  } else {
    e = g.ptr[i];
    p1 = g.ptr[i + 1];
  }
  const int ii = (int)i;
  for (; e + 4 <= p1; e += 4) {
    int jn[4];
#pragma unroll
    for (int u = 0; u < 4; u++) jn[u] = dl ? ii + (int)__ldg(&dl[e + u]) : g.idx[e + u];
    Row16 x[4];
#pragma unroll
    for (int u = 0; u < 4; u++) x[u] = v[jn[u]];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const float3 f = unpack16(x[u]);
      a.x += f.x;
      a.y += f.y;
      a.z += f.z;
    }
  }
  for (; e < p1; e++) {
    const float3 f = unpack16(v[dl ? ii + (int)__ldg(&dl[e]) : g.idx[e]]);
    a.x += f.x;
    a.y += f.y;
    a.z += f.z;
  }
  return a;
}

__device__ __forceinline__ Row16 row16(float3 a, float s) { return pack16(a.x * s, a.y * s, a.z * s); }

// the rows' scale for a pass that forms x = D^-1/2 r itself: xstat[0] = sum d r^2 (fixed-order
// sums), xstat[1] = sigma (row16_scale)
__global__ void __launch_bounds__(256) k_poly_xscale(int64_t n3, const float* __restrict__ r,
                                                     const float* __restrict__ dinv, float* __restrict__ xstat,
                                                     float* __restrict__ partials, unsigned* counter) {
  pdl_wait();
  pdl_launch_dependents();
  float acc[1] = {0.f};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x)
    acc[0] += dinv[i] * r[i] * r[i];
  double t[1];
  if (last_block_sums<1>(acc, partials, counter, t) && threadIdx.x == 0) {
    xstat[0] = (float)t[0];
    xstat[1] = row16_scale((float)t[0], n3);
  }
}

// x rows = sigma D^-1/2 r
__global__ void __launch_bounds__(256) k_scale_sqrt4(int64_t n, const float* __restrict__ r,
                                                     const float* __restrict__ dinv, const float* __restrict__ xstat,
                                                     Row16* __restrict__ x4) {
  pdl_wait();
  pdl_launch_dependents();
  const float sg = xstat[1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = 3 * i;
    x4[i] = pack16(sg * r[o] * sqrtf(dinv[o]), sg * r[o + 1] * sqrtf(dinv[o + 1]), sg * r[o + 2] * sqrtf(dinv[o + 2]));
  }
}

// yout = A yin
__global__ void __launch_bounds__(256) k_poly_fwd(Graph g, const Row16* __restrict__ yin, Row16* __restrict__ yout,
                                                  const int* done) {
  pdl_wait();
  pdl_launch_dependents();
  if (done && *done) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x)
    yout[i] = row16(node_gather16(g, i, yin), g.inv_deg[i]);
}

// y_3 = A y_2 at the node, then w_j = sum_k y_k G[k][j] for j = 0..3 (w: 4 blocks of n rows;
// w_3, the first Horner operand, stored divided by the node's degree)
__global__ void __launch_bounds__(256) k_poly_mid(Graph g, const Row16* __restrict__ x4,
                                                  const Row16* __restrict__ y1, const Row16* __restrict__ y2,
                                                  PolyCoef pc, Row16* __restrict__ w, const int* done) {
  pdl_wait();
  pdl_launch_dependents();
  if (done && *done) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x) {
    const float3 a = node_gather16(g, i, y2);
    const float id = g.inv_deg[i];
    const float3 v0 = unpack16(x4[i]), v1 = unpack16(y1[i]), v2 = unpack16(y2[i]);
    const float y[NL + 1][3] = {{v0.x, v0.y, v0.z}, {v1.x, v1.y, v1.z}, {v2.x, v2.y, v2.z},
                                {a.x * id, a.y * id, a.z * id}};
#pragma unroll
    for (int jj = 0; jj <= NL; jj++) {
      float o[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k <= NL; k++)
#pragma unroll
          for (int b = 0; b < 3; b++) acc += y[k][b] * pc.G[k][jj][3 * b + c];
        o[c] = acc;
      }
      w[jj * g.n + i] = row16(make_float3(o[0], o[1], o[2]), jj == NL ? id : 1.f);
    }
  }
}

// u_i = sum_{j in N(i)} ud_j + wadd_i, stored as u_i / deg_i (ud_j = u_j / deg_j on input)
__global__ void __launch_bounds__(256) k_poly_bwd(Graph g, const Row16* __restrict__ ud,
                                                  const Row16* __restrict__ wadd, Row16* __restrict__ out,
                                                  const int* done) {
  pdl_wait();
  pdl_launch_dependents();
  if (done && *done) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x) {
    const float3 a = node_gather16(g, i, ud);
    const float3 wa = unpack16(wadd[i]);
    out[i] = row16(make_float3(a.x + wa.x, a.y + wa.y, a.z + wa.z), g.inv_deg[i]);
  }
}

// the last Horner pass: z = D^-1/2 (c x + w_0 + A^T u) = c D^-1 r + D^-1/2 (w_0 + A^T u) / sigma, 3n.
// BETA (inside flexible CG): also the Polak-Ribiere sums of the new z,
//   z.(r - rprev), z.r and the same for z_J = D^-1 r, finished by the last block into
//   s->beta, s->rz and s->jac (Jacobi direction when z.r <= 0), like k_fcg_beta.
//   partials: 4 gridDim floats.
template <bool BETA>
__global__ void __launch_bounds__(256) k_poly_last(Graph g, const Row16* __restrict__ ud,
                                                   const Row16* __restrict__ w0, const float* __restrict__ xstat,
                                                   const float* __restrict__ r, const float* __restrict__ dinv,
                                                   float cc, float* __restrict__ out, const int* done,
                                                   const float* __restrict__ rprev, float* __restrict__ partials,
                                                   unsigned* counter, CgScalars* s, CoarseAdd ca) {
  pdl_wait();
  pdl_launch_dependents();
  if (done && *done) return;
  const float isg = 1.f / xstat[1];  // a power of two: exact
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x) {
    const float3 a = node_gather16(g, i, ud);
    const float3 wa = unpack16(w0[i]);
    const float v[3] = {(a.x + wa.x) * isg, (a.y + wa.y) * isg, (a.z + wa.z) * isg};
    // two-level: the coarse correction B_i y_a of the node's aggregate
    float cz[3] = {0.f, 0.f, 0.f};
    if (ca.aid) {
      const float3 t = coarse_prolong_term(ca.y + (int64_t)ca.nm * ca.aid[i], ca.d[i], ca.nm);
      cz[0] = t.x;
      cz[1] = t.y;
      cz[2] = t.z;
    }
    const int64_t o = 3 * i;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float d = dinv[o + c], ri = r[o + c];
      const float z = cc * d * ri + sqrtf(d) * v[c] + cz[c];
      out[o + c] = z;
      if (BETA) {
        const float dr = ri - rprev[o + c], zj = d * ri;
        acc[0] += z * dr;
        acc[1] += z * ri;
        acc[2] += zj * dr;
        acc[3] += zj * ri;
      }
    }
  }
  if (!BETA) return;
  double t[4];
  if (!last_block_sums<4>(acc, partials, counter, t) || threadIdx.x != 0) return;
  if (t[1] > 0.0 && isfinite(t[1]) && isfinite(t[0])) {
    s->beta = t[0] / s->rz;
    s->rz = t[1];
    s->jac = 0;
  } else {
    s->beta = t[2] / s->rz;
    s->rz = t[3];
    s->jac = 1;
  }
}

}  // namespace gnn
}  // namespace sfem
