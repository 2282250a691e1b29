// Device kernels of the learned graph-network preconditioner (included by sfem_gnn.cu).
//
// Network (per free node i, width H = 64, 3 message-passing layers):
//   x_i   = [z_i / s (3), log d_i - mean log d (3), touches a fixed node (1), 1]   z = D^-1 r, s = rms(z)
//   h0_i  = relu(We x_i + be)
//   h_i  <- h_i + relu(Wl [h_i ; mean_{j in N(i)} h_j] + bl)          l = 1..3
//   M(r)_i = z_i + s (Wd h3_i + bd)
// Activations are stored in BF16, GEMMs run on the tensor cores (mma.sync m16n8k16,
// BF16 inputs, FP32 accumulation), everything else in FP32.  Backward kernels write
// per-CTA weight-gradient partials that are summed in a fixed order (deterministic).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sfem_gnn.h"

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

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---- statistics: mean log d (per Jacobi update) and rms(z) (per application) ----
// sum over free DOFs of f(i); partials[blockIdx] then the last block finalises into *out
template <int WHICH>  // 0: log(1/dinv), 1: (r dinv)^2
__global__ void __launch_bounds__(256) k_gnn_stat(int64_t n3, const float* __restrict__ r,
                                                  const float* __restrict__ dinv, float* __restrict__ partials,
                                                  unsigned* counter, Scalars* sc, const int* done) {
  if (done && *done) return;
  float acc = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
    if (WHICH == 0) {
      acc += -logf(dinv[i]);
    } else {
      const float z = r[i] * dinv[i];
      acc += z * z;
    }
  }
  __shared__ float sm[8];
  __shared__ bool last;
  acc = warp_sumf(acc);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.f;
    for (int w = 0; w < 8; w++) b += sm[w];
    partials[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  if (threadIdx.x == 0) {
    __threadfence();
    double t = 0.0;  // fixed order
    for (unsigned b = 0; b < gridDim.x; b++) t += (double)__ldcg(&partials[b]);
    if (WHICH == 0) {
      sc->mean_ld = (float)(t / (double)n3);
    } else {
      const float s = sqrtf((float)(t / (double)n3)) + 1e-30f;
      sc->s = s;
      sc->inv_s = 1.f / s;
    }
    *counter = 0u;
  }
}

// ---- encoder: one warp per node, lane l computes outputs 2l, 2l+1 ----
__global__ void __launch_bounds__(256) k_gnn_encode(int64_t n, const float* __restrict__ r,
                                                    const float* __restrict__ dinv,
                                                    const uint8_t* __restrict__ fixed_nb,
                                                    const float* __restrict__ params, const Scalars* sc,
                                                    __nv_bfloat16* __restrict__ h0, __nv_bfloat16* __restrict__ u0,
                                                    float* __restrict__ xout, const int* done) {
  if (done && *done) return;
  const int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (node >= n) return;
  float x[FIN];
  const float inv_s = sc->inv_s, mld = sc->mean_ld;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float di = dinv[3 * node + c];
    x[c] = r[3 * node + c] * di * inv_s;
    x[3 + c] = -logf(di) - mld;
  }
  x[6] = fixed_nb[node] ? 1.f : 0.f;
  x[7] = 1.f;
  if (xout && lane < FIN) xout[node * FIN + lane] = x[lane];
  float v[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int o = 2 * lane + k;
    float a = params[OFF_BE + o];
#pragma unroll
    for (int f = 0; f < FIN; f++) a += params[OFF_WE + o * FIN + f] * x[f];
    v[k] = a;
  }
  const uint32_t pre = f2bf(v[0], v[1]);
  reinterpret_cast<uint32_t*>(h0)[node * (H / 2) + lane] = f2bf(fmaxf(v[0], 0.f), fmaxf(v[1], 0.f));
  if (u0) reinterpret_cast<uint32_t*>(u0)[node * (H / 2) + lane] = pre;
}

// ---- message-passing layer (forward) ----
// CTA: 64 nodes, 4 warps x 16 nodes.  Shared A tile [64 x (h ; mean h)] and Wl [64 x 128].
__global__ void __launch_bounds__(LT) k_gnn_layer_fwd(Graph g, const __nv_bfloat16* __restrict__ hin,
                                                      const __nv_bfloat16* __restrict__ W,  // [H][AIN]
                                                      const float* __restrict__ bias,
                                                      __nv_bfloat16* __restrict__ hout, __nv_bfloat16* __restrict__ uout,
                                                      const int* done) {
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
  // epilogue: h_out = h_in + relu(acc + b); rows gq and gq + 8 of this warp, cols 8j + 2 t4 + {0,1}
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int row = 16 * w + gq + 8 * half;
    const int64_t node = base + row;
    if (node >= g.n) continue;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int col = 8 * j + 2 * t4;
      const float p0 = acc[j][2 * half] + bias[col], p1 = acc[j][2 * half + 1] + bias[col + 1];
      const float2 hs = bf2f(ld32(&As[row * SROW + col]));
      reinterpret_cast<uint32_t*>(hout)[node * (H / 2) + col / 2] = f2bf(hs.x + fmaxf(p0, 0.f), hs.y + fmaxf(p1, 0.f));
      if (uout) reinterpret_cast<uint32_t*>(uout)[node * (H / 2) + col / 2] = f2bf(p0, p1);
    }
  }
}

// ---- decoder: M(r) = z + s (Wd h3 + bd); one thread per node ----
__global__ void __launch_bounds__(256) k_gnn_decode(int64_t n, const __nv_bfloat16* __restrict__ h3,
                                                    const float* __restrict__ params, const Scalars* sc,
                                                    const float* __restrict__ r, const float* __restrict__ dinv,
                                                    float* __restrict__ out, const int* done) {
  if (done && *done) return;
  __shared__ float Wd[3 * H + 3];
  for (int i = threadIdx.x; i < 3 * H + 3; i += blockDim.x) Wd[i] = params[OFF_WD + i];
  __syncthreads();
  const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= n) return;
  float y0 = Wd[3 * H], y1 = Wd[3 * H + 1], y2 = Wd[3 * H + 2];
  const uint4* hr = reinterpret_cast<const uint4*>(h3 + node * H);
#pragma unroll
  for (int q = 0; q < H / 8; q++) {
    const uint4 v = hr[q];
    const uint32_t vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const float2 f = bf2f(vv[t]);
      const int k = 8 * q + 2 * t;
      y0 += Wd[k] * f.x + Wd[k + 1] * f.y;
      y1 += Wd[H + k] * f.x + Wd[H + k + 1] * f.y;
      y2 += Wd[2 * H + k] * f.x + Wd[2 * H + k + 1] * f.y;
    }
  }
  const float s = sc->s;
  out[3 * node] = r[3 * node] * dinv[3 * node] + s * y0;
  out[3 * node + 1] = r[3 * node + 1] * dinv[3 * node + 1] + s * y1;
  out[3 * node + 2] = r[3 * node + 2] * dinv[3 * node + 2] + s * y2;
}

// ============================== backward ==============================

// decoder backward for one block of 256 nodes: Go = dL/dM(r) (3 per node)
//   gy = s Go,  g_h3 = Wd^T gy,  partial dWd = sum gy (x) h3, partial dbd = sum gy
__global__ void __launch_bounds__(256) k_gnn_decode_bwd(int64_t n, const __nv_bfloat16* __restrict__ h3,
                                                        const float* __restrict__ params, const Scalars* sc,
                                                        const float* __restrict__ Go, float* __restrict__ gh3,
                                                        float* __restrict__ partial /* [grid][3H + 3] */) {
  __shared__ float gy[256 * 3];
  __shared__ __nv_bfloat16 hs[256 * H];
  const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const float s = sc->s;
  float g0 = 0.f, g1 = 0.f, g2 = 0.f;
  if (node < n) {
    g0 = s * Go[3 * node];
    g1 = s * Go[3 * node + 1];
    g2 = s * Go[3 * node + 2];
  }
  gy[3 * threadIdx.x] = g0;
  gy[3 * threadIdx.x + 1] = g1;
  gy[3 * threadIdx.x + 2] = g2;
  for (int k = 0; k < H; k++) {
    const float wk = params[OFF_WD + k] * g0 + params[OFF_WD + H + k] * g1 + params[OFF_WD + 2 * H + k] * g2;
    if (node < n) gh3[node * H + k] = wk;
    hs[threadIdx.x * H + k] = node < n ? h3[node * H + k] : __float2bfloat16(0.f);
  }
  __syncthreads();
  for (int v = threadIdx.x; v < 3 * H + 3; v += blockDim.x) {
    float a = 0.f;
    if (v < 3 * H) {
      const int c = v / H, k = v % H;
      for (int i = 0; i < 256; i++) a += gy[3 * i + c] * __bfloat162float(hs[i * H + k]);
    } else {
      const int c = v - 3 * H;
      for (int i = 0; i < 256; i++) a += gy[3 * i + c];
    }
    partial[(int64_t)blockIdx.x * (3 * H + 3) + v] = a;
  }
}

// layer backward.  h_out = h_in + relu(u), u = Wl a + bl, a = [h_in ; mean h_in].
//   gu = G_out * (u > 0);  g_a = gu Wl  ->  G_self = G_out + g_a[:, :H],  G_msg = g_a[:, H:] / deg
//   partial dWl = gu^T a,  partial dbl = sum gu
// Wt is Wl transposed ([AIN][H], bf16).  Dynamic shared memory.
__global__ void __launch_bounds__(LT) k_gnn_layer_bwd(Graph g, const __nv_bfloat16* __restrict__ hin,
                                                      const __nv_bfloat16* __restrict__ u,
                                                      const float* __restrict__ Gout,
                                                      const __nv_bfloat16* __restrict__ Wt,
                                                      float* __restrict__ Gself, float* __restrict__ Gmsg,
                                                      float* __restrict__ partial /* [grid][LPART] */) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __nv_bfloat16* gu = reinterpret_cast<__nv_bfloat16*>(smraw);  // [TILE][SROW64]  node-major
  __nv_bfloat16* guT = gu + TILE * SROW64;                       // [H][SROW64]     out-major
  __nv_bfloat16* aT = guT + H * SROW64;                          // [AIN][SROW64]   in-major
  __nv_bfloat16* Ws = aT + AIN * SROW64;                         // [AIN][SROW64]   = Wt
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * TILE;
  for (int i = tid; i < AIN * (H / 8); i += LT) {
    const int row = i / (H / 8), c8 = i % (H / 8);
    *reinterpret_cast<uint4*>(&Ws[row * SROW64 + 8 * c8]) = reinterpret_cast<const uint4*>(Wt)[row * (H / 8) + c8];
  }
  const uint32_t* h32 = reinterpret_cast<const uint32_t*>(hin);
  const uint32_t* u32 = reinterpret_cast<const uint32_t*>(u);
  for (int rr = 0; rr < 16; rr++) {
    const int row = 16 * w + rr;
    const int64_t node = base + row;
    float g0 = 0.f, g1 = 0.f;
    uint32_t self = 0, msg = 0;
    if (node < g.n) {
      const float2 gv = *reinterpret_cast<const float2*>(&Gout[node * H + 2 * lane]);
      const float2 uv = bf2f(u32[node * (H / 2) + lane]);
      g0 = uv.x > 0.f ? gv.x : 0.f;
      g1 = uv.y > 0.f ? gv.y : 0.f;
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
    const uint32_t gb = f2bf(g0, g1);
    *reinterpret_cast<uint32_t*>(&gu[row * SROW64 + 2 * lane]) = gb;
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
          const float2 go = *reinterpret_cast<const float2*>(&Gout[node * H + col]);
          *reinterpret_cast<float2*>(&Gself[node * H + col]) = make_float2(go.x + v0, go.y + v1);
        } else {
          *reinterpret_cast<float2*>(&Gmsg[node * H + col - H]) = make_float2(v0 * id, v1 * id);
        }
      }
    }
  }
  // ---- dWl partial [64 out x 128 in] = guT [64 x 64 nodes] . a [64 nodes x 128]; B[k][n] = aT[n][k] ----
  {
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
    // bias partial: sum over the tile's nodes of gu (row of guT), fixed order
    if (tid < H) {
      float sb = 0.f;
      for (int k = 0; k < TILE; k++) sb += __bfloat162float(guT[tid * SROW64 + k]);
      P[H * AIN + tid] = sb;
    }
  }
}
constexpr size_t kLayerBwdSmem = sizeof(__nv_bfloat16) * (TILE * SROW64 + H * SROW64 + 2 * AIN * SROW64);

// G_in[j] = G_self[j] + sum_{i in N(j)} G_msg[i]   (mean aggregation transposed; symmetric graph)
__global__ void __launch_bounds__(256) k_gnn_msg_scatter(Graph g, const float* __restrict__ Gself,
                                                         const float* __restrict__ Gmsg, float* __restrict__ Gin) {
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

// encoder backward for one block of 64 nodes: gu0 = G_in0 * (u0 > 0); partial dWe = gu0^T x, dbe = sum gu0
__global__ void __launch_bounds__(256) k_gnn_encode_bwd(int64_t n, const float* __restrict__ Gin,
                                                        const __nv_bfloat16* __restrict__ u0,
                                                        const float* __restrict__ x,
                                                        float* __restrict__ partial /* [grid][H*FIN + H] */) {
  __shared__ float gs[64 * H];
  __shared__ float xs[64 * FIN];
  const int64_t base = (int64_t)blockIdx.x * 64;
  for (int i = threadIdx.x; i < 64 * H; i += blockDim.x) {
    const int64_t node = base + i / H;
    float v = 0.f;
    if (node < n && __bfloat162float(u0[node * H + i % H]) > 0.f) v = Gin[node * H + i % H];
    gs[i] = v;
  }
  for (int i = threadIdx.x; i < 64 * FIN; i += blockDim.x) {
    const int64_t node = base + i / FIN;
    xs[i] = node < n ? x[node * FIN + i % FIN] : 0.f;
  }
  __syncthreads();
  for (int v = threadIdx.x; v < H * FIN + H; v += blockDim.x) {
    float a = 0.f;
    if (v < H * FIN) {
      const int o = v / FIN, f = v % FIN;
      for (int i = 0; i < 64; i++) a += gs[i * H + o] * xs[i * FIN + f];
    } else {
      const int o = v - H * FIN;
      for (int i = 0; i < 64; i++) a += gs[i * H + o];
    }
    partial[(int64_t)blockIdx.x * (H * FIN + H) + v] = a;
  }
}

// out[off + p] (+)= sum_b partial[b * P + p], b in order
__global__ void k_gnn_reduce_cols(int64_t nb, int P, const float* __restrict__ partial, float* __restrict__ out,
                                  int accumulate) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    double a = 0.0;
    for (int64_t b = 0; b < nb; b++) a += (double)partial[b * P + p];
    out[p] = accumulate ? out[p] + (float)a : (float)a;
  }
}

// loss of one sample in the energy norm:  d = M(r) - e,  q = K d,
//   L = d.q / c,  dL/dM(r) = 2 q / c   (c = e.r = e.K.e);  the last block writes L to *loss
__global__ void __launch_bounds__(256) k_gnn_loss(int64_t n3, const float* __restrict__ d, const float* __restrict__ q,
                                                  float inv_c, float* __restrict__ Go, float* __restrict__ partials,
                                                  unsigned* counter, float* loss) {
  float acc = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
    acc += d[i] * q[i];
    Go[i] = 2.f * q[i] * inv_c;
  }
  __shared__ float sm[8];
  __shared__ bool last;
  acc = warp_sumf(acc);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.f;
    for (int w = 0; w < 8; w++) b += sm[w];
    partials[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  if (threadIdx.x == 0) {
    __threadfence();
    double t = 0.0;
    for (unsigned b = 0; b < gridDim.x; b++) t += (double)__ldcg(&partials[b]);
    *loss = (float)(t * inv_c);
    *counter = 0u;
  }
}

// Adam on the FP32 master parameters, then the BF16 layer weights (row-major and transposed)
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

__global__ void k_gnn_pack(const float* __restrict__ prm, __nv_bfloat16* __restrict__ Wb,
                           __nv_bfloat16* __restrict__ Wtb) {
  const int per = H * AIN;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NL * per; i += gridDim.x * blockDim.x) {
    const int l = i / per, k = i % per, o = k / AIN, a = k % AIN;
    const __nv_bfloat16 v = __float2bfloat16(prm[OFF_L + l * L_STRIDE + k]);
    Wb[i] = v;
    Wtb[l * per + a * H + o] = v;
  }
}

}  // namespace gnn
}  // namespace sfem
