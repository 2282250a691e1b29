// FP32 neo-Hookean patch Hessian-vector product: q = K p over one patch of elements per CTA
// (SolidFEM: FemPhysicsMatrixFree::ComputeForceDifferential, Source/FemPhysicsMatrixFree.cpp:406-496,
// neo-Hookean branch :464-470; MatrixVectorMultiply :523-534).
//
// The reference forms, per element, dF = D(p) X, dP = mu dF + (mu - lambda log J) F^-T dF^T F^-T
// + lambda tr(F^-1 dF) F^-T and the nodal forces -V dP X^T.  With G = X F^-1, L = D(p) G and
// M = X X^T the same forces are
//     -V dP X^T = -V [ mu D(p) M + c1 (G L)^T + lambda tr(L) G^T ],   c1 = mu - lambda log J,
// (dF X^T = D(p) M, F^-T dF^T F^-T X^T = (G L)^T, tr(F^-1 dF) = tr(L), F^-T X^T = G^T), which takes
// about 240 instead of about 330 floating-point instructions per element.  F^-1 enters through the
// adjugate: G = X adj(F) / J, so the 1/J factors fold into the three scalar coefficients.
//
// Data movement: the CTA's element records (X, volume, local corners: 48 bytes each, contiguous in
// patch order) arrive in shared memory through one bulk asynchronous copy (cp.async.bulk, completion
// on an mbarrier) issued before the patch's nodes are staged, so the record stream overlaps the node
// gathers instead of stalling every element on three dependent global loads.  Nodes sit in shared
// memory as 16-byte rows (u, p), one vector load per corner.  Each element's 12 nodal values are
// written over its own record; the patch-local CSR (offsets 12 i + 3 j, element order) sums them
// per node, so every nodal sum is deterministic.  Nodes of one patch write q, shared nodes write a
// partial; p.q is finished by the last CTA in a fixed order (alpha of the Krylov iteration).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "sfem_internal.h"
#include "sfem_pdl.cuh"
#include "sfem_reduce.cuh"

namespace sfem {
namespace {

constexpr int kNT = 256;
constexpr int kRecBytes = 48;
// bounded waits: iterations of mbarrier.try_wait (each suspends for a hardware-defined interval)
constexpr int kWaitIters = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (int it = 0; it < kWaitIters; it++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ float block_sum_f(float v) {
  __shared__ float sm[kNT / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < kNT / 32 ? sm[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

// The 12 nodal values of one element: f[3 (b + 1) + c] for corner b + 1, f[c] = -(sum) for corner 0.
__device__ __forceinline__ void nh_element_forces(const float (&X)[9], float vol, float mu, float la, const float4 (&U)[4],
                                                  const float4 (&P)[4], float (&f)[12]) {
  // F = I + D(u) X, D(u) columns u_{b+1} - u_0
  float Du[9];
  Du[0] = U[1].x - U[0].x; Du[1] = U[2].x - U[0].x; Du[2] = U[3].x - U[0].x;
  Du[3] = U[1].y - U[0].y; Du[4] = U[2].y - U[0].y; Du[5] = U[3].y - U[0].y;
  Du[6] = U[1].z - U[0].z; Du[7] = U[2].z - U[0].z; Du[8] = U[3].z - U[0].z;
  float F[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      F[3 * i + j] = fmaf(Du[3 * i + 2], X[6 + j], fmaf(Du[3 * i + 1], X[3 + j], fmaf(Du[3 * i], X[j], i == j ? 1.f : 0.f)));
  // adjugate (transposed cofactors, Math/matrix3.h:234-249) and J
  float A[9];
  A[0] = F[4] * F[8] - F[5] * F[7];
  A[3] = F[5] * F[6] - F[3] * F[8];
  A[6] = F[3] * F[7] - F[4] * F[6];
  A[1] = F[2] * F[7] - F[1] * F[8];
  A[4] = F[0] * F[8] - F[2] * F[6];
  A[7] = F[1] * F[6] - F[0] * F[7];
  A[2] = F[1] * F[5] - F[2] * F[4];
  A[5] = F[2] * F[3] - F[0] * F[5];
  A[8] = F[0] * F[4] - F[1] * F[3];
  const float J = F[0] * A[0] + F[1] * A[3] + F[2] * A[6];
  const float iJ = __frcp_rn(J);
  const float c1 = mu - la * logf(J);
  // G' = X adj(F) (G = G' / J)
  float Gp[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Gp[3 * i + j] = X[3 * i] * A[j] + X[3 * i + 1] * A[3 + j] + X[3 * i + 2] * A[6 + j];
  // M = X X^T (symmetric)
  const float M00 = X[0] * X[0] + X[1] * X[1] + X[2] * X[2];
  const float M01 = X[0] * X[3] + X[1] * X[4] + X[2] * X[5];
  const float M02 = X[0] * X[6] + X[1] * X[7] + X[2] * X[8];
  const float M11 = X[3] * X[3] + X[4] * X[4] + X[5] * X[5];
  const float M12 = X[3] * X[6] + X[4] * X[7] + X[5] * X[8];
  const float M22 = X[6] * X[6] + X[7] * X[7] + X[8] * X[8];
  // D(p) columns p_{b+1} - p_0
  float Dp[9];
  Dp[0] = P[1].x - P[0].x; Dp[1] = P[2].x - P[0].x; Dp[2] = P[3].x - P[0].x;
  Dp[3] = P[1].y - P[0].y; Dp[4] = P[2].y - P[0].y; Dp[5] = P[3].y - P[0].y;
  Dp[6] = P[1].z - P[0].z; Dp[7] = P[2].z - P[0].z; Dp[8] = P[3].z - P[0].z;
  // L' = D(p) G' (L = L' / J)
  float Lp[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Lp[3 * i + j] = Dp[3 * i] * Gp[j] + Dp[3 * i + 1] * Gp[3 + j] + Dp[3 * i + 2] * Gp[6 + j];
  const float trL = Lp[0] + Lp[4] + Lp[8];
  // D(p) M
  float DM[9];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    DM[3 * i] = Dp[3 * i] * M00 + Dp[3 * i + 1] * M01 + Dp[3 * i + 2] * M02;
    DM[3 * i + 1] = Dp[3 * i] * M01 + Dp[3 * i + 1] * M11 + Dp[3 * i + 2] * M12;
    DM[3 * i + 2] = Dp[3 * i] * M02 + Dp[3 * i + 1] * M12 + Dp[3 * i + 2] * M22;
  }
  // f_{b+1, c} = -V [ mu (D(p) M)_{cb} + c1 / J^2 (G' L')_{bc} + lambda tr(L') / J^2 G'_{bc} ]
  const float iJ2 = iJ * iJ;
  const float a1 = -vol * mu, a2 = -vol * c1 * iJ2, a3 = -vol * la * iJ2 * trL;
#pragma unroll
  for (int b = 0; b < 3; b++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float gl = Gp[3 * b] * Lp[c] + Gp[3 * b + 1] * Lp[3 + c] + Gp[3 * b + 2] * Lp[6 + c];
      f[3 * (b + 1) + c] = fmaf(a1, DM[3 * c + b], fmaf(a2, gl, a3 * Gp[3 * b + c]));
    }
#pragma unroll
  for (int c = 0; c < 3; c++) f[c] = -(f[3 + c] + f[6 + c] + f[9 + c]);
}

template <bool DIR>
__global__ void __launch_bounds__(kNT, 5) k_patch_hvp_nh32(PatchView<float> pv, const float* __restrict__ u,
                                                           const float* __restrict__ p, float* __restrict__ q,
                                                           float* __restrict__ partial, Reduce red, CgScalars* s,
                                                           const float* __restrict__ r, const float* __restrict__ dinv,
                                                           float* __restrict__ p_new, const float* __restrict__ z) {
  pdl_wait();
  pdl_launch_dependents();
  if (s != nullptr && s->done) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float4* srec = reinterpret_cast<float4*>(smem_raw);                           // 3 per element
  float4* snode = reinterpret_cast<float4*>(smem_raw + kRecBytes * kPatchElems);  // (u, p) per node
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + kRecBytes * kPatchElems + 32 * pv.max_nodes);
  const int c = blockIdx.x;
  const int64_t eb = pv.elem_off[c];
  const int ne = (int)(pv.elem_off[c + 1] - eb);
  const int64_t nb = pv.node_off[c];
  const int nn = (int)(pv.node_off[c + 1] - nb);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
    const uint32_t bytes = (uint32_t)(kRecBytes * ne);
    mbar_expect_tx(bar, bytes);
    bulk_g2s(srec, pv.rec + 12 * eb, bytes, bar);
  }
  float beta = 0.f;
  bool use_z = false;  // flexible CG: p = z + beta p_old with z the preconditioner output
  if (DIR) {
    beta = (float)s->beta;
    use_z = z != nullptr && s->jac == 0;
  }
  for (int j = threadIdx.x; j < nn; j += kNT) {
    int g = pv.pnode[nb + j];
    if (g < 0) g = ~g;
    const int64_t o = 3 * (int64_t)g;
    const float4 uu = make_float4(u[o], u[o + 1], u[o + 2], 0.f);
    float4 pp;
    if (DIR) {
      // zero at fixed nodes: r, dinv, z and p stay zero there
      pp.x = (use_z ? z[o] : dinv[o] * r[o]) + beta * p[o];
      pp.y = (use_z ? z[o + 1] : dinv[o + 1] * r[o + 1]) + beta * p[o + 1];
      pp.z = (use_z ? z[o + 2] : dinv[o + 2] * r[o + 2]) + beta * p[o + 2];
      // every patch that touches a node computes the same value from the same inputs
      if (g >= pv.nbc) {
        p_new[o] = pp.x;
        p_new[o + 1] = pp.y;
        p_new[o + 2] = pp.z;
      }
    } else {
      pp.x = p[o];
      pp.y = p[o + 1];
      pp.z = p[o + 2];
    }
    pp.w = 0.f;
    snode[2 * j] = uu;
    snode[2 * j + 1] = pp;
  }
  __syncthreads();
  const bool rec_ok = mbar_wait_bounded(bar, 0);
  for (int k = threadIdx.x; k < ne; k += kNT) {
    if (!rec_ok) break;
    const float4 ra = srec[3 * k], rb = srec[3 * k + 1], rc = srec[3 * k + 2];
    const float X[9] = {ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, rb.w, rc.x};
    const uint32_t w0 = __float_as_uint(rc.z), w1 = __float_as_uint(rc.w);
    const int l0 = (int)(w0 & 0xffffu), l1 = (int)(w0 >> 16), l2 = (int)(w1 & 0xffffu), l3 = (int)(w1 >> 16);
    float mu = pv.mu, la = pv.lambda;
    if (pv.scale) {
      const float sc = pv.scale[eb + k];
      mu *= sc;
      la *= pv.scale_la ? pv.scale_la[eb + k] : sc;
    }
    const float4 U[4] = {snode[2 * l0], snode[2 * l1], snode[2 * l2], snode[2 * l3]};
    const float4 P[4] = {snode[2 * l0 + 1], snode[2 * l1 + 1], snode[2 * l2 + 1], snode[2 * l3 + 1]};
    float f[12];
    nh_element_forces(X, rc.y, mu, la, U, P, f);
    // results over the element's own record (only this thread reads or writes row k)
    srec[3 * k] = make_float4(f[0], f[1], f[2], f[3]);
    srec[3 * k + 1] = make_float4(f[4], f[5], f[6], f[7]);
    srec[3 * k + 2] = make_float4(f[8], f[9], f[10], f[11]);
  }
  const bool bad = __syncthreads_or(rec_ok ? 0 : 1) != 0;
  // p.q is linear in the partial sums, so shared nodes contribute p . partial here
  const float* sres = reinterpret_cast<const float*>(srec);
  float acc = 0.f;
  const uint16_t* lp = pv.lptr + nb + c;
  const uint16_t* le = pv.lent12 + 4 * eb;
  for (int j = threadIdx.x; j < nn; j += kNT) {
    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
    const int t1 = lp[j + 1];
    for (int t = lp[j]; t < t1; t++) {
      const float* src = sres + le[t];
      f0 += src[0];
      f1 += src[1];
      f2 += src[2];
    }
    const float4 pp = snode[2 * j + 1];
    if (pv.pm) {  // implicit dynamics: q = K p + (m / h^2) p (shared nodes: a share per patch)
      const float m = pv.pm[nb + j];
      f0 -= m * pp.x;
      f1 -= m * pp.y;
      f2 -= m * pp.z;
    }
    if (bad) f0 = f1 = f2 = __int_as_float(0x7fc00000);  // records never arrived: NaN ends the solve
    const int g = pv.pnode[nb + j];
    int64_t o = -1;
    float* dst = q;
    if (g >= 0) {
      if (g >= pv.nbc) o = 3 * (int64_t)g;
    } else {
      const int d = pv.pdest[nb + j];
      if (d >= 0) {
        o = 3 * (int64_t)d;
        dst = partial;
      }
    }
    if (o >= 0) {
      dst[o] = -f0;
      dst[o + 1] = -f1;
      dst[o + 2] = -f2;
      acc -= pp.x * f0 + pp.y * f1 + pp.z * f2;
    }
  }
  if (bad && threadIdx.x == 0) mbar_wait_bounded(bar, 0);  // let a late copy land before the CTA exits
  const float v = block_sum_f(acc);
  if (s == nullptr) return;
  __shared__ bool is_last;
  float* Pp = reinterpret_cast<float*>(red.partials);
  if (threadIdx.x == 0) {
    Pp[c] = v;
    __threadfence();
    is_last = atomicAdd(red.counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  float sum[1] = {0.f};
  strided_sums<float, float, 1>(Pp, gridDim.x, gridDim.x, sum);
  const float tot = block_sum_f(sum[0]);
  if (threadIdx.x == 0) {
    *red.counter = 0u;
    const double pq = (double)tot;
    s->pq = pq;
    if (!isfinite(pq)) {
      s->done = 1;
      s->status = -3;
      s->alpha = 0.0;
    } else if (!(pq > 0.0)) {
      s->done = 1;
      s->status = 2;
      s->alpha = 0.0;
    } else {
      s->alpha = s->rz / pq;
    }
  }
}

}  // namespace

size_t patch_hvp_nh32_smem(int max_nodes) { return (size_t)kRecBytes * kPatchElems + 32 * (size_t)max_nodes + 16; }

void launch_patch_hvp_nh32(const PatchView<float>& pv, const float* u, const float* p, float* q, float* partial,
                           Reduce red, CgScalars* s, cudaStream_t st, const float* r, const float* dinv, float* p_new,
                           const float* z) {
  static bool attr_set = false;
  if (!attr_set) {
    const int mx = (int)patch_hvp_nh32_smem(kPatchNodes);
    cudaFuncSetAttribute(k_patch_hvp_nh32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_patch_hvp_nh32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    attr_set = true;
  }
  const size_t smem = patch_hvp_nh32_smem(pv.max_nodes);
  const unsigned grid = (unsigned)pv.n_patches;
  count_launch();
  if (p_new != nullptr)
    launch_pdl(k_patch_hvp_nh32<true>, grid, kNT, smem, st, pv, u, p, q, partial, red, s, r, dinv, p_new, z);
  else
    k_patch_hvp_nh32<false><<<grid, kNT, smem, st>>>(pv, u, p, q, partial, red, s, nullptr, nullptr, nullptr, nullptr);
}

}  // namespace sfem
