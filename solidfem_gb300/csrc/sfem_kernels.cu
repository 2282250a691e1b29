// Element and Krylov kernels of the matrix-free nonlinear elasticity solve.
//
// Per-tetrahedron work (SolidFEM: FemPhysicsMatrixFree::ComputeDeformationGradient
// Source/FemPhysicsMatrixFree.cpp:354-368, ElasticEnergy::ComputeElementStress
// Source/ElasticEnergy.cpp:114-257, ElasticEnergy::ComputeForces :259-282,
// FemPhysicsMatrixFree::ComputeForceDifferential Source/FemPhysicsMatrixFree.cpp:406-496,
// ElasticEnergy::ComputeElementEnergy Source/ElasticEnergy.cpp:40-112) runs one
// element per thread over structure-of-arrays element data.  The deformation
// gradient is formed from nodal displacements, F = I + D(u) Dm^-1, which equals
// the reference's D(x) Dm^-1 but keeps F - I accurate in FP32.
//
// Element results (12 nodal values) go to an element-major scratch array and
// are summed per node through a node->element CSR in element order, so every
// nodal sum is deterministic (no floating-point atomics).
//
// Krylov scalars live on the device (CgScalars); every reduction is a
// warp-shuffle block sum followed by a fixed-order sum of the block partials in
// the last block to finish, so results are run-to-run identical.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <type_traits>
#include <stdint.h>

#include "sfem_internal.h"
#include "sfem_pdl.cuh"
#include "sfem_reduce.cuh"
#include "sfem_row16.cuh"
#include "sfem_coarse.cuh"
#include "sfem_df32.cuh"

namespace sfem {

// Number of kernels this library has launched (all wrappers below count theirs).
static unsigned long long g_launches = 0;
unsigned long long launch_count() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
void count_launch() { __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED); }

// ---------------------------------------------------------------------------
// 3x3 algebra (row-major a[3*i+j])
// ---------------------------------------------------------------------------
template <typename T>
struct M3 {
  T a[9];
};

template <typename T>
__device__ __forceinline__ M3<T> mul(const M3<T>& A, const M3<T>& B) {
  M3<T> C;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) C.a[3 * i + j] = A.a[3 * i] * B.a[j] + A.a[3 * i + 1] * B.a[3 + j] + A.a[3 * i + 2] * B.a[6 + j];
  return C;
}
// A^T B
template <typename T>
__device__ __forceinline__ M3<T> mulTN(const M3<T>& A, const M3<T>& B) {
  M3<T> C;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) C.a[3 * i + j] = A.a[i] * B.a[j] + A.a[3 + i] * B.a[3 + j] + A.a[6 + i] * B.a[6 + j];
  return C;
}
// A B^T
template <typename T>
__device__ __forceinline__ M3<T> mulNT(const M3<T>& A, const M3<T>& B) {
  M3<T> C;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) C.a[3 * i + j] = A.a[3 * i] * B.a[3 * j] + A.a[3 * i + 1] * B.a[3 * j + 1] + A.a[3 * i + 2] * B.a[3 * j + 2];
  return C;
}
template <typename T>
__device__ __forceinline__ T trace(const M3<T>& A) { return A.a[0] + A.a[4] + A.a[8]; }
template <typename T>
__device__ __forceinline__ T det(const M3<T>& A) {
  return A.a[0] * (A.a[4] * A.a[8] - A.a[5] * A.a[7]) + A.a[1] * (A.a[5] * A.a[6] - A.a[3] * A.a[8]) +
         A.a[2] * (A.a[3] * A.a[7] - A.a[4] * A.a[6]);
}
// cofactor inverse (Math/matrix3.h:234-249)
template <typename T>
__device__ __forceinline__ M3<T> inverse(const M3<T>& m, T* det_out = nullptr) {
  M3<T> r;
  r.a[0] = m.a[4] * m.a[8] - m.a[5] * m.a[7];
  r.a[3] = m.a[5] * m.a[6] - m.a[3] * m.a[8];
  r.a[6] = m.a[3] * m.a[7] - m.a[4] * m.a[6];
  r.a[1] = m.a[2] * m.a[7] - m.a[1] * m.a[8];
  r.a[4] = m.a[0] * m.a[8] - m.a[2] * m.a[6];
  r.a[7] = m.a[1] * m.a[6] - m.a[0] * m.a[7];
  r.a[2] = m.a[1] * m.a[5] - m.a[2] * m.a[4];
  r.a[5] = m.a[2] * m.a[3] - m.a[0] * m.a[5];
  r.a[8] = m.a[0] * m.a[4] - m.a[1] * m.a[3];
  T d = m.a[0] * r.a[0] + m.a[1] * r.a[3] + m.a[2] * r.a[6];
  T s = T(1) / d;
#pragma unroll
  for (int k = 0; k < 9; k++) r.a[k] *= s;
  if (det_out) *det_out = d;
  return r;
}

template <typename T>
__device__ __forceinline__ T dev_log(T x);
template <>
__device__ __forceinline__ double dev_log<double>(double x) { return log(x); }
template <>
__device__ __forceinline__ float dev_log<float>(float x) { return logf(x); }
template <typename T>
__device__ __forceinline__ T dev_rsqrt(T x);
template <>
__device__ __forceinline__ double dev_rsqrt<double>(double x) { return 1.0 / sqrt(x); }
template <>
__device__ __forceinline__ float dev_rsqrt<float>(float x) { return 1.0f / sqrtf(x); }

// Gram-Schmidt "polar" decomposition of SolidFEM (Source/PolarDecomposition.cpp:37-47, 269-280):
// R = [r0 r1 r2] from the first two columns of F, U = sym(R^T F).
template <typename T>
__device__ __forceinline__ void polar_qr(const M3<T>& F, M3<T>& R, M3<T>& U) {
  T c0[3] = {F.a[0], F.a[3], F.a[6]};
  T c1[3] = {F.a[1], F.a[4], F.a[7]};
  T s = dev_rsqrt<T>(c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2]);
  T r0[3] = {c0[0] * s, c0[1] * s, c0[2] * s};
  T d = c1[0] * r0[0] + c1[1] * r0[1] + c1[2] * r0[2];
  T r1[3] = {c1[0] - d * r0[0], c1[1] - d * r0[1], c1[2] - d * r0[2]};
  s = dev_rsqrt<T>(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
  r1[0] *= s; r1[1] *= s; r1[2] *= s;
  T r2[3] = {r0[1] * r1[2] - r1[1] * r0[2], -r0[0] * r1[2] + r0[2] * r1[0], r0[0] * r1[1] - r1[0] * r0[1]};
  s = dev_rsqrt<T>(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
  r2[0] *= s; r2[1] *= s; r2[2] *= s;
#pragma unroll
  for (int i = 0; i < 3; i++) { R.a[3 * i] = r0[i]; R.a[3 * i + 1] = r1[i]; R.a[3 * i + 2] = r2[i]; }
  M3<T> V = mulTN(R, F);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) U.a[3 * i + j] = T(0.5) * (V.a[3 * i + j] + V.a[3 * j + i]);
}

// ---------------------------------------------------------------------------
// Constitutive models (material ids of MaterialModelType)
// ---------------------------------------------------------------------------
constexpr int kLinear = 0, kStvk = 1, kCorot = 2, kNeoHookean = 3;
// corotational force with the exact derivative of that force as its tangent
constexpr int kCorotExact = 4;
// the other MaterialModelType values m = 4..12 (FemDataStructures.h:93-107) have the internal id
// m + 1 (FP64 handles): neo-Hookean (Ogden), distortional linear, Mooney, NH2, NH3, Bonet-Wood,
// distortional Ogden, NH6, NH7 (ElasticEnergy.cpp:188-254, 412-479)
constexpr int kNhOgden = 5, kDistLinear = 6, kMooney = 7, kNh2 = 8, kNh3 = 9, kBonetWood = 10, kDistOgden = 11,
              kNh6 = 12, kNh7 = 13;
template <int MAT>
__host__ __device__ constexpr bool is_variant() { return MAT >= kNhOgden; }

// the float literals of the reference's formulas, as they convert to its real type
template <typename T>
__device__ __forceinline__ T c_two_thirds() { return T(2.0f / 3.0f); }
template <typename T>
__device__ __forceinline__ T c_third() { return T(1.0f / 3.0f); }
template <typename T>
__device__ __forceinline__ T dev_pow(T x, T y);
template <>
__device__ __forceinline__ double dev_pow<double>(double x, double y) { return pow(x, y); }
template <>
__device__ __forceinline__ float dev_pow<float>(float x, float y) { return powf(x, y); }

// PK1 stress of the other materials, ElasticEnergy.cpp:188-254 (the reference's formulas)
template <typename T, int MAT>
__device__ __forceinline__ M3<T> variant_stress(const M3<T>& F, T mu, T la) {
  M3<T> P;
  if constexpr (MAT == kDistLinear) {  // 2 mu eps - (2 mu / 3) tr(eps) I, Cauchy strain eps
    T tr = trace(F) - T(3);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        T eps = T(0.5) * (F.a[3 * i + j] + F.a[3 * j + i]) - (i == j ? T(1) : T(0));
        P.a[3 * i + j] = (T(2) * mu) * eps - (i == j ? (T(2) * mu / T(3)) * tr : T(0));
      }
    return P;
  }
  if constexpr (MAT == kMooney || MAT == kNh2 || MAT == kNh3) {
    T c = mu;
    if (MAT == kNh2) c = T(0.5) * (mu * (T(3) * la + T(2) * mu) / (la + mu));  // 0.5 E
    if (MAT == kNh3) c = mu * dev_pow<T>(det(F), -c_two_thirds<T>());
#pragma unroll
    for (int k = 0; k < 9; k++) P.a[k] = c * F.a[k];
    return P;
  }
  const T J = det(F);
  const M3<T> Fi = inverse(F);
  M3<T> Fit;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Fit.a[3 * i + j] = Fi.a[3 * j + i];
  if constexpr (MAT == kBonetWood) {  // mu J^-2/3 (F - (I1 / 3) F^-T)
    T I1 = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) I1 += F.a[k] * F.a[k];
    const T c = mu * dev_pow<T>(J, -c_two_thirds<T>());
#pragma unroll
    for (int k = 0; k < 9; k++) P.a[k] = c * (F.a[k] - (I1 / T(3)) * Fit.a[k]);
    return P;
  }
  if constexpr (MAT == kNh6) {  // mu (F - J F^-T)
#pragma unroll
    for (int k = 0; k < 9; k++) P.a[k] = mu * (F.a[k] - J * Fit.a[k]);
    return P;
  }
  // mu (F - F^-T) + b F^-T: Ogden-Neo-Hookean b = lambda (J - 1) J, distortional Ogden b = 0,
  // NH7 b = lambda1 log J with lambda1 = -2/3 mu
  T b = T(0);
  if constexpr (MAT == kNhOgden) b = la * (J - T(1)) * J;
  if constexpr (MAT == kNh7) b = (-c_two_thirds<T>() * mu) * dev_log<T>(J);
#pragma unroll
  for (int k = 0; k < 9; k++) P.a[k] = mu * (F.a[k] - Fit.a[k]) + b * Fit.a[k];
  return P;
}

// PK1 stress P(F), ElasticEnergy.cpp:132-187
template <typename T, int MAT>
__device__ __forceinline__ M3<T> stress(const M3<T>& F, T mu, T la) {
  M3<T> P;
  if (MAT == kLinear) {
    T tr = trace(F) - T(3);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        T eps = T(0.5) * (F.a[3 * i + j] + F.a[3 * j + i]) - (i == j ? T(1) : T(0));
        P.a[3 * i + j] = T(2) * mu * eps + (i == j ? la * tr : T(0));
      }
  } else if (MAT == kCorot || MAT == kCorotExact) {
    M3<T> R, U;
    polar_qr(F, R, U);
    T tr = trace(U) - T(3);
    M3<T> S;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) S.a[3 * i + j] = T(2) * mu * (U.a[3 * i + j] - (i == j ? T(1) : T(0))) + (i == j ? la * tr : T(0));
    P = mul(R, S);
  } else if (MAT == kStvk) {
    M3<T> C = mulTN(F, F);
    T trE = T(0.5) * (trace(C) - T(3));
    M3<T> S;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) S.a[3 * i + j] = mu * (C.a[3 * i + j] - (i == j ? T(1) : T(0))) + (i == j ? la * trE : T(0));
    P = mul(F, S);
  } else if constexpr (is_variant<MAT>()) {
    P = variant_stress<T, MAT>(F, mu, la);
  } else {
    T J;
    M3<T> Fi = inverse(F, &J);
    T lj = dev_log<T>(J);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) P.a[3 * i + j] = mu * (F.a[3 * i + j] - Fi.a[3 * j + i]) + la * lj * Fi.a[3 * j + i];
  }
  return P;
}

// strain energy density, ElasticEnergy.cpp:52-109
template <typename T, int MAT>
__device__ __forceinline__ T energy_density(const M3<T>& F, T mu, T la) {
  if constexpr (is_variant<MAT>()) {
    // ElasticEnergy.cpp:87-108: only these variants have an energy; the others report 0
    if constexpr (MAT == kNhOgden || MAT == kMooney || MAT == kDistOgden) {
      const M3<T> C = mulTN(F, F);
      const T I1 = trace(C);
      T e = T(0.5) * mu * (I1 - T(3));
      if constexpr (MAT != kMooney) {
        const T J = det(F);
        e -= mu * dev_log<T>(J);
        if constexpr (MAT == kNhOgden) e += T(0.5) * la * (J - T(1)) * (J - T(1));
      }
      return e;
    }
    return T(0);
  }
  if (MAT == kNeoHookean) {
    T J = det(F);
    T I1 = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) I1 += F.a[k] * F.a[k];
    T lj = dev_log<T>(J);
    return T(0.5) * mu * (I1 - T(3)) - mu * lj + T(0.5) * la * lj * lj;
  }
  M3<T> G = F;
  if (MAT == kCorot || MAT == kCorotExact) {
    M3<T> R;
    polar_qr(F, R, G);
  }
  M3<T> eps;
  if (MAT == kStvk) {
    M3<T> C = mulTN(G, G);
#pragma unroll
    for (int k = 0; k < 9; k++) eps.a[k] = T(0.5) * (C.a[k] - ((k % 4) == 0 ? T(1) : T(0)));
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) eps.a[3 * i + j] = T(0.5) * (G.a[3 * i + j] + G.a[3 * j + i]) - (i == j ? T(1) : T(0));
  }
  T tr = trace(eps), dd = 0;
#pragma unroll
  for (int k = 0; k < 9; k++) dd += eps.a[k] * eps.a[k];
  return mu * dd + T(0.5) * la * tr * tr;
}

// Tangent dP(F; dF), FemPhysicsMatrixFree.cpp:436-470: init() once per element,
// apply() per direction.

// Tangents of the other materials: the reference's ElasticEnergy::ComputeLocalForceDifferential
// (ElasticEnergy.cpp:412-479), which its assembled path uses (its matrix-free product covers only
// the four main materials).  Written as dP = a dF + b dF^T + c tr(dF) I + d F^-T dF^T F^-T
// + e tr(F^-1 dF) F^-T (+ the Bonet-Wood terms).
template <typename T, int MAT>
struct Tangent {
  static_assert(is_variant<MAT>(), "variant materials only");
  M3<T> F, Fit;
  T mu, la, J, I1, cj;
  __device__ void init(const M3<T>& Fm, T m, T l) {
    F = Fm;
    mu = m;
    la = l;
    J = det(F);
    const M3<T> Fi = inverse(F);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) Fit.a[3 * i + j] = Fi.a[3 * j + i];
    I1 = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) I1 += F.a[k] * F.a[k];
    cj = (MAT == kNh3 || MAT == kBonetWood) ? mu * dev_pow<T>(J, -c_two_thirds<T>()) : T(0);
  }
  __device__ M3<T> apply(const M3<T>& dF) const {
    M3<T> P;
    if constexpr (MAT == kDistLinear) {
      const T tr = trace(dF);
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
          P.a[3 * i + j] = mu * (dF.a[3 * i + j] + dF.a[3 * j + i]) - (i == j ? c_two_thirds<T>() * mu * tr : T(0));
      return P;
    }
    if constexpr (MAT == kMooney || MAT == kNh2 || MAT == kNh3) {
      T c = mu;
      if (MAT == kNh2) c = T(0.5) * (mu * (T(3) * la + T(2) * mu) / (la + mu));
      if (MAT == kNh3) c = cj;
#pragma unroll
      for (int k = 0; k < 9; k++) P.a[k] = c * dF.a[k];
      return P;
    }
    const M3<T> B = mul(mulNT(Fit, dF), Fit);  // F^-T dF^T F^-T
    T trFi = 0;                                // tr(F^-1 dF)
#pragma unroll
    for (int k = 0; k < 9; k++) trFi += Fit.a[k] * dF.a[k];
    if constexpr (MAT == kBonetWood) {
      T trdC = 0;  // tr(dF^T F + F^T dF)
#pragma unroll
      for (int k = 0; k < 9; k++) trdC += T(2) * dF.a[k] * F.a[k];
#pragma unroll
      for (int k = 0; k < 9; k++) {
        const T Q = F.a[k] - c_third<T>() * I1 * Fit.a[k];
        const T dQ = dF.a[k] - c_third<T>() * (trdC * Fit.a[k] - I1 * B.a[k]);
        P.a[k] = cj * (dQ - c_two_thirds<T>() * trFi * Q);
      }
      return P;
    }
    T cb = 0, ce = 0;
    if constexpr (MAT == kNhOgden) {
      cb = mu - la * (J - T(1));
      ce = la * J;
    } else if constexpr (MAT == kDistOgden) {
      cb = mu;
    } else if constexpr (MAT == kNh6) {
      cb = mu * J;
      ce = -mu * J;
    } else if constexpr (MAT == kNh7) {
      const T l1 = -c_two_thirds<T>() * mu;
      cb = mu - l1 * dev_log<T>(J);
      ce = l1;
    }
#pragma unroll
    for (int k = 0; k < 9; k++) P.a[k] = mu * dF.a[k] + cb * B.a[k] + ce * trFi * Fit.a[k];
    return P;
  }
};

template <typename T>
struct Tangent<T, kLinear> {
  T mu, la;
  __device__ void init(const M3<T>&, T m, T l) { mu = m; la = l; }
  __device__ M3<T> apply(const M3<T>& dF) const {
    M3<T> P;
    T tr = trace(dF);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) P.a[3 * i + j] = mu * (dF.a[3 * i + j] + dF.a[3 * j + i]) + (i == j ? la * tr : T(0));
    return P;
  }
};

template <typename T>
struct Tangent<T, kNeoHookean> {
  M3<T> Fit;  // F^-T
  T mu, la, c1;  // c1 = mu - lambda log J
  __device__ void init(const M3<T>& F, T m, T l) {
    mu = m; la = l;
    T J;
    M3<T> Fi = inverse(F, &J);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) Fit.a[3 * i + j] = Fi.a[3 * j + i];
    c1 = mu - la * dev_log<T>(J);
  }
  // dP = mu dF + c1 F^-T dF^T F^-T + lambda tr(F^-1 dF) F^-T
  __device__ M3<T> apply(const M3<T>& dF) const {
    M3<T> A = mulNT(Fit, dF);  // F^-T dF^T
    M3<T> B = mul(A, Fit);
    T tr = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) tr += Fit.a[k] * dF.a[k];
    T c2 = la * tr;
    M3<T> P;
#pragma unroll
    for (int k = 0; k < 9; k++) P.a[k] = mu * dF.a[k] + c1 * B.a[k] + c2 * Fit.a[k];
    return P;
  }
};

template <typename T>
struct Tangent<T, kCorot> {
  M3<T> R, Ainv;
  T mu, la, k;
  __device__ void init(const M3<T>& F, T m, T l) {
    mu = m; la = l;
    M3<T> S;
    polar_qr(F, R, S);
    T trS = trace(S);
    M3<T> A = S;
    A.a[0] -= trS; A.a[4] -= trS; A.a[8] -= trS;
    Ainv = inverse(A);
    k = la * (trS - T(3)) - T(2) * mu;
  }
  __device__ M3<T> apply(const M3<T>& dF) const {
    M3<T> dS = mulTN(R, dF);
    T w0 = dS.a[5] - dS.a[7], w1 = dS.a[2] - dS.a[6], w2 = dS.a[1] - dS.a[3];
    T r0 = Ainv.a[0] * w0 + Ainv.a[1] * w1 + Ainv.a[2] * w2;
    T r1 = Ainv.a[3] * w0 + Ainv.a[4] * w1 + Ainv.a[5] * w2;
    T r2 = Ainv.a[6] * w0 + Ainv.a[7] * w1 + Ainv.a[8] * w2;
    // skew(r) = [[0,-r2,r1],[r2,0,-r0],[-r1,r0,0]]
    M3<T> Sk;
    Sk.a[0] = 0; Sk.a[1] = -r2; Sk.a[2] = r1;
    Sk.a[3] = r2; Sk.a[4] = 0; Sk.a[5] = -r0;
    Sk.a[6] = -r1; Sk.a[7] = r0; Sk.a[8] = 0;
    M3<T> dR = mul(R, Sk);
    T c = la * trace(dS);
    M3<T> P;
#pragma unroll
    for (int q = 0; q < 9; q++) P.a[q] = T(2) * mu * dF.a[q] + c * R.a[q] + k * dR.a[q];
    return P;
  }
};

// Exact derivative of the corotational stress P = R S(U) with the Gram-Schmidt R and
// U = sym(R^T F): differentiates r0 = c0/|c0|, r1 = v1/|v1| (v1 = c1 - (c1.r0) r0),
// r2 = r0 x r1 / |r0 x r1|, then dU = sym(dR^T F + R^T dF), dP = dR S + R dS.
// (The reference's differential, FemPhysicsMatrixFree.cpp:441-456, assumes a true polar R.)
template <typename T>
struct Tangent<T, kCorotExact> {
  M3<T> F, R, S;
  T mu, la, n0, n1, n2, a;
  __device__ void init(const M3<T>& Fin, T m, T l) {
    mu = m; la = l; F = Fin;
    T c0[3] = {F.a[0], F.a[3], F.a[6]}, c1[3] = {F.a[1], F.a[4], F.a[7]};
    n0 = sqrt(c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2]);
    T r0[3] = {c0[0] / n0, c0[1] / n0, c0[2] / n0};
    a = c1[0] * r0[0] + c1[1] * r0[1] + c1[2] * r0[2];
    T v1[3] = {c1[0] - a * r0[0], c1[1] - a * r0[1], c1[2] - a * r0[2]};
    n1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
    T r1[3] = {v1[0] / n1, v1[1] / n1, v1[2] / n1};
    T v2[3] = {r0[1] * r1[2] - r1[1] * r0[2], -r0[0] * r1[2] + r0[2] * r1[0], r0[0] * r1[1] - r1[0] * r0[1]};
    n2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
#pragma unroll
    for (int i = 0; i < 3; i++) { R.a[3 * i] = r0[i]; R.a[3 * i + 1] = r1[i]; R.a[3 * i + 2] = v2[i] / n2; }
    M3<T> V = mulTN(R, F);
    T tr = T(0);
#pragma unroll
    for (int i = 0; i < 3; i++) tr += V.a[4 * i] - T(1);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        S.a[3 * i + j] = mu * (V.a[3 * i + j] + V.a[3 * j + i]) - (i == j ? T(2) * mu - la * tr : T(0));
  }
  __device__ M3<T> apply(const M3<T>& dF) const {
    T r0[3] = {R.a[0], R.a[3], R.a[6]}, r1[3] = {R.a[1], R.a[4], R.a[7]}, r2[3] = {R.a[2], R.a[5], R.a[8]};
    T c1[3] = {F.a[1], F.a[4], F.a[7]};
    T dc0[3] = {dF.a[0], dF.a[3], dF.a[6]}, dc1[3] = {dF.a[1], dF.a[4], dF.a[7]};
    T t = r0[0] * dc0[0] + r0[1] * dc0[1] + r0[2] * dc0[2];
    T dr0[3], dv1[3], dr1[3], dv2[3], dr2[3];
#pragma unroll
    for (int i = 0; i < 3; i++) dr0[i] = (dc0[i] - t * r0[i]) / n0;
    T da = dc1[0] * r0[0] + dc1[1] * r0[1] + dc1[2] * r0[2] + c1[0] * dr0[0] + c1[1] * dr0[1] + c1[2] * dr0[2];
#pragma unroll
    for (int i = 0; i < 3; i++) dv1[i] = dc1[i] - da * r0[i] - a * dr0[i];
    t = r1[0] * dv1[0] + r1[1] * dv1[1] + r1[2] * dv1[2];
#pragma unroll
    for (int i = 0; i < 3; i++) dr1[i] = (dv1[i] - t * r1[i]) / n1;
    dv2[0] = dr0[1] * r1[2] - dr0[2] * r1[1] + r0[1] * dr1[2] - r0[2] * dr1[1];
    dv2[1] = dr0[2] * r1[0] - dr0[0] * r1[2] + r0[2] * dr1[0] - r0[0] * dr1[2];
    dv2[2] = dr0[0] * r1[1] - dr0[1] * r1[0] + r0[0] * dr1[1] - r0[1] * dr1[0];
    t = r2[0] * dv2[0] + r2[1] * dv2[1] + r2[2] * dv2[2];
#pragma unroll
    for (int i = 0; i < 3; i++) dr2[i] = (dv2[i] - t * r2[i]) / n2;
    M3<T> dR;
#pragma unroll
    for (int i = 0; i < 3; i++) { dR.a[3 * i] = dr0[i]; dR.a[3 * i + 1] = dr1[i]; dR.a[3 * i + 2] = dr2[i]; }
    M3<T> dV = mulTN(dR, F), W = mulTN(R, dF);
    T trdU = T(0);
#pragma unroll
    for (int q = 0; q < 9; q++) dV.a[q] += W.a[q];
#pragma unroll
    for (int i = 0; i < 3; i++) trdU += dV.a[4 * i];
    M3<T> dS;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) dS.a[3 * i + j] = mu * (dV.a[3 * i + j] + dV.a[3 * j + i]) + (i == j ? la * trdU : T(0));
    M3<T> P1 = mul(dR, S), P2 = mul(R, dS);
#pragma unroll
    for (int q = 0; q < 9; q++) P1.a[q] += P2.a[q];
    return P1;
  }
};

template <typename T>
struct Tangent<T, kStvk> {
  M3<T> F, S;  // S = 2 mu E + lambda tr(E) I
  T mu, la;
  __device__ void init(const M3<T>& Fin, T m, T l) {
    mu = m; la = l; F = Fin;
    M3<T> C = mulTN(F, F);
    T trE = T(0.5) * (trace(C) - T(3));
#pragma unroll
    for (int q = 0; q < 9; q++) S.a[q] = mu * (C.a[q] - ((q % 4) == 0 ? T(1) : T(0))) + ((q % 4) == 0 ? la * trE : T(0));
  }
  // dP = dF S + F (2 mu dE + lambda tr(dE) I), dE = sym(F^T dF)
  __device__ M3<T> apply(const M3<T>& dF) const {
    M3<T> W = mulTN(F, dF);
    T trdE = trace(W);
    M3<T> dS;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) dS.a[3 * i + j] = mu * (W.a[3 * i + j] + W.a[3 * j + i]) + (i == j ? la * trdE : T(0));
    M3<T> P1 = mul(dF, S), P2 = mul(F, dS);
#pragma unroll
    for (int q = 0; q < 9; q++) P1.a[q] += P2.a[q];
    return P1;
  }
};

// ---------------------------------------------------------------------------
// Reductions
// ---------------------------------------------------------------------------
template <typename A, int K>
__device__ __forceinline__ void block_sum(A (&v)[K]) {
  __shared__ A sm[K][32];
#pragma unroll
  for (int k = 0; k < K; k++)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; k++) sm[k][w] = v[k];
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      v[k] = lane < nw ? sm[k][lane] : A(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    }
  }
  __syncthreads();
}

// Block partials, then a fixed-order sum in the last block.  Returns true in
// the last block; tot[] is valid in its thread 0.
template <typename A, int K>
__device__ __forceinline__ bool reduce_last(A (&v)[K], Reduce red, A (&tot)[K]) {
  __shared__ bool is_last;
  A* P = reinterpret_cast<A*>(red.partials);
  block_sum<A, K>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) P[k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    unsigned t = atomicAdd(red.counter, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  A s[K];
#pragma unroll
  for (int k = 0; k < K; k++) s[k] = A(0);
  strided_sums<A, A, K>(P, gridDim.x, gridDim.x, s);
  block_sum<A, K>(s);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) tot[k] = s[k];
    *red.counter = 0u;
  }
  return true;
}

__host__ __device__ inline int grid_for(int64_t n, int cap = kMaxBlocks) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

// ---------------------------------------------------------------------------
// Element pass
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void load3(const T* __restrict__ a, int g, T* o) {
  o[0] = a[3 * (int64_t)g];
  o[1] = a[3 * (int64_t)g + 1];
  o[2] = a[3 * (int64_t)g + 2];
}

// D = [v1 - v0, v2 - v0, v3 - v0] (columns), returns D * X
template <typename T>
__device__ __forceinline__ M3<T> grad_of(const T* __restrict__ v, int4 t, const M3<T>& X) {
  T a0[3], a1[3], a2[3], a3[3];
  load3(v, t.x, a0);
  load3(v, t.y, a1);
  load3(v, t.z, a2);
  load3(v, t.w, a3);
  M3<T> D;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    D.a[3 * i] = a1[i] - a0[i];
    D.a[3 * i + 1] = a2[i] - a0[i];
    D.a[3 * i + 2] = a3[i] - a0[i];
  }
  return mul(D, X);
}

// 12 nodal values of H = s M X^T: f_{k+1} = column k, f_0 = -(f_1 + f_2 + f_3)
template <typename T>
__device__ __forceinline__ void nodal_forces(const M3<T>& M, const M3<T>& X, T s, T* f) {
  M3<T> H = mulNT(M, X);
#pragma unroll
  for (int c = 0; c < 3; c++) {
    T h0 = s * H.a[3 * c], h1 = s * H.a[3 * c + 1], h2 = s * H.a[3 * c + 2];
    f[3 + c] = h0;
    f[6 + c] = h1;
    f[9 + c] = h2;
    f[c] = -(h0 + h1 + h2);
  }
}

template <typename T>
__device__ __forceinline__ void store12(T* __restrict__ fe, int64_t e, const T* f);
template <>
__device__ __forceinline__ void store12<double>(double* __restrict__ fe, int64_t e, const double* f) {
  double2* o = reinterpret_cast<double2*>(fe + 12 * e);
#pragma unroll
  for (int k = 0; k < 6; k++) o[k] = make_double2(f[2 * k], f[2 * k + 1]);
}
template <>
__device__ __forceinline__ void store12<float>(float* __restrict__ fe, int64_t e, const float* f) {
  float4* o = reinterpret_cast<float4*>(fe + 12 * e);
#pragma unroll
  for (int k = 0; k < 3; k++) o[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
}

template <typename T, int MAT, int MODE>
__global__ void __launch_bounds__(kThreads) k_element(ElemView<T> ev, const T* __restrict__ u,
                                                      const T* __restrict__ p, T* __restrict__ fe, Reduce red,
                                                      double* result, int* n_inv, const CgScalars* s) {
  if (MODE == MODE_HVP && s != nullptr && s->done) return;
  double eacc = 0.0;
  int ninv = 0;
  const int64_t E = ev.E;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const int4 t = ev.tets[e];
    M3<T> X;
#pragma unroll
    for (int k = 0; k < 9; k++) X.a[k] = ev.X[k * E + e];
    const T vol = ev.vol[e];
    T mu = ev.mu, la = ev.lambda;
    if (ev.scale) {
      const T sc = ev.scale[e];
      mu *= sc;
      la *= ev.scale_la ? ev.scale_la[e] : sc;
    }
    M3<T> F = grad_of(u, t, X);
    F.a[0] += T(1);
    F.a[4] += T(1);
    F.a[8] += T(1);
    T f[12];
    if (MODE == MODE_FORCE || MODE == MODE_FORCE_ENERGY) {
      if (det(F) <= T(0)) ninv++;
      M3<T> P = stress<T, MAT>(F, mu, la);
      nodal_forces(P, X, -vol, f);
      store12(fe, e, f);
      if (MODE == MODE_FORCE_ENERGY) eacc += (double)(vol * energy_density<T, MAT>(F, mu, la));
    } else if (MODE == MODE_ENERGY) {
      if (det(F) <= T(0)) ninv++;
      eacc += (double)(vol * energy_density<T, MAT>(F, mu, la));
    } else if (MODE == MODE_HVP) {
      Tangent<T, MAT> tg;
      tg.init(F, mu, la);
      M3<T> dF = grad_of(p, t, X);
      M3<T> dP = tg.apply(dF);
      nodal_forces(dP, X, -vol, f);
      store12(fe, e, f);
    } else if (MODE == MODE_STRESS) {
      M3<T> P = stress<T, MAT>(F, mu, la);
#pragma unroll
      for (int q = 0; q < 9; q++) f[q] = P.a[q];
      f[9] = f[10] = f[11] = T(0);
      store12(fe, e, f);
    } else if (MODE == MODE_PMU || MODE == MODE_PLAMBDA) {
      // ElasticEnergy::ComputeStress splits the neo-Hookean P = mu Pmu + lambda Plambda
      // (ElasticEnergy.cpp:183-186); other materials report zero parts.
      M3<T> Pp;
#pragma unroll
      for (int q = 0; q < 9; q++) Pp.a[q] = T(0);
      if (MAT == kNeoHookean) {
        T J;
        M3<T> Fi = inverse(F, &J);
        const T lj = dev_log<T>(J);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++)
            Pp.a[3 * i + j] = MODE == MODE_PMU ? F.a[3 * i + j] - Fi.a[3 * j + i] : lj * Fi.a[3 * j + i];
      } else if (MAT == kDistOgden && MODE == MODE_PMU) {  // Pmu = F - F^-T (ElasticEnergy.cpp:239-245)
        const M3<T> Fi = inverse(F);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) Pp.a[3 * i + j] = F.a[3 * i + j] - Fi.a[3 * j + i];
      }
      nodal_forces(Pp, X, -vol, f);
      store12(fe, e, f);
    } else if (MODE == MODE_NODALVOL) {
#pragma unroll
      for (int q = 0; q < 12; q++) f[q] = (q % 3 == 0) ? T(0.25) * vol : T(0);
      store12(fe, e, f);
    } else {  // MODE_DIAG: diagonal of the local stiffness, K_aa,cc = -df_{a,c}(e_{a,c})
      Tangent<T, MAT> tg;
      tg.init(F, mu, la);
#pragma unroll 1
      for (int a = 0; a < 4; a++) {
        T g[3];
        if (a == 0) {
          g[0] = -(X.a[0] + X.a[3] + X.a[6]);
          g[1] = -(X.a[1] + X.a[4] + X.a[7]);
          g[2] = -(X.a[2] + X.a[5] + X.a[8]);
        } else {
          g[0] = X.a[3 * (a - 1)];
          g[1] = X.a[3 * (a - 1) + 1];
          g[2] = X.a[3 * (a - 1) + 2];
        }
#pragma unroll 1
        for (int c = 0; c < 3; c++) {
          M3<T> dF;
#pragma unroll
          for (int q = 0; q < 9; q++) dF.a[q] = T(0);
          dF.a[3 * c] = g[0];
          dF.a[3 * c + 1] = g[1];
          dF.a[3 * c + 2] = g[2];
          M3<T> dP = tg.apply(dF);
          // df_a,c = -vol * (dP X^T)_{c, a-1} (a>0), -sum_k(...) (a=0); K = -df.
          // (dP X^T)_{c,k} = sum_j dP_cj X_kj; df_a,c for node a uses g_a: sum_j dP_cj g_j
          T hv = dP.a[3 * c] * g[0] + dP.a[3 * c + 1] * g[1] + dP.a[3 * c + 2] * g[2];
          f[3 * a + c] = vol * hv;
        }
      }
      store12(fe, e, f);
    }
  }
  if (MODE == MODE_ENERGY || MODE == MODE_FORCE_ENERGY) {
    double v[1] = {eacc}, tot[1];
    if (reduce_last<double, 1>(v, red, tot) && threadIdx.x == 0) *result = tot[0];
  }
  if ((MODE == MODE_FORCE || MODE == MODE_ENERGY || MODE == MODE_FORCE_ENERGY) && n_inv != nullptr) {
    int v[1] = {ninv};
    block_sum<int, 1>(v);
    if (threadIdx.x == 0 && v[0] != 0) atomicAdd(n_inv, v[0]);
  }
}

template <typename T, int MAT>
void launch_element(int mode, const ElemView<T>& ev, const T* u, const T* p, T* fe, Reduce red, double* result,
                    int* n_inverted, const CgScalars* s, cudaStream_t st) {
  count_launch();
  const int grid = grid_for(ev.E, 152 * 12);
  switch (mode) {
    case MODE_FORCE:
      k_element<T, MAT, MODE_FORCE><<<grid, kThreads, 0, st>>>(ev, u, p, fe, red, result, n_inverted, s);
      break;
    case MODE_HVP:
      k_element<T, MAT, MODE_HVP><<<grid, kThreads, 0, st>>>(ev, u, p, fe, red, result, n_inverted, s);
      break;
    case MODE_DIAG:
      k_element<T, MAT, MODE_DIAG><<<grid, kThreads, 0, st>>>(ev, u, p, fe, red, result, n_inverted, s);
      break;
    case MODE_ENERGY:
      k_element<T, MAT, MODE_ENERGY><<<grid, kThreads, 0, st>>>(ev, u, p, fe, red, result, n_inverted, s);
      break;
    case MODE_FORCE_ENERGY:
      k_element<T, MAT, MODE_FORCE_ENERGY><<<grid, kThreads, 0, st>>>(ev, u, p, fe, red, result, n_inverted, s);
      break;
    case MODE_STRESS:
      k_element<T, MAT, MODE_STRESS><<<grid, kThreads, 0, st>>>(ev, u, p, fe, red, result, n_inverted, s);
      break;
    case MODE_PMU:
      k_element<T, MAT, MODE_PMU><<<grid, kThreads, 0, st>>>(ev, u, p, fe, red, result, n_inverted, s);
      break;
    case MODE_PLAMBDA:
      k_element<T, MAT, MODE_PLAMBDA><<<grid, kThreads, 0, st>>>(ev, u, p, fe, red, result, n_inverted, s);
      break;
    default:
      k_element<T, MAT, MODE_NODALVOL><<<grid, kThreads, 0, st>>>(ev, u, p, fe, red, result, n_inverted, s);
      break;
  }
}

// ---- the neo-Hookean residual's element pass in two-term FP32 arithmetic ----
//
// Forces -V P X^T (and the energy sum of V psi) of the neo-Hookean material to FP64 accuracy on the
// FP32 pipes (df32::nh_element: ElasticEnergy.cpp:170-186 and :80-86 on H = F - I), from the FP64
// displacement: the differences u_a - u_0 are taken in FP64 (nine subtractions per element) and
// split exactly; X and V are the FP32 copies plus their low parts (DfGeom).  Each element writes its
// 12 forces as (hi, lo) pairs, which k_gather_force<float2> sums per node in element order.
template <bool ENERGY>
__global__ void __launch_bounds__(kThreads) k_element_nh_df(ElemView<double> ev, DfGeom dg,
                                                            const double* __restrict__ u, float2* __restrict__ fe,
                                                            Reduce red, double* result, int* n_inv) {
  using df32::df;
  using df32::DfSum;
  DfSum eacc;
  int ninv = 0;
  const int64_t E = ev.E;
  const df mu0 = df32::split_f64(ev.mu), la0 = df32::split_f64(ev.lambda);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const int4 t = ev.tets[e];
    double a0[3], a1[3], a2[3], a3[3];
    load3(u, t.x, a0);
    load3(u, t.y, a1);
    load3(u, t.z, a2);
    load3(u, t.w, a3);
    df D[9], X[9];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      D[3 * i] = df32::split_f64(a1[i] - a0[i]);
      D[3 * i + 1] = df32::split_f64(a2[i] - a0[i]);
      D[3 * i + 2] = df32::split_f64(a3[i] - a0[i]);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) X[k] = df{dg.Xhi[k * E + e], dg.Xlo[k * E + e]};
    const df vol = {dg.volhi[e], dg.vollo[e]};
    df mu = mu0, la = la0;
    if (ev.scale) {
      const double sc = ev.scale[e];
      mu = df32::split_f64(ev.mu * sc);
      la = df32::split_f64(ev.lambda * (ev.scale_la ? ev.scale_la[e] : sc));
    }
    df f[12], psi = {0.0f, 0.0f};
    if (df32::nh_element(D, X, vol, mu, la, ENERGY, f, &psi)) ninv++;
    float4* o = reinterpret_cast<float4*>(fe + 12 * e);
#pragma unroll
    for (int k = 0; k < 6; k++) o[k] = make_float4(f[2 * k].hi, f[2 * k].lo, f[2 * k + 1].hi, f[2 * k + 1].lo);
    if (ENERGY) eacc.add(psi);
  }
  if (ENERGY) {
    double v[1] = {df32::to_f64(eacc.value())}, tot[1];
    if (reduce_last<double, 1>(v, red, tot) && threadIdx.x == 0) *result = tot[0];
  }
  if (n_inv != nullptr) {
    int v[1] = {ninv};
    block_sum<int, 1>(v);
    if (threadIdx.x == 0 && v[0] != 0) atomicAdd(n_inv, v[0]);
  }
}

void launch_element_nh_df(bool energy, const ElemView<double>& ev, const DfGeom& dg, const double* u, float2* fe,
                          Reduce red, double* result, int* n_inverted, cudaStream_t st) {
  count_launch();
  const int grid = grid_for(ev.E, 152 * 12);
  if (energy)
    k_element_nh_df<true><<<grid, kThreads, 0, st>>>(ev, dg, u, fe, red, result, n_inverted);
  else
    k_element_nh_df<false><<<grid, kThreads, 0, st>>>(ev, dg, u, fe, red, result, n_inverted);
}

// low parts of the element geometry: lo = RN(x - hi) for the FP32 copies hi = RN(x) of X and V
__global__ void __launch_bounds__(kThreads) k_split_geom(int64_t n, const double* __restrict__ x,
                                                         const float* __restrict__ hi, float* __restrict__ lo) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    lo[i] = (float)(x[i] - (double)hi[i]);
}
void launch_split_geom(int64_t n, const double* x, const float* hi, float* lo, cudaStream_t st) {
  count_launch();
  k_split_geom<<<grid_for(n), kThreads, 0, st>>>(n, x, hi, lo);
}

// Element stiffness (12 x 12, row-major, per element) from the tangent:
//   K_(a,i),(b,c) = vol * (dP^{(b,c)} g_a)_i,  dP^{(b,c)} = tangent(e_c g_b^T),
// the columns of ElasticEnergy::ComputeLocalStiffnessMatrixFromDifferential
// (Source/ElasticEnergy.cpp:493-517) in closed form; FP64.
template <typename T, int MAT>
__global__ void __launch_bounds__(kThreads) k_element_stiffness(ElemView<T> ev, const T* __restrict__ u,
                                                                T* __restrict__ Ke) {
  const int64_t E = ev.E;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const int4 t = ev.tets[e];
    M3<T> X;
#pragma unroll
    for (int k = 0; k < 9; k++) X.a[k] = ev.X[k * E + e];
    const T vol = ev.vol[e];
    T mu = ev.mu, la = ev.lambda;
    if (ev.scale) {
      const T sc = ev.scale[e];
      mu *= sc;
      la *= ev.scale_la ? ev.scale_la[e] : sc;
    }
    M3<T> F = grad_of(u, t, X);
    F.a[0] += T(1);
    F.a[4] += T(1);
    F.a[8] += T(1);
    Tangent<T, MAT> tg;
    tg.init(F, mu, la);
    T g[4][3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      g[0][j] = -(X.a[j] + X.a[3 + j] + X.a[6 + j]);
      g[1][j] = X.a[j];
      g[2][j] = X.a[3 + j];
      g[3][j] = X.a[6 + j];
    }
    T* K = Ke + 144 * e;
#pragma unroll 1
    for (int b = 0; b < 4; b++) {
#pragma unroll 1
      for (int c = 0; c < 3; c++) {
        M3<T> dF;
#pragma unroll
        for (int q = 0; q < 9; q++) dF.a[q] = T(0);
        dF.a[3 * c] = g[b][0];
        dF.a[3 * c + 1] = g[b][1];
        dF.a[3 * c + 2] = g[b][2];
        const M3<T> dP = tg.apply(dF);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int i = 0; i < 3; i++)
            K[(3 * a + i) * 12 + 3 * b + c] =
                vol * (dP.a[3 * i] * g[a][0] + dP.a[3 * i + 1] * g[a][1] + dP.a[3 * i + 2] * g[a][2]);
      }
    }
  }
}

template <typename T, int MAT>
void launch_element_stiffness(const ElemView<T>& ev, const T* u, T* Ke, cudaStream_t st) {
  count_launch();
  k_element_stiffness<T, MAT><<<grid_for(ev.E), kThreads, 0, st>>>(ev, u, Ke);
}
#define SFEM_INST_STIFF(M)                                                                                     \
  template void launch_element_stiffness<double, M>(const ElemView<double>&, const double*, double*, cudaStream_t);
#define SFEM_INST_STIFF32(M)                                                                                   \
  template void launch_element_stiffness<float, M>(const ElemView<float>&, const float*, float*, cudaStream_t);
SFEM_INST_STIFF(0)
SFEM_INST_STIFF(1)
SFEM_INST_STIFF(2)
SFEM_INST_STIFF(3)
SFEM_INST_STIFF(4)
SFEM_INST_STIFF32(0)
SFEM_INST_STIFF32(1)
SFEM_INST_STIFF32(2)
SFEM_INST_STIFF32(3)
SFEM_INST_STIFF32(4)
SFEM_INST_STIFF(5)
SFEM_INST_STIFF(6)
SFEM_INST_STIFF(7)
SFEM_INST_STIFF(8)
SFEM_INST_STIFF(9)
SFEM_INST_STIFF(10)
SFEM_INST_STIFF(11)
SFEM_INST_STIFF(12)
SFEM_INST_STIFF(13)

// Block-CSR assembly over free nodes, one thread per row in element order (deterministic):
// vals[9 s] += K_e block (a, b) for every element entry (e, a) of the row's node and every
// free corner b (s = slot[16 e + 4 a + b]); plus (m / h^2) I on the diagonal block (dynamics).
__global__ void __launch_bounds__(kThreads) k_assemble_bsr(int64_t nbc, int64_t N, NodeCsr csr,
                                                           const double* __restrict__ Ke,
                                                           const int32_t* __restrict__ slot,
                                                           const int32_t* __restrict__ dslot,
                                                           const double* __restrict__ mass, double inv_h2,
                                                           double* __restrict__ vals) {
  for (int64_t g = nbc + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
    for (int64_t k = csr.ptr[g]; k < csr.ptr[g + 1]; k++) {
      const int64_t ent = csr.ent[k];
      const int64_t e = ent >> 2;
      const int a = (int)(ent & 3);
      const double* K = Ke + 144 * e;
#pragma unroll 1
      for (int b = 0; b < 4; b++) {
        const int32_t sl = slot[16 * e + 4 * a + b];
        if (sl < 0) continue;
        double* V = vals + 9 * (int64_t)sl;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int c = 0; c < 3; c++) V[3 * i + c] += K[(3 * a + i) * 12 + 3 * b + c];
      }
    }
    if (mass) {
      double* V = vals + 9 * (int64_t)dslot[g - nbc];
      const double m = mass[g] * inv_h2;
      V[0] += m;
      V[4] += m;
      V[8] += m;
    }
  }
}
void launch_assemble_bsr(int64_t nbc, int64_t N, NodeCsr csr, const double* Ke, const int32_t* slot,
                         const int32_t* dslot, const double* mass, double inv_h2, double* vals, cudaStream_t st) {
  count_launch();
  k_assemble_bsr<<<grid_for(N - nbc), kThreads, 0, st>>>(nbc, N, csr, Ke, slot, dslot, mass, inv_h2, vals);
}

// Element stiffness for the sliced-ELL assembly, block (a, b) row-major [i][c] in 12 slots (9 used),
// written as 16-byte stores.  Symmetric tangents (linear, StVK, neo-Hookean) store the ten blocks
// a <= b in the order (0,0) (0,1) (0,2) (0,3) (1,1) (1,2) (1,3) (2,2) (2,3) (3,3) (120 values per
// element); the corotational tangents, which are not symmetric, all sixteen in the order 4 a + b
// (192 values).  Neo-Hookean in closed form, with g_a the corner gradients and h_a = F^-T g_a:
//   K_ab[i][c] = vol (mu (g_a . g_b) d_ic + (mu - lambda log J) (h_b)_i (h_a)_c + lambda (h_a)_i (h_b)_c),
// the other materials from their tangent's columns as k_element_stiffness.
template <int MAT>
__host__ __device__ constexpr int stiffness_blocks() { return (MAT == kCorot || MAT == kCorotExact) ? 16 : 10; }

template <typename T, int MAT>
__global__ void __launch_bounds__(kThreads) k_element_stiffness_sym(ElemView<T> ev, const T* __restrict__ u,
                                                                    T* __restrict__ Ke) {
  constexpr int NB = stiffness_blocks<MAT>();
  const int64_t E = ev.E;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const int4 t = ev.tets[e];
    M3<T> X;
#pragma unroll
    for (int k = 0; k < 9; k++) X.a[k] = ev.X[k * E + e];
    const T vol = ev.vol[e];
    T mu = ev.mu, la = ev.lambda;
    if (ev.scale) {
      const T sc = ev.scale[e];
      mu *= sc;
      la *= ev.scale_la ? ev.scale_la[e] : sc;
    }
    M3<T> F = grad_of(u, t, X);
    F.a[0] += T(1);
    F.a[4] += T(1);
    F.a[8] += T(1);
    T g[4][3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      g[0][j] = -(X.a[j] + X.a[3 + j] + X.a[6 + j]);
      g[1][j] = X.a[j];
      g[2][j] = X.a[3 + j];
      g[3][j] = X.a[6 + j];
    }
    T* K = Ke + 12 * NB * e;
    if constexpr (MAT == kNeoHookean) {
      T J;
      const M3<T> Fi = inverse(F, &J);
      const T c1 = mu - la * dev_log<T>(J);
      T hh[4][3];  // h_a = F^-T g_a: (h_a)_i = sum_k Fi[k][i] g_a[k]
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int i = 0; i < 3; i++) hh[a][i] = Fi.a[i] * g[a][0] + Fi.a[3 + i] * g[a][1] + Fi.a[6 + i] * g[a][2];
      int blk = 0;
#pragma unroll
      for (int a = 0; a < 4; a++) {
#pragma unroll
        for (int b = a; b < 4; b++, blk++) {
          const T gg = mu * (g[a][0] * g[b][0] + g[a][1] * g[b][1] + g[a][2] * g[b][2]);
          T v[12];
#pragma unroll
          for (int i = 0; i < 3; i++)
#pragma unroll
            for (int c = 0; c < 3; c++)
              v[3 * i + c] = vol * ((i == c ? gg : T(0)) + c1 * hh[b][i] * hh[a][c] + la * hh[a][i] * hh[b][c]);
          v[9] = v[10] = v[11] = T(0);
          store12(K + 12 * blk, 0, v);
        }
      }
    } else {
      Tangent<T, MAT> tg;
      tg.init(F, mu, la);
      // column (b, c) of the element matrix gives rows a <= b of block (a, b)
      T cols[3][12];
#pragma unroll 1
      for (int b = 0; b < 4; b++) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
          M3<T> dF;
#pragma unroll
          for (int q = 0; q < 9; q++) dF.a[q] = T(0);
          dF.a[3 * c] = g[b][0];
          dF.a[3 * c + 1] = g[b][1];
          dF.a[3 * c + 2] = g[b][2];
          const M3<T> dP = tg.apply(dF);
#pragma unroll
          for (int a = 0; a < 4; a++)
#pragma unroll
            for (int i = 0; i < 3; i++)
              cols[c][3 * a + i] = vol * (dP.a[3 * i] * g[a][0] + dP.a[3 * i + 1] * g[a][1] + dP.a[3 * i + 2] * g[a][2]);
        }
#pragma unroll 1
        for (int a = 0; a < (NB == 16 ? 4 : b + 1); a++) {
          const int blk = NB == 16 ? 4 * a + b : a == 0 ? b : a == 1 ? 3 + b : a == 2 ? 5 + b : 9;
          T v[12];
#pragma unroll
          for (int i = 0; i < 3; i++)
#pragma unroll
            for (int c = 0; c < 3; c++) v[3 * i + c] = cols[c][3 * a + i];
          v[9] = v[10] = v[11] = T(0);
          store12(K + 12 * blk, 0, v);
        }
      }
    }
  }
}
template <typename T, int MAT>
int launch_element_stiffness_sym(const ElemView<T>& ev, const T* u, T* Ke, cudaStream_t st) {
  count_launch();
  k_element_stiffness_sym<T, MAT><<<grid_for(ev.E), kThreads, 0, st>>>(ev, u, Ke);
  return stiffness_blocks<MAT>();
}
template int launch_element_stiffness_sym<float, 0>(const ElemView<float>&, const float*, float*, cudaStream_t);
template int launch_element_stiffness_sym<float, 1>(const ElemView<float>&, const float*, float*, cudaStream_t);
template int launch_element_stiffness_sym<float, 2>(const ElemView<float>&, const float*, float*, cudaStream_t);
template int launch_element_stiffness_sym<float, 3>(const ElemView<float>&, const float*, float*, cudaStream_t);
template int launch_element_stiffness_sym<float, 4>(const ElemView<float>&, const float*, float*, cudaStream_t);
template int launch_element_stiffness_sym<double, 0>(const ElemView<double>&, const double*, double*, cudaStream_t);
template int launch_element_stiffness_sym<double, 1>(const ElemView<double>&, const double*, double*, cudaStream_t);
template int launch_element_stiffness_sym<double, 2>(const ElemView<double>&, const double*, double*, cudaStream_t);
template int launch_element_stiffness_sym<double, 3>(const ElemView<double>&, const double*, double*, cudaStream_t);
template int launch_element_stiffness_sym<double, 4>(const ElemView<double>&, const double*, double*, cudaStream_t);

// ---- assembled tangent in sliced ELL (32 rows per slice) for the Krylov loops ----
// Block-slot t of free row r (slice r / 32, lane l = r % 32, position k in the row) is
// t = base[slice] + 32 k + l; its nine values sit at vals[9 (t - l) + 32 q + l] (q = 3 i + c), so a
// warp (one slice) reads each value of a row position with one coalesced 128-byte load.

// the nine used values of a 12-slot, 16-byte aligned block
__device__ __forceinline__ void load9(const double* K, double (&kb)[9]) {
  const double2* K2 = reinterpret_cast<const double2*>(K);
  const double2 a = K2[0], b = K2[1], c = K2[2], d = K2[3], e = K2[4];
  kb[0] = a.x; kb[1] = a.y; kb[2] = b.x; kb[3] = b.y; kb[4] = c.x; kb[5] = c.y; kb[6] = d.x; kb[7] = d.y;
  kb[8] = e.x;
}
__device__ __forceinline__ void load9(const float* K, float (&kb)[9]) {
  const float4* K4 = reinterpret_cast<const float4*>(K);
  const float4 a = K4[0], b = K4[1], c = K4[2];
  kb[0] = a.x; kb[1] = a.y; kb[2] = a.z; kb[3] = a.w;
  kb[4] = b.x; kb[5] = b.y; kb[6] = b.z; kb[7] = b.w;
  kb[8] = c.x;
}

// assembly, one thread per block-slot: the slot's contributions K_e(a, b) (code = 16 e + 4 a + b;
// Ke in the ten-block symmetric layout of k_element_stiffness_sym) in the order of its row's element entries (the node->element CSR order, deterministic), summed
// in registers and stored once (consecutive slots of a slice store coalesced)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_assemble_sell(int64_t nslots, const int64_t* __restrict__ cptr,
                                                            const uint32_t* __restrict__ code, const T* __restrict__ Ke,
                                                            int nb, T* __restrict__ vals) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nslots; t += (int64_t)gridDim.x * blockDim.x) {
    T acc[9];
#pragma unroll
    for (int q = 0; q < 9; q++) acc[q] = T(0);
    for (int64_t c = cptr[t]; c < cptr[t + 1]; c++) {
      const uint32_t v = code[c];
      const int a = (int)((v >> 2) & 3), b = (int)(v & 3);
      const int lo = a < b ? a : b, hi = a < b ? b : a;
      const int blk = nb == 16 ? 4 * a + b : lo == 0 ? hi : lo == 1 ? 3 + hi : lo == 2 ? 5 + hi : 9;
      T kb[9];
      load9(Ke + 12 * nb * (int64_t)(v >> 4) + 12 * blk, kb);
      if (nb == 16 || a <= b) {
#pragma unroll
        for (int q = 0; q < 9; q++) acc[q] += kb[q];
      } else {  // block (a, b) is the transpose of the stored block (b, a)
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int cc = 0; cc < 3; cc++) acc[3 * i + cc] += kb[3 * cc + i];
      }
    }
    T* V = vals + 9 * (t & ~(int64_t)31) + (t & 31);
#pragma unroll
    for (int q = 0; q < 9; q++) V[32 * q] = acc[q];
  }
}
// FP32 neo-Hookean factors of the element tangent for the sliced-ELL assembly, kNhFactors floats per
// element (six 16-byte stores) instead of its ten 3x3 blocks: h_a = F^-T g_a (corner-major, 12), vol mu
// (g_a . g_b) for the ten pairs a <= b (in the blocks' order of k_element_stiffness_sym), vol (mu -
// lambda log J), vol lambda.  Block (a, b) of any corner pair is then
//   K_ab[i][c] = vol mu (g_a . g_b) d_ic + vol c1 (h_b)_i (h_a)_c + vol lambda (h_a)_i (h_b)_c,
// formed where the assembly sums it (k_assemble_sell_nh): a fifth of the bytes written and read.
constexpr int kNhFactors = 24;
__global__ void __launch_bounds__(kThreads) k_element_factors_nh(ElemView<float> ev, const float* __restrict__ u,
                                                                 float* __restrict__ Kf) {
  const int64_t E = ev.E;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const int4 t = ev.tets[e];
    M3<float> X;
#pragma unroll
    for (int k = 0; k < 9; k++) X.a[k] = ev.X[k * E + e];
    const float vol = ev.vol[e];
    float mu = ev.mu, la = ev.lambda;
    if (ev.scale) {
      const float sc = ev.scale[e];
      mu *= sc;
      la *= ev.scale_la ? ev.scale_la[e] : sc;
    }
    M3<float> F = grad_of(u, t, X);
    F.a[0] += 1.f;
    F.a[4] += 1.f;
    F.a[8] += 1.f;
    float g[4][3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      g[0][j] = -(X.a[j] + X.a[3 + j] + X.a[6 + j]);
      g[1][j] = X.a[j];
      g[2][j] = X.a[3 + j];
      g[3][j] = X.a[6 + j];
    }
    float J;
    const M3<float> Fi = inverse(F, &J);
    float f[kNhFactors];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int i = 0; i < 3; i++) f[3 * a + i] = Fi.a[i] * g[a][0] + Fi.a[3 + i] * g[a][1] + Fi.a[6 + i] * g[a][2];
    int blk = 0;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = a; b < 4; b++, blk++) f[12 + blk] = vol * mu * (g[a][0] * g[b][0] + g[a][1] * g[b][1] + g[a][2] * g[b][2]);
    f[22] = vol * (mu - la * dev_log<float>(J));
    f[23] = vol * la;
    float4* K4 = reinterpret_cast<float4*>(Kf + kNhFactors * e);
#pragma unroll
    for (int k = 0; k < kNhFactors / 4; k++) K4[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
  }
}

// assembly from the neo-Hookean factors: one thread per block-slot, its contributions (code = 16 e +
// 4 a + b) formed from element e's factors and summed in the order of k_assemble_sell (deterministic)
__global__ void __launch_bounds__(kThreads) k_assemble_sell_nh(int64_t nslots, const int64_t* __restrict__ cptr,
                                                               const uint32_t* __restrict__ code,
                                                               const float* __restrict__ Kf, float* __restrict__ vals) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nslots; t += (int64_t)gridDim.x * blockDim.x) {
    float acc[9];
#pragma unroll
    for (int q = 0; q < 9; q++) acc[q] = 0.f;
    for (int64_t c = cptr[t]; c < cptr[t + 1]; c++) {
      const uint32_t v = code[c];
      const int a = (int)((v >> 2) & 3), b = (int)(v & 3);
      const int lo = a < b ? a : b, hi = a < b ? b : a;
      const int blk = lo == 0 ? hi : lo == 1 ? 3 + hi : lo == 2 ? 5 + hi : 9;
      const float* f = Kf + (int64_t)kNhFactors * (v >> 4);
      const float ha[3] = {__ldg(f + 3 * a), __ldg(f + 3 * a + 1), __ldg(f + 3 * a + 2)};
      const float hb[3] = {__ldg(f + 3 * b), __ldg(f + 3 * b + 1), __ldg(f + 3 * b + 2)};
      const float gg = __ldg(f + 12 + blk), c1 = __ldg(f + 22), la = __ldg(f + 23);
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int cc = 0; cc < 3; cc++) acc[3 * i + cc] += (i == cc ? gg : 0.f) + c1 * hb[i] * ha[cc] + la * ha[i] * hb[cc];
    }
    float* V = vals + 9 * (t & ~(int64_t)31) + (t & 31);
#pragma unroll
    for (int q = 0; q < 9; q++) V[32 * q] = acc[q];
  }
}

// implicit dynamics: (m / h^2) I added to each free row's diagonal block
template <typename T>
__global__ void __launch_bounds__(kThreads) k_sell_mass(int64_t nbc, int64_t nf, const int32_t* __restrict__ dslot,
                                                        const double* __restrict__ mass, double inv_h2,
                                                        T* __restrict__ vals) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nf; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = dslot[r];
    T* V = vals + 9 * (t & ~(int64_t)31) + (t & 31);
    const T m = (T)(mass[nbc + r] * inv_h2);
    V[0] += m;
    V[32 * 4] += m;
    V[32 * 8] += m;
  }
}
void launch_assemble_sell_nh32(const ElemView<float>& ev, const float* u, float* Kf, int64_t nslots, const int64_t* cptr,
                               const uint32_t* code, int64_t nbc, int64_t nf, const int32_t* dslot, const double* mass,
                               double inv_h2, float* vals, cudaStream_t st) {
  count_launch();
  k_element_factors_nh<<<grid_for(ev.E), kThreads, 0, st>>>(ev, u, Kf);
  count_launch();
  k_assemble_sell_nh<<<grid_for(nslots), kThreads, 0, st>>>(nslots, cptr, code, Kf, vals);
  if (mass) {
    count_launch();
    k_sell_mass<float><<<grid_for(nf), kThreads, 0, st>>>(nbc, nf, dslot, mass, inv_h2, vals);
  }
}

// the Jacobi diagonal's inverse from the assembled operator: each free row's diagonal block (slot
// dslot[r]) holds the row's three diagonal entries (with the mass term of implicit dynamics)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_sell_diag_inv(int64_t nbc, int64_t nf, const int32_t* __restrict__ dslot,
                                                            const T* __restrict__ vals, T* __restrict__ dinv) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nf; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = dslot[r];
    const T* V = vals + 9 * (t & ~(int64_t)31) + (t & 31);
    const int64_t o = 3 * (nbc + r);
    dinv[o] = T(1) / V[0];
    dinv[o + 1] = T(1) / V[32 * 4];
    dinv[o + 2] = T(1) / V[32 * 8];
  }
}
template <typename T>
void launch_sell_diag_inv(int64_t nbc, int64_t nf, const int32_t* dslot, const T* vals, T* dinv, cudaStream_t st) {
  count_launch();
  k_sell_diag_inv<T><<<grid_for(nf), kThreads, 0, st>>>(nbc, nf, dslot, vals, dinv);
}
template void launch_sell_diag_inv<float>(int64_t, int64_t, const int32_t*, const float*, float*, cudaStream_t);
template void launch_sell_diag_inv<double>(int64_t, int64_t, const int32_t*, const double*, double*, cudaStream_t);

template <typename T>
void launch_assemble_sell(int64_t nslots, const int64_t* cptr, const uint32_t* code, const T* Ke, int nb,
                          int64_t nbc, int64_t nf, const int32_t* dslot, const double* mass, double inv_h2, T* vals,
                          cudaStream_t st) {
  count_launch();
  k_assemble_sell<T><<<grid_for(nslots), kThreads, 0, st>>>(nslots, cptr, code, Ke, nb, vals);
  if (mass) {
    count_launch();
    k_sell_mass<T><<<grid_for(nf), kThreads, 0, st>>>(nbc, nf, dslot, mass, inv_h2, vals);
  }
}
template void launch_assemble_sell<float>(int64_t, const int64_t*, const uint32_t*, const float*, int, int64_t,
                                          int64_t, const int32_t*, const double*, double, float*, cudaStream_t);
template void launch_assemble_sell<double>(int64_t, const int64_t*, const uint32_t*, const double*, int, int64_t,
                                           int64_t, const int32_t*, const double*, double, double*, cudaStream_t);

// q = K p over the free rows from the sliced-ELL tangent, one thread per row (a warp per slice).
// DIR (Krylov iteration): the direction is formed where it is read, as in the patch product,
// p = (z or D^-1 r) + beta p_old, and written to p_new for the row's node.  With s: p.q and
// alpha = r.z / p.q by the last block (non-finite or non-positive p.q ends the solve).
template <typename T, bool DIR, typename CI>
__global__ void __launch_bounds__(kThreads) k_sell_hvp(int64_t nbc, int64_t nf, const int64_t* __restrict__ base,
                                                       const CI* __restrict__ col, const T* __restrict__ vals,
                                                       const T* __restrict__ p, T* __restrict__ q, Reduce red,
                                                       CgScalars* s, const T* __restrict__ r,
                                                       const T* __restrict__ dinv, T* __restrict__ p_new,
                                                       const T* __restrict__ z) {
  pdl_wait();
  pdl_launch_dependents();
  if (s != nullptr && s->done) return;
  T beta = T(0);
  bool use_z = false;
  if (DIR) {
    beta = (T)s->beta;
    use_z = z != nullptr && s->jac == 0;
  }
  T acc = T(0);
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < nf; row += (int64_t)gridDim.x * blockDim.x) {
    const int64_t sl = row >> 5;
    const int lane = (int)(row & 31);
    const int64_t b0 = base[sl];
    const int w = (int)((base[sl + 1] - b0) >> 5);
    const CI* cl = col + b0 + lane;
    // a column is the free-node index (32-bit) or its difference to the row (16-bit)
    const int64_t cbase = sizeof(CI) == 2 ? row : 0;
    const T* Vb = vals + 9 * b0 + lane;
    // the direction at free node jf (3 components)
    auto xdir = [&](int64_t jf, T& x0, T& x1, T& x2) {
      const int64_t j = 3 * (nbc + jf);
      if (DIR) {
        x0 = (use_z ? z[j] : dinv[j] * r[j]) + beta * p[j];
        x1 = (use_z ? z[j + 1] : dinv[j + 1] * r[j + 1]) + beta * p[j + 1];
        x2 = (use_z ? z[j + 2] : dinv[j + 2] * r[j + 2]) + beta * p[j + 2];
      } else {
        x0 = p[j];
        x1 = p[j + 1];
        x2 = p[j + 2];
      }
    };
    T y0 = T(0), y1 = T(0), y2 = T(0);
    int k = 0;
    // two block positions per step: their column, value and direction loads are all in flight
    for (; k + 2 <= w; k += 2) {
      const int64_t ja = cbase + cl[32 * k], jb = cbase + cl[32 * k + 32];
      const T* Va = Vb + 288 * k;
      const T* Wb = Va + 288;
      T va[9], vb[9];
#pragma unroll
      for (int q = 0; q < 9; q++) {
        va[q] = Va[32 * q];
        vb[q] = Wb[32 * q];
      }
      T xa0, xa1, xa2, xb0, xb1, xb2;
      xdir(ja, xa0, xa1, xa2);
      xdir(jb, xb0, xb1, xb2);
      y0 += va[0] * xa0 + va[1] * xa1 + va[2] * xa2;
      y1 += va[3] * xa0 + va[4] * xa1 + va[5] * xa2;
      y2 += va[6] * xa0 + va[7] * xa1 + va[8] * xa2;
      y0 += vb[0] * xb0 + vb[1] * xb1 + vb[2] * xb2;
      y1 += vb[3] * xb0 + vb[4] * xb1 + vb[5] * xb2;
      y2 += vb[6] * xb0 + vb[7] * xb1 + vb[8] * xb2;
    }
    if (k < w) {
      const T* Va = Vb + 288 * k;
      T x0, x1, x2;
      xdir(cbase + cl[32 * k], x0, x1, x2);
      y0 += Va[0] * x0 + Va[32] * x1 + Va[64] * x2;
      y1 += Va[96] * x0 + Va[128] * x1 + Va[160] * x2;
      y2 += Va[192] * x0 + Va[224] * x1 + Va[256] * x2;
    }
    const int64_t o = 3 * (nbc + row);
    T p0, p1, p2;
    if (DIR) {
      p0 = (use_z ? z[o] : dinv[o] * r[o]) + beta * p[o];
      p1 = (use_z ? z[o + 1] : dinv[o + 1] * r[o + 1]) + beta * p[o + 1];
      p2 = (use_z ? z[o + 2] : dinv[o + 2] * r[o + 2]) + beta * p[o + 2];
      p_new[o] = p0;
      p_new[o + 1] = p1;
      p_new[o + 2] = p2;
    } else {
      p0 = p[o];
      p1 = p[o + 1];
      p2 = p[o + 2];
    }
    q[o] = y0;
    q[o + 1] = y1;
    q[o + 2] = y2;
    acc += p0 * y0 + p1 * y1 + p2 * y2;
  }
  if (s == nullptr) return;
  T v[1] = {acc}, tot[1];
  if (reduce_last<T, 1>(v, red, tot) && threadIdx.x == 0) {
    const double pq = (double)tot[0];
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
template <typename T>
void launch_sell_hvp(int64_t nbc, int64_t nf, const int64_t* base, const int32_t* col, const int16_t* col16,
                     const T* vals, const T* p, T* q, Reduce red, CgScalars* s, cudaStream_t st, const T* r,
                     const T* dinv, T* p_new, const T* z) {
  static const int wave = std::min(std::min(resident_ctas(k_sell_hvp<T, true, int32_t>, kThreads, 0),
                                            resident_ctas(k_sell_hvp<T, false, int32_t>, kThreads, 0)),
                                   std::min(resident_ctas(k_sell_hvp<T, true, int16_t>, kThreads, 0),
                                            resident_ctas(k_sell_hvp<T, false, int16_t>, kThreads, 0)));
  const int grid = std::max(1, std::min(wave, (int)((nf + kThreads - 1) / kThreads)));
  count_launch();
  if (col16 && p_new != nullptr)
    launch_pdl(k_sell_hvp<T, true, int16_t>, grid, kThreads, 0, st, nbc, nf, base, col16, vals, p, q, red, s, r, dinv,
               p_new, z);
  else if (col16)
    launch_pdl(k_sell_hvp<T, false, int16_t>, grid, kThreads, 0, st, nbc, nf, base, col16, vals, p, q, red, s,
               nullptr, nullptr, nullptr, nullptr);
  else if (p_new != nullptr)
    launch_pdl(k_sell_hvp<T, true, int32_t>, grid, kThreads, 0, st, nbc, nf, base, col, vals, p, q, red, s, r, dinv,
               p_new, z);
  else
    launch_pdl(k_sell_hvp<T, false, int32_t>, grid, kThreads, 0, st, nbc, nf, base, col, vals, p, q, red, s,
               nullptr, nullptr, nullptr, nullptr);
}
template void launch_sell_hvp<float>(int64_t, int64_t, const int64_t*, const int32_t*, const int16_t*, const float*,
                                     const float*, float*, Reduce, CgScalars*, cudaStream_t, const float*,
                                     const float*, float*, const float*);
template void launch_sell_hvp<double>(int64_t, int64_t, const int64_t*, const int32_t*, const int16_t*, const double*,
                                      const double*, double*, Reduce, CgScalars*, cudaStream_t, const double*,
                                      const double*, double*, const double*);

// q = K p from the symmetric tangent's diagonal and upper blocks, one thread per row (a warp per slice).
// The row's lower blocks K_rj = K_jr^T are read from their mirror slots in row j (lower entries in
// column order, then the stored blocks: the order of the full row), so each stored block streams
// from HBM once and its mirror read, by a row up to the mesh's bandwidth away processed at about the
// same time, hits L2.  DIR and the p.q / alpha finish as in k_sell_hvp.
template <typename T, bool DIR, typename CI>
__global__ void __launch_bounds__(kThreads, 4) k_ssell_hvp(int64_t nbc, int64_t nf, const int64_t* __restrict__ base,
                                                        const CI* __restrict__ col, const int64_t* __restrict__ lbase,
                                                        const CI* __restrict__ lcol, const int32_t* __restrict__ lslot,
                                                        const T* __restrict__ vals, const T* __restrict__ p,
                                                        T* __restrict__ q, Reduce red, CgScalars* s,
                                                        const T* __restrict__ r, const T* __restrict__ dinv,
                                                        T* __restrict__ p_new, const T* __restrict__ z) {
  pdl_wait();
  pdl_launch_dependents();
  if (s != nullptr && s->done) return;
  T beta = T(0);
  bool use_z = false;
  if (DIR) {
    beta = (T)s->beta;
    use_z = z != nullptr && s->jac == 0;
  }
  T acc = T(0);
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < nf; row += (int64_t)gridDim.x * blockDim.x) {
    const int64_t sl = row >> 5;
    const int lane = (int)(row & 31);
    const int64_t cbase = sizeof(CI) == 2 ? row : 0;
    auto xdir = [&](int64_t jf, T& x0, T& x1, T& x2) {
      const int64_t j = 3 * (nbc + jf);
      if (DIR) {
        x0 = (use_z ? z[j] : dinv[j] * r[j]) + beta * p[j];
        x1 = (use_z ? z[j + 1] : dinv[j + 1] * r[j + 1]) + beta * p[j + 1];
        x2 = (use_z ? z[j + 2] : dinv[j + 2] * r[j + 2]) + beta * p[j + 2];
      } else {
        x0 = p[j];
        x1 = p[j + 1];
        x2 = p[j + 2];
      }
    };
    T y0 = T(0), y1 = T(0), y2 = T(0);
    // lower blocks, transposed from the mirror rows (two entries per step: both slots, values and
    // directions in flight; padding, slot -1, follows the row's last lower block)
    {
      const int64_t lb0 = lbase[sl];
      const int wl = (int)((lbase[sl + 1] - lb0) >> 5);
      const CI* lc = lcol + lb0 + lane;
      const int32_t* ls = lslot + lb0 + lane;
      auto mirror = [&](int64_t t, T (&v)[9]) {
        const T* V = vals + 9 * (t & ~(int64_t)31) + (t & 31);
#pragma unroll
        for (int qq = 0; qq < 9; qq++) v[qq] = V[32 * qq];
      };
      // the next pair's slots and columns are loaded while this pair's values are (one dependent
      // round trip per pair instead of two)
      int k = 0;
      int ta = -1, tb = -1;
      int64_t ja = 0, jb = 0;
      if (wl >= 2) {
        ta = ls[0], tb = ls[32];
        ja = cbase + lc[0], jb = cbase + lc[32];
      }
      for (; k + 2 <= wl; k += 2) {
        if (ta < 0) break;
        int tan = -1, tbn = -1;
        int64_t jan = 0, jbn = 0;
        if (tb >= 0 && k + 4 <= wl) {
          tan = ls[32 * k + 64], tbn = ls[32 * k + 96];
          jan = cbase + lc[32 * k + 64], jbn = cbase + lc[32 * k + 96];
        }
        T va[9], vb[9], xa0, xa1, xa2, xb0 = T(0), xb1 = T(0), xb2 = T(0);
        mirror(ta, va);
        xdir(ja, xa0, xa1, xa2);
        if (tb >= 0) {
          mirror(tb, vb);
          xdir(jb, xb0, xb1, xb2);
        } else {
#pragma unroll
          for (int qq = 0; qq < 9; qq++) vb[qq] = T(0);
        }
        y0 += va[0] * xa0 + va[3] * xa1 + va[6] * xa2;
        y1 += va[1] * xa0 + va[4] * xa1 + va[7] * xa2;
        y2 += va[2] * xa0 + va[5] * xa1 + va[8] * xa2;
        y0 += vb[0] * xb0 + vb[3] * xb1 + vb[6] * xb2;
        y1 += vb[1] * xb0 + vb[4] * xb1 + vb[7] * xb2;
        y2 += vb[2] * xb0 + vb[5] * xb1 + vb[8] * xb2;
        if (tb < 0) {
          k = wl;
          break;
        }
        ta = tan, tb = tbn, ja = jan, jb = jbn;
      }
      if (k < wl) {
        const int ta = ls[32 * k];
        if (ta >= 0) {
          T va[9], x0, x1, x2;
          mirror(ta, va);
          xdir(cbase + lc[32 * k], x0, x1, x2);
          y0 += va[0] * x0 + va[3] * x1 + va[6] * x2;
          y1 += va[1] * x0 + va[4] * x1 + va[7] * x2;
          y2 += va[2] * x0 + va[5] * x1 + va[8] * x2;
        }
      }
    }
    // the diagonal and upper blocks of the row itself
    const int64_t b0 = base[sl];
    const int w = (int)((base[sl + 1] - b0) >> 5);
    const CI* cl = col + b0 + lane;
    const T* Vb = vals + 9 * b0 + lane;
    int k = 0;
    CI ca = 0, cb = 0;
    if (w >= 2) ca = cl[0], cb = cl[32];
    for (; k + 2 <= w; k += 2) {
      const int64_t ja = cbase + ca, jb = cbase + cb;
      if (k + 4 <= w) ca = cl[32 * k + 64], cb = cl[32 * k + 96];
      const T* Va = Vb + 288 * k;
      const T* Wb = Va + 288;
      T va[9], vb[9];
#pragma unroll
      for (int qq = 0; qq < 9; qq++) {
        va[qq] = Va[32 * qq];
        vb[qq] = Wb[32 * qq];
      }
      T xa0, xa1, xa2, xb0, xb1, xb2;
      xdir(ja, xa0, xa1, xa2);
      xdir(jb, xb0, xb1, xb2);
      y0 += va[0] * xa0 + va[1] * xa1 + va[2] * xa2;
      y1 += va[3] * xa0 + va[4] * xa1 + va[5] * xa2;
      y2 += va[6] * xa0 + va[7] * xa1 + va[8] * xa2;
      y0 += vb[0] * xb0 + vb[1] * xb1 + vb[2] * xb2;
      y1 += vb[3] * xb0 + vb[4] * xb1 + vb[5] * xb2;
      y2 += vb[6] * xb0 + vb[7] * xb1 + vb[8] * xb2;
    }
    if (k < w) {
      const T* Va = Vb + 288 * k;
      T x0, x1, x2;
      xdir(cbase + cl[32 * k], x0, x1, x2);
      y0 += Va[0] * x0 + Va[32] * x1 + Va[64] * x2;
      y1 += Va[96] * x0 + Va[128] * x1 + Va[160] * x2;
      y2 += Va[192] * x0 + Va[224] * x1 + Va[256] * x2;
    }
    const int64_t o = 3 * (nbc + row);
    T p0, p1, p2;
    if (DIR) {
      p0 = (use_z ? z[o] : dinv[o] * r[o]) + beta * p[o];
      p1 = (use_z ? z[o + 1] : dinv[o + 1] * r[o + 1]) + beta * p[o + 1];
      p2 = (use_z ? z[o + 2] : dinv[o + 2] * r[o + 2]) + beta * p[o + 2];
      p_new[o] = p0;
      p_new[o + 1] = p1;
      p_new[o + 2] = p2;
    } else {
      p0 = p[o];
      p1 = p[o + 1];
      p2 = p[o + 2];
    }
    q[o] = y0;
    q[o + 1] = y1;
    q[o + 2] = y2;
    acc += p0 * y0 + p1 * y1 + p2 * y2;
  }
  if (s == nullptr) return;
  T v[1] = {acc}, tot[1];
  if (reduce_last<T, 1>(v, red, tot) && threadIdx.x == 0) {
    const double pq = (double)tot[0];
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
template <typename T>
void launch_ssell_hvp(int64_t nbc, int64_t nf, const int64_t* base, const int32_t* col, const int16_t* col16,
                      const int64_t* lbase, const int32_t* lcol, const int16_t* lcol16, const int32_t* lslot,
                      const T* vals, const T* p, T* q, Reduce red, CgScalars* s, cudaStream_t st, const T* r,
                      const T* dinv, T* p_new, const T* z) {
  static const int wave = std::min(std::min(resident_ctas(k_ssell_hvp<T, true, int32_t>, kThreads, 0),
                                            resident_ctas(k_ssell_hvp<T, false, int32_t>, kThreads, 0)),
                                   std::min(resident_ctas(k_ssell_hvp<T, true, int16_t>, kThreads, 0),
                                            resident_ctas(k_ssell_hvp<T, false, int16_t>, kThreads, 0)));
  const int grid = std::max(1, std::min(wave, (int)((nf + kThreads - 1) / kThreads)));
  count_launch();
  if (col16 && p_new != nullptr)
    launch_pdl(k_ssell_hvp<T, true, int16_t>, grid, kThreads, 0, st, nbc, nf, base, col16, lbase, lcol16, lslot, vals,
               p, q, red, s, r, dinv, p_new, z);
  else if (col16)
    launch_pdl(k_ssell_hvp<T, false, int16_t>, grid, kThreads, 0, st, nbc, nf, base, col16, lbase, lcol16, lslot,
               vals, p, q, red, s, nullptr, nullptr, nullptr, nullptr);
  else if (p_new != nullptr)
    launch_pdl(k_ssell_hvp<T, true, int32_t>, grid, kThreads, 0, st, nbc, nf, base, col, lbase, lcol, lslot, vals, p,
               q, red, s, r, dinv, p_new, z);
  else
    launch_pdl(k_ssell_hvp<T, false, int32_t>, grid, kThreads, 0, st, nbc, nf, base, col, lbase, lcol, lslot, vals,
               p, q, red, s, nullptr, nullptr, nullptr, nullptr);
}
template void launch_ssell_hvp<float>(int64_t, int64_t, const int64_t*, const int32_t*, const int16_t*,
                                      const int64_t*, const int32_t*, const int16_t*, const int32_t*, const float*,
                                      const float*, float*, Reduce, CgScalars*, cudaStream_t, const float*,
                                      const float*, float*, const float*);
template void launch_ssell_hvp<double>(int64_t, int64_t, const int64_t*, const int32_t*, const int16_t*,
                                       const int64_t*, const int32_t*, const int16_t*, const int32_t*, const double*,
                                       const double*, double*, Reduce, CgScalars*, cudaStream_t, const double*,
                                       const double*, double*, const double*);

// y = A x for a block-CSR matrix with 3 x 3 blocks (one thread per block row)
__global__ void __launch_bounds__(kThreads) k_bsr_spmv(int64_t nrows, const int32_t* __restrict__ rowptr,
                                                       const int32_t* __restrict__ col,
                                                       const double* __restrict__ vals, const double* __restrict__ x,
                                                       double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nrows; i += (int64_t)gridDim.x * blockDim.x) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
      const int64_t j = 3 * (int64_t)col[k];
      const double* V = vals + 9 * (int64_t)k;
      const double x0 = x[j], x1 = x[j + 1], x2 = x[j + 2];
      a0 += V[0] * x0 + V[1] * x1 + V[2] * x2;
      a1 += V[3] * x0 + V[4] * x1 + V[5] * x2;
      a2 += V[6] * x0 + V[7] * x1 + V[8] * x2;
    }
    y[3 * i] = a0;
    y[3 * i + 1] = a1;
    y[3 * i + 2] = a2;
  }
}
void launch_bsr_spmv(int64_t nrows, const int32_t* rowptr, const int32_t* col, const double* vals, const double* x,
                     double* y, cudaStream_t st) {
  count_launch();
  k_bsr_spmv<<<grid_for(nrows), kThreads, 0, st>>>(nrows, rowptr, col, vals, x, y);
}

#define SFEM_INST_ELEM(T, M)                                                                                   \
  template void launch_element<T, M>(int, const ElemView<T>&, const T*, const T*, T*, Reduce, double*, int*, \
                                     const CgScalars*, cudaStream_t);
SFEM_INST_ELEM(double, 0)
SFEM_INST_ELEM(double, 1)
SFEM_INST_ELEM(double, 2)
SFEM_INST_ELEM(double, 3)
SFEM_INST_ELEM(double, 5)
SFEM_INST_ELEM(double, 6)
SFEM_INST_ELEM(double, 7)
SFEM_INST_ELEM(double, 8)
SFEM_INST_ELEM(double, 9)
SFEM_INST_ELEM(double, 10)
SFEM_INST_ELEM(double, 11)
SFEM_INST_ELEM(double, 12)
SFEM_INST_ELEM(double, 13)
SFEM_INST_ELEM(float, 0)
SFEM_INST_ELEM(float, 1)
SFEM_INST_ELEM(float, 2)
SFEM_INST_ELEM(float, 3)
SFEM_INST_ELEM(double, 4)
SFEM_INST_ELEM(float, 4)

// ---------------------------------------------------------------------------
// Node gathers
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void gather_node(NodeCsr csr, const T* __restrict__ fe, int64_t g, T* acc) {
  acc[0] = acc[1] = acc[2] = T(0);
  const int64_t b = csr.ptr[g], en = csr.ptr[g + 1];
  for (int64_t k = b; k < en; k++) {
    const int64_t x = csr.ent[k];
    const T* src = fe + 12 * (x >> 2) + 3 * (x & 3);
    acc[0] += src[0];
    acc[1] += src[1];
    acc[2] += src[2];
  }
}

__global__ void __launch_bounds__(kThreads) k_pressure_tris(PressureView pv, const double* __restrict__ x0,
                                                            const double* __restrict__ u, double ff) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < pv.n_tris; t += (int64_t)gridDim.x * blockDim.x) {
    double p[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int64_t o = 3 * (int64_t)pv.tri[3 * t + k];
#pragma unroll
      for (int c = 0; c < 3; c++) p[k][c] = x0[o + c] + u[o + c];
    }
    const double a[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
    const double b[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
    const double n[3] = {a[1] * b[2] - b[1] * a[2], -a[0] * b[2] + a[2] * b[0], a[0] * b[1] - b[0] * a[1]};
    const double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double s = ff * (0.5 * len / 3.0) * pv.pressure / len;
#pragma unroll
    for (int c = 0; c < 3; c++) pv.ptf[3 * t + c] = s * n[c];
  }
}
void launch_pressure_tris(PressureView pv, const double* x0, const double* u, double ff, cudaStream_t st) {
  count_launch();
  k_pressure_tris<<<grid_for(pv.n_tris), kThreads, 0, st>>>(pv, x0, u, ff);
}

// the nodal sums of two-term (hi, lo) element forces, in element order, converted to FP64 once
__device__ __forceinline__ void gather_node(NodeCsr csr, const float2* __restrict__ fe, int64_t g, double* acc) {
  df32::df a[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
  const int64_t b = csr.ptr[g], en = csr.ptr[g + 1];
  for (int64_t k = b; k < en; k++) {
    const int64_t x = csr.ent[k];
    const float2* src = fe + 12 * (x >> 2) + 3 * (x & 3);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float2 v = src[c];
      a[c] = df32::df_add(a[c], df32::df{v.x, v.y});
    }
  }
#pragma unroll
  for (int c = 0; c < 3; c++) acc[c] = df32::to_f64(a[c]);
}

// FE = double: FP64 element forces; FE = float2: two-term ones (k_element_nh_df)
template <typename FE>
__global__ void __launch_bounds__(kThreads) k_gather_force(int64_t nbc, int64_t N, NodeCsr csr,
                                                           const FE* __restrict__ fe,
                                                           const double* __restrict__ mass,
                                                           const double* __restrict__ fext, double g0, double g1,
                                                           double g2, double ff, double* __restrict__ r,
                                                           Reduce red, double* rr_out, PressureView pv, DynView dv,
                                                           const double* __restrict__ u) {
  double acc = 0.0;
  for (int64_t g = nbc + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
    double f[3];
    gather_node(csr, fe, g, f);
    if (pv.n_tris > 0) {
      for (int k = pv.tptr[g]; k < pv.tptr[g + 1]; k++) {
        const int64_t t = pv.tent[k];
        f[0] += pv.ptf[3 * t];
        f[1] += pv.ptf[3 * t + 1];
        f[2] += pv.ptf[3 * t + 2];
      }
    }
    const double mf = mass[g] * ff;
    const double gr[3] = {g0, g1, g2};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double v = f[c] + mf * gr[c];
      if (dv.vel) {
        v += (mass[g] * dv.inv_h) * dv.vel[3 * g + c];
        v -= (mass[g] * dv.inv_h2) * (u[3 * g + c] - dv.u_start[3 * g + c]);
      }
      v += ff * fext[3 * g + c];
      r[3 * g + c] = v;
      acc += v * v;
    }
  }
  double v[1] = {acc}, tot[1];
  if (reduce_last<double, 1>(v, red, tot) && threadIdx.x == 0 && rr_out) *rr_out = tot[0];
}

void launch_gather_force(int64_t nbc, int64_t N, NodeCsr csr, const double* fe, const double* mass,
                         const double* fext, const double* grav, double ff, double* r, Reduce red, double* rr_out,
                         cudaStream_t st, const PressureView* pv, const DynView* dv, const double* u, bool fe_df) {
  count_launch();
  PressureView none{0, nullptr, nullptr, nullptr, nullptr, 0.0};
  DynView nodyn{nullptr, nullptr, 0.0, 0.0};
  if (fe_df)
    k_gather_force<float2><<<grid_for(N - nbc), kThreads, 0, st>>>(
        nbc, N, csr, reinterpret_cast<const float2*>(fe), mass, fext, grav[0], grav[1], grav[2], ff, r, red, rr_out,
        pv ? *pv : none, dv ? *dv : nodyn, u);
  else
    k_gather_force<double><<<grid_for(N - nbc), kThreads, 0, st>>>(nbc, N, csr, fe, mass, fext, grav[0], grav[1],
                                                                  grav[2], ff, r, red, rr_out, pv ? *pv : none,
                                                                  dv ? *dv : nodyn, u);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_gather_hvp(int64_t nbc, int64_t N, NodeCsr csr,
                                                         const T* __restrict__ fe, const T* __restrict__ p,
                                                         T* __restrict__ q, Reduce red, CgScalars* s) {
  if (s != nullptr && s->done) return;
  T acc = T(0);
  for (int64_t g = nbc + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
    T f[3];
    gather_node(csr, fe, g, f);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const T v = -f[c];
      q[3 * g + c] = v;
      acc += p[3 * g + c] * v;
    }
  }
  if (s == nullptr) return;
  T v[1] = {acc}, tot[1];
  if (reduce_last<T, 1>(v, red, tot) && threadIdx.x == 0) {
    const double pq = (double)tot[0];
    s->pq = pq;
    if (!isfinite(pq)) {
      s->done = 1;
      s->status = -3;
      s->alpha = 0.0;
    } else if (!(pq > 0.0)) {  // negative curvature: truncated CG stops here (status 2)
      s->done = 1;
      s->status = 2;
      s->alpha = 0.0;
    } else {
      s->alpha = s->rz / pq;
    }
  }
}

template <typename T>
void launch_gather_hvp(int64_t nbc, int64_t N, NodeCsr csr, const T* fe, const T* p, T* q, Reduce red, CgScalars* s,
                       cudaStream_t st) {
  count_launch();
  k_gather_hvp<T><<<grid_for(N - nbc), kThreads, 0, st>>>(nbc, N, csr, fe, p, q, red, s);
}
template void launch_gather_hvp<double>(int64_t, int64_t, NodeCsr, const double*, const double*, double*, Reduce,
                                        CgScalars*, cudaStream_t);
template void launch_gather_hvp<float>(int64_t, int64_t, NodeCsr, const float*, const float*, float*, Reduce,
                                       CgScalars*, cudaStream_t);

template <typename T>
__global__ void __launch_bounds__(kThreads) k_gather_diag(int64_t nbc, int64_t N, NodeCsr csr,
                                                          const T* __restrict__ fe, T* __restrict__ dinv,
                                                          T* __restrict__ diag, const double* __restrict__ mass,
                                                          double inv_h2) {
  for (int64_t g = nbc + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
    T f[3];
    gather_node(csr, fe, g, f);
    if (mass) {
      const T m = (T)(mass[g] * inv_h2);
      f[0] += m;
      f[1] += m;
      f[2] += m;
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
      if (diag) diag[3 * g + c] = f[c];
      if (dinv) dinv[3 * g + c] = T(1) / f[c];
    }
  }
}

template <typename T>
void launch_gather_diag(int64_t nbc, int64_t N, NodeCsr csr, const T* fe, T* dinv, T* diag, cudaStream_t st,
                        const double* mass, double inv_h2) {
  count_launch();
  k_gather_diag<T><<<grid_for(N - nbc), kThreads, 0, st>>>(nbc, N, csr, fe, dinv, diag, mass, inv_h2);
}
template void launch_gather_diag<double>(int64_t, int64_t, NodeCsr, const double*, double*, double*, cudaStream_t,
                                         const double*, double);
template void launch_gather_diag<float>(int64_t, int64_t, NodeCsr, const float*, float*, float*, cudaStream_t,
                                        const double*, double);

__global__ void __launch_bounds__(kThreads) k_adjoint_elem(const int4* __restrict__ tets, int64_t E, int64_t nbc,
                                                           const double* __restrict__ fe,
                                                           const double* __restrict__ lam,
                                                           const double* __restrict__ young_e,
                                                           const int32_t* __restrict__ perm,
                                                           double* __restrict__ dLdE) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const int4 t = tets[e];
    const int idx[4] = {t.x, t.y, t.z, t.w};
    double s = 0.0;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      if (idx[a] < nbc) continue;
#pragma unroll
      for (int c = 0; c < 3; c++) s += lam[3 * (int64_t)idx[a] + c] * fe[12 * e + 3 * a + c];
    }
    // young_e is in patch order; dLdE is written in the caller's element order
    dLdE[perm[e]] = s / young_e[e];
  }
}

void launch_adjoint_elem(const int4* tets, int64_t E, int64_t nbc, const double* fe, const double* lam,
                         const double* young_e, const int32_t* perm, double* dLdE, cudaStream_t st) {
  count_launch();
  k_adjoint_elem<<<grid_for(E, 152 * 12), kThreads, 0, st>>>(tets, E, nbc, fe, lam, young_e, perm, dLdE);
}

__global__ void k_permute(int64_t E, const int32_t* __restrict__ perm, const double* __restrict__ in,
                          double* __restrict__ out) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E; k += (int64_t)gridDim.x * blockDim.x)
    out[k] = in[perm[k]];
}
void launch_permute(int64_t E, const int32_t* perm, const double* in, double* out, cudaStream_t st) {
  count_launch();
  k_permute<<<grid_for(E), kThreads, 0, st>>>(E, perm, in, out);
}

// ---------------------------------------------------------------------------
// Fused patch Hessian-vector product
// ---------------------------------------------------------------------------
// One CTA per patch.  Phase 1 stages the patch's nodal u and p in shared memory
// (forming p = dinv r + beta p_old on the fly inside Krylov iterations), phase 2
// computes the 12 nodal values of every element into shared memory, phase 3 sums
// them per local node through the patch-local CSR (element order, deterministic)
// and writes q = -sum for nodes that only this patch touches, or a partial for
// shared nodes.  Block partials of p.q go to red.partials[c].

template <typename T>
struct ElemLoad {  // one element's data, loaded ahead of its use
  ushort4 li;
  T X[9];
  T vol, sc, scl;
};

// one element's row of the patch-product records: 16-byte loads (3 in FP32, 6 in FP64)
__device__ __forceinline__ void load_rec(const float* rec, int64_t e, float (&x)[9], float& vol, ushort4& li) {
  const float4* r4 = reinterpret_cast<const float4*>(rec + 12 * e);
  const float4 a = __ldg(r4), b = __ldg(r4 + 1), c = __ldg(r4 + 2);
  x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
  x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
  x[8] = c.x;
  vol = c.y;
  const uint32_t w0 = __float_as_uint(c.z), w1 = __float_as_uint(c.w);
  li = make_ushort4((unsigned short)(w0 & 0xffffu), (unsigned short)(w0 >> 16), (unsigned short)(w1 & 0xffffu),
                    (unsigned short)(w1 >> 16));
}
__device__ __forceinline__ void load_rec(const double* rec, int64_t e, double (&x)[9], double& vol, ushort4& li) {
  const double2* r2 = reinterpret_cast<const double2*>(rec + 12 * e);
  const double2 a = __ldg(r2), b = __ldg(r2 + 1), c = __ldg(r2 + 2), d = __ldg(r2 + 3), f = __ldg(r2 + 4),
                g = __ldg(r2 + 5);
  x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y; x[4] = c.x; x[5] = c.y; x[6] = d.x; x[7] = d.y; x[8] = f.x;
  vol = f.y;
  const unsigned long long w = (unsigned long long)__double_as_longlong(g.x);
  li = make_ushort4((unsigned short)(w & 0xffffu), (unsigned short)((w >> 16) & 0xffffu),
                    (unsigned short)((w >> 32) & 0xffffu), (unsigned short)(w >> 48));
}

template <typename T>
__device__ __forceinline__ void load_elem(const PatchView<T>& pv, int64_t e, ElemLoad<T>& d) {
  load_rec(pv.rec, e, d.X, d.vol, d.li);
  d.sc = pv.scale ? pv.scale[e] : T(1);
  d.scl = pv.scale_la ? pv.scale_la[e] : d.sc;
}

// Neo-Hookean tangent factors per element for the cached Hessian-vector product: F^-T (9),
// mu_e, lambda_e and c1 = mu_e - lambda_e log J, SoA cache[k E + e], k = 0..11 (one element pass
// at the start of every Krylov solve; the product then needs neither u nor F).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_nh_cache(ElemView<T> ev, const T* __restrict__ u, T* __restrict__ c) {
  const int64_t E = ev.E;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const int4 t = ev.tets[e];
    M3<T> X;
#pragma unroll
    for (int k = 0; k < 9; k++) X.a[k] = ev.X[k * E + e];
    T mu = ev.mu, la = ev.lambda;
    if (ev.scale) {
      const T sc = ev.scale[e];
      mu *= sc;
      la *= ev.scale_la ? ev.scale_la[e] : sc;
    }
    M3<T> F = grad_of(u, t, X);
    F.a[0] += T(1);
    F.a[4] += T(1);
    F.a[8] += T(1);
    Tangent<T, kNeoHookean> tg;
    tg.init(F, mu, la);
#pragma unroll
    for (int k = 0; k < 9; k++) c[k * E + e] = tg.Fit.a[k];
    c[9 * E + e] = tg.mu;
    c[10 * E + e] = tg.la;
    c[11 * E + e] = tg.c1;
  }
}
template <typename T>
void launch_nh_cache(const ElemView<T>& ev, const T* u, T* cache, cudaStream_t st) {
  count_launch();
  k_nh_cache<T><<<grid_for(ev.E), kThreads, 0, st>>>(ev, u, cache);
}
template void launch_nh_cache<double>(const ElemView<double>&, const double*, double*, cudaStream_t);
template void launch_nh_cache<float>(const ElemView<float>&, const float*, float*, cudaStream_t);

template <typename T, int MAT, int NT, bool DIR, bool CACHED>
__global__ void __launch_bounds__(NT) k_patch_hvp(PatchView<T> pv, const T* __restrict__ u,
                                                  const T* __restrict__ p, T* __restrict__ q,
                                                  T* __restrict__ partial, Reduce red, CgScalars* s,
                                                  const T* __restrict__ r, const T* __restrict__ dinv,
                                                  T* __restrict__ p_new, const T* __restrict__ z) {
  pdl_wait();
  pdl_launch_dependents();
  if (s != nullptr && s->done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sfe = reinterpret_cast<T*>(smem_raw);         // kPatchElems * kFeStride
  T* su = sfe + kPatchElems * kFeStride;           // max_nodes * 3 (not with CACHED)
  T* sp = CACHED ? su : su + pv.max_nodes * 3;     // max_nodes * 3
  const int c = blockIdx.x;
  const int64_t eb = pv.elem_off[c], ne = pv.elem_off[c + 1] - eb;
  const int64_t nb = pv.node_off[c];
  const int nn = (int)(pv.node_off[c + 1] - nb);
  T beta = T(0);
  bool use_z = false;  // flexible CG: p = z + beta p_old with z the preconditioner output
  if (DIR) {
    beta = (T)s->beta;
    use_z = z != nullptr && s->jac == 0;
  }
  for (int j = threadIdx.x; j < nn; j += NT) {
    int g = pv.pnode[nb + j];
    if (g < 0) g = ~g;
    const int64_t o = 3 * (int64_t)g;
    if (!CACHED) {
      su[3 * j] = u[o];
      su[3 * j + 1] = u[o + 1];
      su[3 * j + 2] = u[o + 2];
    }
    if (DIR) {
      // zero at fixed nodes: r, dinv, z and p stay zero there
      const T p0 = (use_z ? z[o] : dinv[o] * r[o]) + beta * p[o];
      const T p1 = (use_z ? z[o + 1] : dinv[o + 1] * r[o + 1]) + beta * p[o + 1];
      const T p2 = (use_z ? z[o + 2] : dinv[o + 2] * r[o + 2]) + beta * p[o + 2];
      sp[3 * j] = p0;
      sp[3 * j + 1] = p1;
      sp[3 * j + 2] = p2;
      // every patch that touches a node computes the same value from the same inputs
      if (g >= pv.nbc) {
        p_new[o] = p0;
        p_new[o + 1] = p1;
        p_new[o + 2] = p2;
      }
    } else {
      sp[3 * j] = p[o];
      sp[3 * j + 1] = p[o + 1];
      sp[3 * j + 2] = p[o + 2];
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < ne; k += NT) {
    ElemLoad<T> cur;
    load_elem(pv, eb + k, cur);
    const ushort4 li = cur.li;
    M3<T> X;
#pragma unroll
    for (int q9 = 0; q9 < 9; q9++) X.a[q9] = cur.X[q9];
    M3<T> Dp;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const T b0 = sp[3 * li.x + i];
      Dp.a[3 * i] = sp[3 * li.y + i] - b0;
      Dp.a[3 * i + 1] = sp[3 * li.z + i] - b0;
      Dp.a[3 * i + 2] = sp[3 * li.w + i] - b0;
    }
    M3<T> dP;
    if constexpr (CACHED) {
      Tangent<T, kNeoHookean> tg;
      const int64_t e = eb + k;
#pragma unroll
      for (int q9 = 0; q9 < 9; q9++) tg.Fit.a[q9] = pv.nhc[q9 * pv.E + e];
      tg.mu = pv.nhc[9 * pv.E + e];
      tg.la = pv.nhc[10 * pv.E + e];
      tg.c1 = pv.nhc[11 * pv.E + e];
      dP = tg.apply(mul(Dp, X));
    } else {
      const T mu = pv.mu * cur.sc, la = pv.lambda * cur.scl;
      M3<T> D;
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const T a0 = su[3 * li.x + i];
        D.a[3 * i] = su[3 * li.y + i] - a0;
        D.a[3 * i + 1] = su[3 * li.z + i] - a0;
        D.a[3 * i + 2] = su[3 * li.w + i] - a0;
      }
      M3<T> F = mul(D, X);
      F.a[0] += T(1);
      F.a[4] += T(1);
      F.a[8] += T(1);
      Tangent<T, MAT> tg;
      tg.init(F, mu, la);
      dP = tg.apply(mul(Dp, X));
    }
    T f[12];
    nodal_forces(dP, X, -cur.vol, f);
#pragma unroll
    for (int t = 0; t < 12; t++) sfe[kFeStride * k + t] = f[t];
  }
  __syncthreads();
  // p.q is linear in the partial sums, so shared nodes contribute p . partial here
  T acc = T(0);
  const uint16_t* lp = pv.lptr + nb + c;
  const uint16_t* le = pv.lent + 4 * eb;
  for (int j = threadIdx.x; j < nn; j += NT) {
    T f0 = T(0), f1 = T(0), f2 = T(0);
    const int t1 = lp[j + 1];
    for (int t = lp[j]; t < t1; t++) {
      const T* src = sfe + le[t];
      f0 += src[0];
      f1 += src[1];
      f2 += src[2];
    }
    if (pv.pm) {  // implicit dynamics: q = K p + (m / h^2) p (shared nodes: a share per patch)
      const T m = pv.pm[nb + j];
      f0 -= m * sp[3 * j];
      f1 -= m * sp[3 * j + 1];
      f2 -= m * sp[3 * j + 2];
    }
    const int g = pv.pnode[nb + j];
    int64_t o = -1;
    T* dst = q;
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
      acc -= sp[3 * j] * f0 + sp[3 * j + 1] * f1 + sp[3 * j + 2] * f2;
    }
  }
  T v[1] = {acc};
  block_sum<T, 1>(v);
  if (s == nullptr) return;
  __shared__ bool is_last;
  T* P = reinterpret_cast<T*>(red.partials);
  if (threadIdx.x == 0) {
    P[c] = v[0];
    __threadfence();
    is_last = atomicAdd(red.counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  T sum[1] = {T(0)};
  strided_sums<T, T, 1>(P, gridDim.x, gridDim.x, sum);
  block_sum<T, 1>(sum);
  if (threadIdx.x == 0) {
    *red.counter = 0u;
    const double pq = (double)sum[0];
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

// Shared free nodes: q = sum of the patch partials in patch order (used when the
// caller needs the complete vector q; the fused Krylov update sums them itself).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_patch_boundary(PatchBoundary pb, const T* __restrict__ partial,
                                                             T* __restrict__ q, const CgScalars* s) {
  if (s != nullptr && s->done) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < pb.n; i += (int64_t)gridDim.x * blockDim.x) {
    T f0 = T(0), f1 = T(0), f2 = T(0);
    const int t1 = pb.ptr[i + 1];
    for (int t = pb.ptr[i]; t < t1; t++) {
      f0 += partial[3 * (int64_t)t];
      f1 += partial[3 * (int64_t)t + 1];
      f2 += partial[3 * (int64_t)t + 2];
    }
    const int64_t o = 3 * (int64_t)pb.node[i];
    q[o] = f0;
    q[o + 1] = f1;
    q[o + 2] = f2;
  }
}

// q at node g: from q (nodes of one patch, slot.y == 0) or the sum of its patch partials
// partial[slot.x .. slot.x + slot.y) in patch order (shared nodes)
template <typename T>
__device__ __forceinline__ void node_q(const T* __restrict__ q, const T* __restrict__ partial, int2 slot, int64_t o,
                                       T (&qq)[3]) {
  if (slot.y == 0) {
    qq[0] = q[o];
    qq[1] = q[o + 1];
    qq[2] = q[o + 2];
  } else {
    qq[0] = qq[1] = qq[2] = T(0);
    const int t1 = slot.x + slot.y;
    for (int t = slot.x; t < t1; t++) {
      qq[0] += partial[3 * (int64_t)t];
      qq[1] += partial[3 * (int64_t)t + 1];
      qq[2] += partial[3 * (int64_t)t + 2];
    }
  }
}

// Fused Krylov update over nodes: q_g from q or the node's patch partials (node_q), then
// x += alpha p, r -= alpha q, z = dinv r, r.z and r.r with the fixed-order last-block finish
// (beta, convergence test).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_update_patch(int64_t nbc, int64_t N, const int2* __restrict__ bslot,
                                                              const T* __restrict__ partial,
                                                              T* __restrict__ x, T* __restrict__ r,
                                                              const T* __restrict__ p, const T* __restrict__ q,
                                                              const T* __restrict__ dinv, Reduce red, CgScalars* s) {
  pdl_wait();
  pdl_launch_dependents();
  if (s->done) return;
  const T a = (T)s->alpha;
  T rz = T(0), rr = T(0);
  for (int64_t g = nbc + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = 3 * g;
    T qq[3];
    node_q(q, partial, bslot ? bslot[g] : make_int2(0, 0), o, qq);
#pragma unroll
    for (int c2 = 0; c2 < 3; c2++) {
      x[o + c2] += a * p[o + c2];
      const T ri = r[o + c2] - a * qq[c2];
      r[o + c2] = ri;
      rz += ri * (dinv[o + c2] * ri);
      rr += ri * ri;
    }
  }
  T v[2] = {rz, rr}, tot[2];
  if (reduce_last<T, 2>(v, red, tot) && threadIdx.x == 0) {
    const double rzn = (double)tot[0];
    s->beta = rzn / s->rz;
    s->rz = rzn;
    s->rr = (double)tot[1];
    s->it += 1;
    if (!isfinite(s->rr)) {
      s->done = 1;
      s->status = -3;
    } else if (s->rr <= s->tol2) {
      s->done = 1;
    } else if (s->it >= s->max_it) {
      s->done = 1;
      s->status = 1;
    }
  }
}

// Flexible-CG update over nodes: q_g from q (owned) or its patch partials (shared), then
// x += alpha p, rprev = r, r -= alpha q and r.r with the fixed-order last-block finish.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_fcg_update_patch(int64_t nbc, int64_t N,
                                                               const int2* __restrict__ bslot,
                                                               const T* __restrict__ partial, T* __restrict__ x,
                                                               T* __restrict__ r, T* __restrict__ rprev,
                                                               const T* __restrict__ p, const T* __restrict__ q,
                                                               Reduce red, CgScalars* s, const T* __restrict__ dinv,
                                                               gnn::Row16* __restrict__ xs, float* __restrict__ xstat) {
  pdl_wait();
  pdl_launch_dependents();
  if (s->done) return;
  const T a = (T)s->alpha;
  T rr = T(0);
  float xx = 0.f;
  // the rows' scale from the previous rows' sum (xstat[0] is overwritten by the last block only,
  // after every block has read it)
  const float sg = xs ? gnn::row16_scale(xstat[0], 3 * (N - nbc)) : 1.f;
  if (xs && blockIdx.x == 0 && threadIdx.x == 0) xstat[1] = sg;
  for (int64_t g = nbc + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = 3 * g;
    T qq[3];
    node_q(q, partial, bslot ? bslot[g] : make_int2(0, 0), o, qq);
    T rn[3];
#pragma unroll
    for (int c2 = 0; c2 < 3; c2++) {
      x[o + c2] += a * p[o + c2];
      const T rp = r[o + c2];
      rprev[o + c2] = rp;
      rn[c2] = rp - a * qq[c2];
      r[o + c2] = rn[c2];
      rr += rn[c2] * rn[c2];
    }
    if (xs) {  // the preconditioner's input sigma D^-1/2 r
      float xv[3];
#pragma unroll
      for (int c2 = 0; c2 < 3; c2++) {
        const float d = (float)dinv[o + c2], rv = (float)rn[c2];
        xx += d * rv * rv;
        xv[c2] = sg * rv * sqrtf(d);
      }
      xs[g - nbc] = gnn::pack16(xv[0], xv[1], xv[2]);
    }
  }
  T v[2] = {rr, (T)xx}, tot[2];
  if (reduce_last<T, 2>(v, red, tot) && threadIdx.x == 0) {
    if (xs) xstat[0] = (float)tot[1];
    s->rr = (double)tot[0];
    s->it += 1;
    if (!isfinite(s->rr)) {
      s->done = 1;
      s->status = -3;
    } else if (s->rr <= s->tol2) {
      s->done = 1;
    } else if (s->it >= s->max_it) {
      s->done = 1;
      s->status = 1;
    }
  }
}

// The flexible-CG update when q is complete (the assembled operator: no shared-node partials), over
// groups of four nodes: twelve consecutive values, three 16-byte loads or stores per array.  Groups
// start at the first node g0 >= nbc with g0 % 4 == 0 (12 g0 bytes then 16-byte aligned); the nodes
// before g0 and after the last whole group are updated one by one.
__device__ __forceinline__ void fcg_node(int64_t g, float a, float* __restrict__ x, float* __restrict__ r,
                                         float* __restrict__ rprev, const float* __restrict__ p,
                                         const float* __restrict__ q, const float* __restrict__ dinv,
                                         gnn::Row16* __restrict__ xs, float sg, int64_t nbc, float& rr, float& xx,
                                         float (&rn)[3]) {
  const int64_t o = 3 * g;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    x[o + c] += a * p[o + c];
    const float rp = r[o + c];
    rprev[o + c] = rp;
    rn[c] = rp - a * q[o + c];
    r[o + c] = rn[c];
    rr += rn[c] * rn[c];
  }
  if (xs) {
    float xv[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float d = dinv[o + c];
      xx += d * rn[c] * rn[c];
      xv[c] = sg * rn[c] * sqrtf(d);
    }
    xs[g - nbc] = gnn::pack16(xv[0], xv[1], xv[2]);
  }
}
__device__ __forceinline__ void ld12(const float* __restrict__ a, float (&v)[12]) {
  const float4* a4 = reinterpret_cast<const float4*>(a);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float4 t = a4[k];
    v[4 * k] = t.x;
    v[4 * k + 1] = t.y;
    v[4 * k + 2] = t.z;
    v[4 * k + 3] = t.w;
  }
}
__device__ __forceinline__ void st12(float* __restrict__ a, const float (&v)[12]) {
  float4* a4 = reinterpret_cast<float4*>(a);
#pragma unroll
  for (int k = 0; k < 3; k++) a4[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
}
__global__ void __launch_bounds__(kThreads) k_fcg_update_vec(int64_t nbc, int64_t N, float* __restrict__ x,
                                                             float* __restrict__ r, float* __restrict__ rprev,
                                                             const float* __restrict__ p, const float* __restrict__ q,
                                                             Reduce red, CgScalars* s, const float* __restrict__ dinv,
                                                             gnn::Row16* __restrict__ xs, float* __restrict__ xstat) {
  pdl_wait();
  pdl_launch_dependents();
  if (s->done) return;
  const float a = (float)s->alpha;
  float rr = 0.f, xx = 0.f;
  // the rows' scale from the previous rows' sum (xstat[0] is overwritten by the last block only,
  // after every block has read it)
  const float sg = xs ? gnn::row16_scale(xstat[0], 3 * (N - nbc)) : 1.f;
  if (xs && blockIdx.x == 0 && threadIdx.x == 0) xstat[1] = sg;
  const int64_t g0a = (nbc + 3) & ~(int64_t)3, g0 = g0a < N ? g0a : N;
  const int64_t ng = (N - g0) / 4, gend = g0 + 4 * ng;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = tid; k < ng; k += stride) {
    const int64_t g = g0 + 4 * k, o = 3 * g;
    float xv[12], rv[12], pv[12], qv[12], dv[12];
    ld12(x + o, xv);
    ld12(r + o, rv);
    ld12(p + o, pv);
    ld12(q + o, qv);
    if (xs) ld12(dinv + o, dv);
    st12(rprev + o, rv);
    float rn[12];
#pragma unroll
    for (int i = 0; i < 12; i++) {
      xv[i] += a * pv[i];
      rn[i] = rv[i] - a * qv[i];
      rr += rn[i] * rn[i];
    }
    st12(x + o, xv);
    st12(r + o, rn);
    if (xs) {
#pragma unroll
      for (int i = 0; i < 12; i++) xx += dv[i] * rn[i] * rn[i];
#pragma unroll
      for (int m = 0; m < 4; m++)
        xs[g + m - nbc] = gnn::pack16(sg * rn[3 * m] * sqrtf(dv[3 * m]), sg * rn[3 * m + 1] * sqrtf(dv[3 * m + 1]),
                                      sg * rn[3 * m + 2] * sqrtf(dv[3 * m + 2]));
    }
  }
  // the nodes before the first group and after the last
  const int64_t nhead = g0 - nbc, ntail = N - gend;
  float rn1[3];
  if (tid < nhead) fcg_node(nbc + tid, a, x, r, rprev, p, q, dinv, xs, sg, nbc, rr, xx, rn1);
  else if (tid < nhead + ntail) fcg_node(gend + (tid - nhead), a, x, r, rprev, p, q, dinv, xs, sg, nbc, rr, xx, rn1);
  float v[2] = {rr, xx}, tot[2];
  if (reduce_last<float, 2>(v, red, tot) && threadIdx.x == 0) {
    if (xs) xstat[0] = tot[1];
    s->rr = (double)tot[0];
    s->it += 1;
    if (!isfinite(s->rr)) {
      s->done = 1;
      s->status = -3;
    } else if (s->rr <= s->tol2) {
      s->done = 1;
    } else if (s->it >= s->max_it) {
      s->done = 1;
      s->status = 1;
    }
  }
}

// k_fcg_update_vec with the coarse restriction's run sums fused in (two-level preconditioner): CTA c
// takes restriction blocks 2c and 2c + 1 in turn (so the grid is one resident wave at the bench's
// size), each block's 256 groups one per thread (block 0 also the nodes before the first group, the
// last block those after the last group; coarse_block_start); it stages each node's six restriction
// terms from the new r in shared memory and sums the block's runs like k_coarse_runs, so that r is
// not read again for the restriction.  Four CTAs per SM (at most 64 registers).
__global__ void __launch_bounds__(kThreads, 4) k_fcg_update_runs(int64_t nbc, int64_t N, float* __restrict__ x,
                                                              float* __restrict__ r, float* __restrict__ rprev,
                                                              const float* __restrict__ p, const float* __restrict__ q,
                                                              Reduce red, CgScalars* s, const float* __restrict__ dinv,
                                                              gnn::Row16* __restrict__ xs, float* __restrict__ xstat,
                                                              CoarseView cv) {
  __shared__ float sv[6][kCoarseSpan];
  pdl_wait();
  pdl_launch_dependents();
  if (s->done) return;
  const float a = (float)s->alpha;
  float rr = 0.f, xx = 0.f;
  const float sg = xs ? gnn::row16_scale(xstat[0], 3 * (N - nbc)) : 1.f;
  if (xs && blockIdx.x == 0 && threadIdx.x == 0) xstat[1] = sg;
  const int64_t g0a = (nbc + 3) & ~(int64_t)3, g0 = g0a < N ? g0a : N;
  const int64_t ng = (N - g0) / 4, gend = g0 + 4 * ng;
  const int64_t nhead = g0 - nbc, ntail = N - gend;
  for (int half = 0; half < 2; half++) {
    const int b = 2 * blockIdx.x + half;  // the same for the whole CTA
    if (b >= cv.n_blocks) break;
    if (half) __syncthreads();  // the previous block's runs have read sv
    const int64_t base = coarse_block_start(b, cv.n_blocks, cv.blk_off, cv.nf);
    const int64_t k = (int64_t)b * kThreads + threadIdx.x;
    if (k < ng) {
      const int64_t g = g0 + 4 * k, o = 3 * g;
      float xv[12], rv[12], pv[12], qv[12], dv[12];
      ld12(x + o, xv);
      ld12(r + o, rv);
      ld12(p + o, pv);
      ld12(q + o, qv);
      if (xs) ld12(dinv + o, dv);
      st12(rprev + o, rv);
      float rn[12];
#pragma unroll
      for (int i = 0; i < 12; i++) {
        xv[i] += a * pv[i];
        rn[i] = rv[i] - a * qv[i];
        rr += rn[i] * rn[i];
      }
      st12(x + o, xv);
      st12(r + o, rn);
      if (xs) {
#pragma unroll
        for (int i = 0; i < 12; i++) xx += dv[i] * rn[i] * rn[i];
#pragma unroll
        for (int m = 0; m < 4; m++)
          xs[g + m - nbc] = gnn::pack16(sg * rn[3 * m] * sqrtf(dv[3 * m]), sg * rn[3 * m + 1] * sqrtf(dv[3 * m + 1]),
                                        sg * rn[3 * m + 2] * sqrtf(dv[3 * m + 2]));
      }
#pragma unroll
      for (int m = 0; m < 4; m++) coarse_stage(cv, g + m - nbc, base, rn[3 * m], rn[3 * m + 1], rn[3 * m + 2], sv);
    }
    // the nodes before the first group (block 0) and after the last (the last block)
    float rn1[3];
    if (b == 0 && threadIdx.x < nhead) {
      const int64_t g = nbc + threadIdx.x;
      fcg_node(g, a, x, r, rprev, p, q, dinv, xs, sg, nbc, rr, xx, rn1);
      coarse_stage(cv, g - nbc, base, rn1[0], rn1[1], rn1[2], sv);
    }
    if (b == cv.n_blocks - 1 && threadIdx.x < ntail) {
      const int64_t g = gend + threadIdx.x;
      fcg_node(g, a, x, r, rprev, p, q, dinv, xs, sg, nbc, rr, xx, rn1);
      coarse_stage(cv, g - nbc, base, rn1[0], rn1[1], rn1[2], sv);
    }
    __syncthreads();
    coarse_block_runs(cv, b, base, sv);
  }
  float v[2] = {rr, xx}, tot[2];
  if (reduce_last<float, 2>(v, red, tot) && threadIdx.x == 0) {
    if (xs) xstat[0] = tot[1];
    s->rr = (double)tot[0];
    s->it += 1;
    if (!isfinite(s->rr)) {
      s->done = 1;
      s->status = -3;
    } else if (s->rr <= s->tol2) {
      s->done = 1;
    } else if (s->it >= s->max_it) {
      s->done = 1;
      s->status = 1;
    }
  }
}

template <typename T>
bool launch_fcg_update_patch(int64_t nbc, int64_t N, const int2* bslot, const T* partial, T* x,
                             T* r, T* rprev, const T* p, const T* q, Reduce red, CgScalars* s, cudaStream_t st,
                             const T* dinv, gnn::Row16* xs, float* xstat, const CoarseView* cv) {
  if constexpr (std::is_same<T, float>::value) {
    if (bslot == nullptr && cv && cv->n_blocks > 0 && cv->n_blocks <= 8 * kMaxBlocks) {
      // q complete, with the coarse run sums: one CTA per two restriction blocks (the reduction's
      // partials hold 2 floats per CTA: 8 kMaxBlocks floats of the 4 kMaxBlocks doubles)
      count_launch();
      launch_pdl(k_fcg_update_runs, (unsigned)((cv->n_blocks + 1) / 2), kThreads, 0, st, nbc, N, x, r, rprev, p, q, red,
                 s, dinv, xs, xstat, *cv);
      return true;
    }
    if (bslot == nullptr) {  // q complete: the grouped update
      static const int wave_v = resident_ctas(k_fcg_update_vec, kThreads, 0);
      const int64_t groups = (N - nbc) / 4 + 1;
      count_launch();
      launch_pdl(k_fcg_update_vec, std::max(1, (int)std::min<int64_t>(wave_v, (groups + kThreads - 1) / kThreads)),
                 kThreads, 0, st, nbc, N, x, r, rprev, p, q, red, s, dinv, xs, xstat);
      return false;
    }
  }
  count_launch();
  static const int wave = resident_ctas(k_fcg_update_patch<T>, kThreads, 0);
  launch_pdl(k_fcg_update_patch<T>, std::min(grid_for(N - nbc), wave), kThreads, 0, st, nbc, N, bslot, partial, x, r,
             rprev, p, q, red, s, dinv, xs, xstat);
  return false;
}
template bool launch_fcg_update_patch<float>(int64_t, int64_t, const int2*, const float*, float*,
                                             float*, float*, const float*, const float*, Reduce, CgScalars*,
                                             cudaStream_t, const float*, gnn::Row16*, float*, const CoarseView*);

// 12 consecutive values (4 nodes) with 16-byte loads and stores, FP64
__device__ __forceinline__ void ld12(const double* __restrict__ a, double (&v)[12]) {
  const double2* a2 = reinterpret_cast<const double2*>(a);
#pragma unroll
  for (int k = 0; k < 6; k++) {
    const double2 t = a2[k];
    v[2 * k] = t.x;
    v[2 * k + 1] = t.y;
  }
}
__device__ __forceinline__ void st12(double* __restrict__ a, const double (&v)[12]) {
  double2* a2 = reinterpret_cast<double2*>(a);
#pragma unroll
  for (int k = 0; k < 6; k++) a2[k] = make_double2(v[2 * k], v[2 * k + 1]);
}

// The preconditioned-CG update when q is complete (the assembled operator), over groups of four
// nodes as k_fcg_update_vec: x += alpha p, r -= alpha q, r.(D^-1 r) and r.r, then beta and the
// convergence test in the last block.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_update_vec(int64_t nbc, int64_t N, T* __restrict__ x,
                                                            T* __restrict__ r, const T* __restrict__ p,
                                                            const T* __restrict__ q, const T* __restrict__ dinv,
                                                            Reduce red, CgScalars* s) {
  pdl_wait();
  pdl_launch_dependents();
  if (s->done) return;
  const T a = (T)s->alpha;
  T rz = T(0), rr = T(0);
  const int64_t g0a = (nbc + 3) & ~(int64_t)3, g0 = g0a < N ? g0a : N;
  const int64_t ng = (N - g0) / 4, gend = g0 + 4 * ng;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = tid; k < ng; k += stride) {
    const int64_t o = 3 * (g0 + 4 * k);
    T xv[12], rv[12], pv[12], qv[12], dv[12];
    ld12(x + o, xv);
    ld12(r + o, rv);
    ld12(p + o, pv);
    ld12(q + o, qv);
    ld12(dinv + o, dv);
#pragma unroll
    for (int i = 0; i < 12; i++) {
      xv[i] += a * pv[i];
      rv[i] -= a * qv[i];
      rz += rv[i] * (dv[i] * rv[i]);
      rr += rv[i] * rv[i];
    }
    st12(x + o, xv);
    st12(r + o, rv);
  }
  const int64_t nhead = g0 - nbc, ntail = N - gend;
  int64_t g = -1;
  if (tid < nhead) g = nbc + tid;
  else if (tid < nhead + ntail) g = gend + (tid - nhead);
  if (g >= 0) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const int64_t o = 3 * g + c;
      x[o] += a * p[o];
      const T ri = r[o] - a * q[o];
      r[o] = ri;
      rz += ri * (dinv[o] * ri);
      rr += ri * ri;
    }
  }
  T v[2] = {rz, rr}, tot[2];
  if (reduce_last<T, 2>(v, red, tot) && threadIdx.x == 0) {
    const double rzn = (double)tot[0];
    s->beta = rzn / s->rz;
    s->rz = rzn;
    s->rr = (double)tot[1];
    s->it += 1;
    if (!isfinite(s->rr)) {
      s->done = 1;
      s->status = -3;
    } else if (s->rr <= s->tol2) {
      s->done = 1;
    } else if (s->it >= s->max_it) {
      s->done = 1;
      s->status = 1;
    }
  }
}

template <typename T>
void launch_cg_update_patch(int64_t nbc, int64_t N, const int2* bslot, const T* partial, T* x,
                            T* r, const T* p, const T* q, const T* dinv, Reduce red, CgScalars* s, cudaStream_t st) {
  if (bslot == nullptr) {  // q complete: the grouped update
    static const int wave_v = resident_ctas(k_cg_update_vec<T>, kThreads, 0);
    const int64_t groups = (N - nbc) / 4 + 1;
    count_launch();
    launch_pdl(k_cg_update_vec<T>, std::max(1, (int)std::min<int64_t>(wave_v, (groups + kThreads - 1) / kThreads)),
               kThreads, 0, st, nbc, N, x, r, p, q, dinv, red, s);
    return;
  }
  count_launch();
  static const int wave = resident_ctas(k_cg_update_patch<T>, kThreads, 0);
  launch_pdl(k_cg_update_patch<T>, std::min(grid_for(N - nbc), wave), kThreads, 0, st, nbc, N, bslot, partial, x, r, p,
             q, dinv, red, s);
}
template void launch_cg_update_patch<double>(int64_t, int64_t, const int2*, const double*, double*,
                                             double*, const double*, const double*, const double*, Reduce,
                                             CgScalars*, cudaStream_t);
template void launch_cg_update_patch<float>(int64_t, int64_t, const int2*, const float*, float*,
                                            float*, const float*, const float*, const float*, Reduce, CgScalars*,
                                            cudaStream_t);

template <typename T, int MAT>
void launch_patch_hvp(const PatchView<T>& pv, PatchBoundary pb, const T* u, const T* p, T* q, T* partial, Reduce red,
                      CgScalars* s, cudaStream_t st, cudaEvent_t mid, const T* r, const T* dinv, T* p_new,
                      const T* z) {
  constexpr int NT = 256;
  constexpr bool kNH = MAT == kNeoHookean;
  const bool cached = kNH && pv.nhc != nullptr;
  constexpr size_t smem_max = sizeof(T) * (kPatchElems * kFeStride + kPatchNodes * 6);
  const size_t smem = sizeof(T) * (kPatchElems * kFeStride + (size_t)pv.max_nodes * 6);
  const size_t smem_c = sizeof(T) * (kPatchElems * kFeStride + (size_t)pv.max_nodes * 3);
  static bool attr_set = false;  // per instantiation
  if (!attr_set) {
    const int mx = (int)smem_max;
    cudaFuncSetAttribute(k_patch_hvp<T, MAT, NT, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_patch_hvp<T, MAT, NT, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    if (kNH) {
      cudaFuncSetAttribute(k_patch_hvp<T, MAT, NT, false, kNH>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
      cudaFuncSetAttribute(k_patch_hvp<T, MAT, NT, true, kNH>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    }
    attr_set = true;
  }
  if constexpr (std::is_same<T, float>::value && kNH) {
    if (!cached && pv.lent12 != nullptr) {  // the FP32 neo-Hookean product (sfem_patch_nh32.cu)
      launch_patch_hvp_nh32(pv, u, p, q, partial, red, s, st, r, dinv, p_new, z);
      if (mid) cudaEventRecord(mid, st);
      if (p_new != nullptr) return;  // Krylov iteration: the fused update completes the shared nodes
      count_launch();
      k_patch_boundary<T><<<grid_for(pb.n), kThreads, 0, st>>>(pb, partial, q, s);
      return;
    }
  }
  const unsigned grid = (unsigned)pv.n_patches;
  count_launch();
  if (p_new != nullptr) {
    // Krylov iteration: the fused update (k_cg_update_patch) completes the shared nodes
    if (cached)
      launch_pdl(k_patch_hvp<T, MAT, NT, true, kNH>, grid, NT, smem_c, st, pv, u, p, q, partial, red, s, r, dinv, p_new,
                 z);
    else
      launch_pdl(k_patch_hvp<T, MAT, NT, true, false>, grid, NT, smem, st, pv, u, p, q, partial, red, s, r, dinv, p_new,
                 z);
    if (mid) cudaEventRecord(mid, st);
    return;
  }
  if (cached)
    k_patch_hvp<T, MAT, NT, false, kNH><<<grid, NT, smem_c, st>>>(pv, u, p, q, partial, red, s, nullptr, nullptr,
                                                                  nullptr, nullptr);
  else
    k_patch_hvp<T, MAT, NT, false, false><<<grid, NT, smem, st>>>(pv, u, p, q, partial, red, s, nullptr, nullptr,
                                                                  nullptr, nullptr);
  if (mid) cudaEventRecord(mid, st);
  count_launch();
  k_patch_boundary<T><<<grid_for(pb.n), kThreads, 0, st>>>(pb, partial, q, s);
}

#define SFEM_INST_PATCH(T, M)                                                                                   \
  template void launch_patch_hvp<T, M>(const PatchView<T>&, PatchBoundary, const T*, const T*, T*, T*, Reduce, \
                                       CgScalars*, cudaStream_t, cudaEvent_t, const T*, const T*, T*, const T*);
SFEM_INST_PATCH(double, 0)
SFEM_INST_PATCH(double, 1)
SFEM_INST_PATCH(double, 2)
SFEM_INST_PATCH(double, 3)
SFEM_INST_PATCH(double, 4)
SFEM_INST_PATCH(double, 5)
SFEM_INST_PATCH(double, 6)
SFEM_INST_PATCH(double, 7)
SFEM_INST_PATCH(double, 8)
SFEM_INST_PATCH(double, 9)
SFEM_INST_PATCH(double, 10)
SFEM_INST_PATCH(double, 11)
SFEM_INST_PATCH(double, 12)
SFEM_INST_PATCH(double, 13)
SFEM_INST_PATCH(float, 0)
SFEM_INST_PATCH(float, 1)
SFEM_INST_PATCH(float, 2)
SFEM_INST_PATCH(float, 3)
SFEM_INST_PATCH(float, 4)

// ---------------------------------------------------------------------------
// Krylov vector kernels over the free-DOF range (pointers pre-offset)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_init(int64_t n, const T* __restrict__ b, T* __restrict__ x,
                                                      T* __restrict__ r, T* __restrict__ p,
                                                      const T* __restrict__ dinv, Reduce red, CgScalars* s) {
  T rz = T(0), bb = T(0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T ri = b[i];
    const T zi = dinv ? ri * dinv[i] : ri;
    x[i] = T(0);
    r[i] = ri;
    p[i] = zi;
    rz += ri * zi;
    bb += ri * ri;
  }
  T v[2] = {rz, bb}, tot[2];
  if (reduce_last<T, 2>(v, red, tot) && threadIdx.x == 0) {
    s->rz = (double)tot[0];
    s->bb = (double)tot[1];
    s->rr = (double)tot[1];
    s->tol2 = s->tol2 * (double)tot[1];
    s->it = 0;
    s->beta = 0.0;
    s->status = 0;
    s->done = (tot[1] == T(0)) ? 1 : 0;
    if (!isfinite(s->bb)) {
      s->done = 1;
      s->status = -3;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_update(int64_t n, T* __restrict__ x, T* __restrict__ r,
                                                        const T* __restrict__ p, const T* __restrict__ q,
                                                        const T* __restrict__ dinv, Reduce red, CgScalars* s) {
  if (s->done) return;
  const T a = (T)s->alpha;
  T rz = T(0), rr = T(0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += a * p[i];
    const T ri = r[i] - a * q[i];
    r[i] = ri;
    const T zi = dinv ? ri * dinv[i] : ri;
    rz += ri * zi;
    rr += ri * ri;
  }
  T v[2] = {rz, rr}, tot[2];
  if (reduce_last<T, 2>(v, red, tot) && threadIdx.x == 0) {
    const double rzn = (double)tot[0];
    s->beta = rzn / s->rz;
    s->rz = rzn;
    s->rr = (double)tot[1];
    s->it += 1;
    if (!isfinite(s->rr)) {
      s->done = 1;
      s->status = -3;
    } else if (s->rr <= s->tol2) {
      s->done = 1;
    } else if (s->it >= s->max_it) {
      s->done = 1;
      s->status = 1;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_direction(int64_t n, const T* __restrict__ r,
                                                           const T* __restrict__ dinv, T* __restrict__ p,
                                                           const CgScalars* s) {
  if (s->done) return;
  const T beta = (T)s->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T zi = dinv ? r[i] * dinv[i] : r[i];
    p[i] = zi + beta * p[i];
  }
}

template <typename T>
void launch_cg_init(int64_t n, const T* b, T* x, T* r, T* p, const T* dinv, Reduce red, CgScalars* s,
                    cudaStream_t st) {
  count_launch();
  k_cg_init<T><<<grid_for(n), kThreads, 0, st>>>(n, b, x, r, p, dinv, red, s);
}
template <typename T>
void launch_cg_update(int64_t n, T* x, T* r, const T* p, const T* q, const T* dinv, Reduce red, CgScalars* s,
                      cudaStream_t st) {
  count_launch();
  k_cg_update<T><<<grid_for(n), kThreads, 0, st>>>(n, x, r, p, q, dinv, red, s);
}
template <typename T>
void launch_cg_direction(int64_t n, const T* r, const T* dinv, T* p, const CgScalars* s, cudaStream_t st) {
  count_launch();
  k_cg_direction<T><<<grid_for(n), kThreads, 0, st>>>(n, r, dinv, p, s);
}
#define SFEM_INST_CG(T)                                                                                        \
  template void launch_cg_init<T>(int64_t, const T*, T*, T*, T*, const T*, Reduce, CgScalars*, cudaStream_t); \
  template void launch_cg_update<T>(int64_t, T*, T*, const T*, const T*, const T*, Reduce, CgScalars*,        \
                                    cudaStream_t);                                                             \
  template void launch_cg_direction<T>(int64_t, const T*, const T*, T*, const CgScalars*, cudaStream_t);
SFEM_INST_CG(double)
SFEM_INST_CG(float)

// ---------------------------------------------------------------------------
// Independent instances (batched solves): per-segment norms and masks
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_segment_norms(const int64_t* __restrict__ seg,
                                                            const double* __restrict__ v, double* __restrict__ out) {
  const int k = blockIdx.x;
  double acc = 0.0;
  for (int64_t i = seg[k] + threadIdx.x; i < seg[k + 1]; i += blockDim.x) acc += v[i] * v[i];
  double a[1] = {acc};
  block_sum<double, 1>(a);
  if (threadIdx.x == 0) out[k] = sqrt(a[0]);
}
void launch_segment_norms(int k, const int64_t* seg, const double* v, double* out, cudaStream_t st) {
  count_launch();
  k_segment_norms<<<k, kThreads, 0, st>>>(seg, v, out);
}

template <typename T>
__global__ void k_segment_mask(const int64_t* __restrict__ seg, const int32_t* __restrict__ active, T* __restrict__ v) {
  const int k = blockIdx.x;
  if (active[k]) return;
  for (int64_t i = seg[k] + threadIdx.x; i < seg[k + 1]; i += blockDim.x) v[i] = T(0);
}
template <typename T>
void launch_segment_mask(int k, const int64_t* seg, const int32_t* active, T* v, cudaStream_t st) {
  count_launch();
  k_segment_mask<T><<<k, kThreads, 0, st>>>(seg, active, v);
}
template void launch_segment_mask<double>(int, const int64_t*, const int32_t*, double*, cudaStream_t);
template void launch_segment_mask<float>(int, const int64_t*, const int32_t*, float*, cudaStream_t);

// ---------------------------------------------------------------------------
// Misc
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_dot(int64_t n, const double* __restrict__ a,
                                                  const double* __restrict__ b, Reduce red, double* out) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += a[i] * b[i];
  double v[1] = {acc}, tot[1];
  if (reduce_last<double, 1>(v, red, tot) && threadIdx.x == 0) *out = tot[0];
}
void launch_dot(int64_t n, const double* a, const double* b, Reduce red, double* out, cudaStream_t st) {
  count_launch();
  k_dot<<<grid_for(n), kThreads, 0, st>>>(n, a, b, red, out);
}

__global__ void __launch_bounds__(kThreads) k_potential(int64_t nbc, int64_t N, const double* __restrict__ x0,
                                                        const double* __restrict__ u,
                                                        const double* __restrict__ mass,
                                                        const double* __restrict__ fext, double g0, double g1,
                                                        double g2, double ff, Reduce red, double* out, DynView dv) {
  double acc = 0.0;
  const double gr[3] = {g0, g1, g2};
  for (int64_t g = nbc + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const double x = x0[3 * g + c] + u[3 * g + c];
      acc -= ff * (mass[g] * gr[c] + fext[3 * g + c]) * x;
      if (dv.vel) {  // inertia of backward Euler: m / (2 h^2) |x - x_start - h v|^2
        const double d = u[3 * g + c] - dv.u_start[3 * g + c] - dv.vel[3 * g + c] / dv.inv_h;
        acc += 0.5 * mass[g] * dv.inv_h2 * d * d;
      }
    }
  }
  double v[1] = {acc}, tot[1];
  if (reduce_last<double, 1>(v, red, tot) && threadIdx.x == 0) *out = tot[0];
}
void launch_potential(int64_t nbc, int64_t N, const double* x0, const double* u, const double* mass,
                      const double* fext, const double* grav, double ff, Reduce red, double* out, cudaStream_t st,
                      const DynView* dv) {
  count_launch();
  DynView nodyn{nullptr, nullptr, 0.0, 0.0};
  k_potential<<<grid_for(N - nbc), kThreads, 0, st>>>(nbc, N, x0, u, mass, fext, grav[0], grav[1], grav[2], ff, red,
                                                     out, dv ? *dv : nodyn);
}

template <typename T>
__global__ void k_patch_mass(int64_t n_slots, int64_t nbc, const int32_t* __restrict__ pnode,
                             const int32_t* __restrict__ bidx, PatchBoundary pb, const double* __restrict__ mass,
                             double inv_h2, T* __restrict__ pm) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_slots; s += (int64_t)gridDim.x * blockDim.x) {
    int g = pnode[s];
    const bool shared = g < 0;
    if (shared) g = ~g;
    double m = 0.0;
    if (g >= nbc) {
      m = mass[g] * inv_h2;
      const int b = shared ? bidx[g] : -1;
      if (b >= 0) m /= (double)(pb.ptr[b + 1] - pb.ptr[b]);
    }
    pm[s] = (T)m;
  }
}
template <typename T>
void launch_patch_mass(int64_t n_slots, int64_t nbc, const int32_t* pnode, const int32_t* bidx, PatchBoundary pb,
                       const double* mass, double inv_h2, T* pm, cudaStream_t st) {
  count_launch();
  k_patch_mass<T><<<grid_for(n_slots), kThreads, 0, st>>>(n_slots, nbc, pnode, bidx, pb, mass, inv_h2, pm);
}
template void launch_patch_mass<double>(int64_t, int64_t, const int32_t*, const int32_t*, PatchBoundary,
                                        const double*, double, double*, cudaStream_t);
template void launch_patch_mass<float>(int64_t, int64_t, const int32_t*, const int32_t*, PatchBoundary,
                                       const double*, double, float*, cudaStream_t);

__global__ void k_explicit_substep(int64_t nbc, int64_t N, const double* __restrict__ f,
                                   const double* __restrict__ mass, double g0, double g1, double g2, double hs,
                                   double* __restrict__ vel, double* __restrict__ u) {
  const double gr[3] = {g0, g1, g2};
  for (int64_t g = nbc + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < N; g += (int64_t)gridDim.x * blockDim.x) {
    if (mass[g] == 0.0) continue;
    const double a = hs * (1.0 / mass[g]);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const double v = vel[3 * g + c] + (a * f[3 * g + c] + hs * gr[c]);
      vel[3 * g + c] = v;
      u[3 * g + c] += hs * v;
    }
  }
}
void launch_explicit_substep(int64_t nbc, int64_t N, const double* f, const double* mass, const double* grav,
                             double hs, double* vel, double* u, cudaStream_t st) {
  count_launch();
  k_explicit_substep<<<grid_for(N - nbc), kThreads, 0, st>>>(nbc, N, f, mass, grav[0], grav[1], grav[2], hs, vel, u);
}

__global__ void k_velocity_update(int64_t nbc, int64_t N, const double* __restrict__ u,
                                  const double* __restrict__ us, double inv_h, double* __restrict__ vel) {
  for (int64_t i = 3 * nbc + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * N;
       i += (int64_t)gridDim.x * blockDim.x)
    vel[i] = inv_h * (u[i] - us[i]);
}
void launch_velocity_update(int64_t nbc, int64_t N, const double* u, const double* u_start, double inv_h,
                            double* vel, cudaStream_t st) {
  count_launch();
  k_velocity_update<<<grid_for(3 * (N - nbc)), kThreads, 0, st>>>(nbc, N, u, u_start, inv_h, vel);
}

// Node vectors between the caller's node order and the reshuffled device order (map: original ->
// reshuffled), so host arrays travel as one contiguous copy and the permutation runs here.
// in:  dst[3 map[i] + c] = src[3 i + c] - sub[3 map[i] + c] (sub optional), zero where map[i] < nzero
// out: dst[3 i + c] = a[3 map[i] + c] + b[3 map[i] + c] (b optional)
__global__ void k_nodes_in(int64_t N, const int32_t* __restrict__ map, const double* __restrict__ src,
                           const double* __restrict__ sub, int64_t nzero, double* __restrict__ dst) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < 3 * N; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = k / 3, c = k - 3 * i, g = map[i];
    const int64_t o = 3 * g + c;
    dst[o] = g < nzero ? 0.0 : src[k] - (sub ? sub[o] : 0.0);
  }
}
__global__ void k_nodes_out(int64_t N, const int32_t* __restrict__ map, const double* __restrict__ a,
                            const double* __restrict__ b, double* __restrict__ dst) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < 3 * N; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = k / 3, c = k - 3 * i;
    const int64_t o = 3 * (int64_t)map[i] + c;
    dst[k] = a[o] + (b ? b[o] : 0.0);
  }
}
void launch_nodes_in(int64_t N, const int32_t* map, const double* src, const double* sub, int64_t nzero, double* dst,
                     cudaStream_t st) {
  count_launch();
  k_nodes_in<<<grid_for(3 * N), kThreads, 0, st>>>(N, map, src, sub, nzero, dst);
}
void launch_nodes_out(int64_t N, const int32_t* map, const double* a, const double* b, double* dst, cudaStream_t st) {
  count_launch();
  k_nodes_out<<<grid_for(3 * N), kThreads, 0, st>>>(N, map, a, b, dst);
}

template <typename Tin, typename Tout>
__global__ void k_convert(int64_t n, const Tin* __restrict__ a, Tout* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (Tout)a[i];
}
template <typename Tin, typename Tout>
void launch_convert(int64_t n, const Tin* a, Tout* b, cudaStream_t st) {
  count_launch();
  k_convert<Tin, Tout><<<grid_for(n), kThreads, 0, st>>>(n, a, b);
}
template void launch_convert<double, float>(int64_t, const double*, float*, cudaStream_t);
template void launch_convert<float, double>(int64_t, const float*, double*, cudaStream_t);

// ---------------------------------------------------------------------------
// Batched independent bodies: every instance's PCG in one persistent cooperative launch
// ---------------------------------------------------------------------------
// Grid-wide barrier of a cooperative launch whose wait is bounded: after `limit` polls (or once
// another block has reported a failure) it sets *err and returns false; every block then leaves.
__device__ __forceinline__ bool grid_sync_bounded(unsigned* bar, int32_t* err, long long limit) {
  __shared__ int fail;
  __syncthreads();
  if (threadIdx.x == 0) {
    fail = 0;
    volatile unsigned* gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long it = 0;
      while (*gen == g) {
        if (*(volatile int32_t*)err != 0 || ++it > limit) {
          atomicCAS(err, 0, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    fail = *(volatile int32_t*)err != 0;
  }
  __syncthreads();
  return fail == 0;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// fixed-order sum of component c of instance k's tile partials (every warp gets the same bits)
__device__ __forceinline__ double inst_sum(const BatchPcg& b, int k, int c, int lane) {
  double v = 0.0;
  const int t1 = __ldcg(b.inst_tile + k + 1);
  for (int t = __ldcg(b.inst_tile + k) + lane; t < t1; t += 32) v += __ldcg(b.part + 3 * t + c);
  return warp_sum_d(v);
}

template <typename T>
__device__ __forceinline__ void load3cg(const T* a, int g, T* o) {
  o[0] = __ldcg(a + 3 * (int64_t)g);
  o[1] = __ldcg(a + 3 * (int64_t)g + 1);
  o[2] = __ldcg(a + 3 * (int64_t)g + 2);
}

// Phases per iteration (each followed by a grid barrier): A element products K_e p of the running
// instances; B q = K p at every free node (node->element CSR, element order) and the tiles' p.q;
// C alpha_k = r.z_k / p.q_k, x += alpha p, r -= alpha q, z = D^-1 r and the tiles' r.z, r.r;
// D beta_k, the instance's convergence test (r.r <= tol^2 b.b) and p = z + beta p.  Data written by
// other blocks during the launch is read with L2 loads (__ldcg).
template <typename T, int MAT>
__global__ void __launch_bounds__(kThreads) k_batched_pcg(ElemView<T> ev, NodeCsr csr, BatchPcg b,
                                                          const T* __restrict__ u, const T* __restrict__ rhs, T* x,
                                                          T* r, T* z, T* p, T* q, const T* __restrict__ dinv, T* fe) {
  const int lane = threadIdx.x & 31;
  const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), nw = (int)((gridDim.x * blockDim.x) >> 5);
  const int K = b.K;
  const int64_t nbc = b.nbc, E = ev.E;
  if (b.wait_test && blockIdx.x == 0 && threadIdx.x == 0) {
    // a flag that nothing sets: the bounded wait gives up and reports it
    volatile unsigned* never = b.bar + 2;
    long long it = 0;
    while (*never == 0u) {
      if (++it > b.wait_limit) {
        atomicCAS(b.err, 0, 2);
        break;
      }
      __nanosleep(64);
    }
  }
  // x = 0, r = b, z = D^-1 r, p = z; tile partials of r.z and r.r (a warp sums in T, the tiles in FP64)
  for (int t = gw; t < b.n_tiles; t += nw) {
    T rz = T(0), rr = T(0);
    if (lane < b.tile_cnt[t]) {
      const int64_t o = 3 * (nbc + b.tile_node[t] + lane);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const T ri = rhs[o + c], zi = dinv[o + c] * ri;
        x[o + c] = T(0);
        r[o + c] = ri;
        z[o + c] = zi;
        p[o + c] = zi;
        rz += ri * zi;
        rr += ri * ri;
      }
    }
    rz = warp_sum_t(rz);
    rr = warp_sum_t(rr);
    if (lane == 0) {
      b.part[3 * t] = 0.0;
      b.part[3 * t + 1] = (double)rz;
      b.part[3 * t + 2] = (double)rr;
    }
  }
  if (!grid_sync_bounded(b.bar, b.err, b.wait_limit)) return;
  for (int k = gw; k < K; k += nw) {  // one warp per instance writes its start values
    const double rz = inst_sum(b, k, 1, lane), rr = inst_sum(b, k, 2, lane);
    if (lane == 0) {
      b.rz[k] = rz;
      b.tol2bb[k] = b.tol * b.tol * rr;
      b.done[k] = rr > 0.0 ? 0 : 1;
      b.done[2 * K + k] = rr > 0.0 ? 0 : 1;
      b.iters[k] = 0;
      b.rr[k] = rr;
    }
  }
  if (!grid_sync_bounded(b.bar, b.err, b.wait_limit)) return;
  for (int it = 0; it < b.max_it; it++) {
    const int cur = it & 1, nxt = cur ^ 1;
    const int32_t* done = b.done + cur * K;
    // A: element products
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
      if (__ldcg(done + b.einst[e]) != 0) continue;
      const int4 t4 = ev.tets[e];
      M3<T> X;
#pragma unroll
      for (int k9 = 0; k9 < 9; k9++) X.a[k9] = ev.X[k9 * E + e];
      const T vol = ev.vol[e];
      T mu = ev.mu, la = ev.lambda;
      if (ev.scale) {
        const T sc = ev.scale[e];
        mu *= sc;
        la *= ev.scale_la ? ev.scale_la[e] : sc;
      }
      M3<T> F = grad_of(u, t4, X);
      F.a[0] += T(1);
      F.a[4] += T(1);
      F.a[8] += T(1);
      Tangent<T, MAT> tg;
      tg.init(F, mu, la);
      T a0[3], a1[3], a2[3], a3[3];
      load3cg(p, t4.x, a0);
      load3cg(p, t4.y, a1);
      load3cg(p, t4.z, a2);
      load3cg(p, t4.w, a3);
      M3<T> D;
#pragma unroll
      for (int i = 0; i < 3; i++) {
        D.a[3 * i] = a1[i] - a0[i];
        D.a[3 * i + 1] = a2[i] - a0[i];
        D.a[3 * i + 2] = a3[i] - a0[i];
      }
      const M3<T> dP = tg.apply(mul(D, X));
      T f[12];
      nodal_forces(dP, X, -vol, f);
      store12(fe, e, f);
    }
    if (!grid_sync_bounded(b.bar, b.err, b.wait_limit)) return;
    // B: q at the free nodes of the running instances, tile p.q
    for (int t = gw; t < b.n_tiles; t += nw) {
      const int k = b.tile_inst[t];
      T pq = T(0);
      if (__ldcg(done + k) == 0 && lane < b.tile_cnt[t]) {
        const int64_t g = nbc + b.tile_node[t] + lane;
        T f0 = T(0), f1 = T(0), f2 = T(0);
        for (int64_t c = csr.ptr[g]; c < csr.ptr[g + 1]; c++) {
          const int64_t ent = csr.ent[c];
          const T* src = fe + 12 * (ent >> 2) + 3 * (ent & 3);
          f0 += __ldcg(src);
          f1 += __ldcg(src + 1);
          f2 += __ldcg(src + 2);
        }
        const int64_t o = 3 * g;
        q[o] = -f0;
        q[o + 1] = -f1;
        q[o + 2] = -f2;
        pq = -(__ldcg(p + o) * f0 + __ldcg(p + o + 1) * f1 + __ldcg(p + o + 2) * f2);
      }
      pq = warp_sum_t(pq);
      if (lane == 0) b.part[3 * t] = (double)pq;
    }
    if (!grid_sync_bounded(b.bar, b.err, b.wait_limit)) return;
    // C: alpha and the updates, tile r.z and r.r
    for (int t = gw; t < b.n_tiles; t += nw) {
      const int k = b.tile_inst[t];
      T rz = T(0), rr = T(0);
      if (__ldcg(done + k) == 0) {
        const double pq = inst_sum(b, k, 0, lane);
        const double alpha = (isfinite(pq) && pq > 0.0) ? __ldcg(b.rz + cur * K + k) / pq : 0.0;
        if (lane < b.tile_cnt[t]) {
          const int64_t o = 3 * (nbc + b.tile_node[t] + lane);
          const T a = (T)alpha;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const T pi = __ldcg(p + o + c), qi = __ldcg(q + o + c);
            x[o + c] = __ldcg(x + o + c) + a * pi;
            const T ri = __ldcg(r + o + c) - a * qi, zi = dinv[o + c] * ri;
            r[o + c] = ri;
            z[o + c] = zi;
            rz += ri * zi;
            rr += ri * ri;
          }
        }
      }
      rz = warp_sum_t(rz);
      rr = warp_sum_t(rr);
      if (lane == 0) {
        b.part[3 * t + 1] = (double)rz;
        b.part[3 * t + 2] = (double)rr;
      }
    }
    if (!grid_sync_bounded(b.bar, b.err, b.wait_limit)) return;
    // D: beta, convergence, directions
    for (int t = gw; t < b.n_tiles; t += nw) {
      const int k = b.tile_inst[t];
      const bool lead = t == b.inst_tile[k] && lane == 0;
      if (__ldcg(done + k) != 0) {
        if (lead) b.done[nxt * K + k] = __ldcg(done + k);
        continue;
      }
      const double pq = inst_sum(b, k, 0, lane), rzn = inst_sum(b, k, 1, lane), rr = inst_sum(b, k, 2, lane);
      int st = 0;
      if (!isfinite(pq) || !isfinite(rzn)) st = 4;
      else if (!(pq > 0.0)) st = 2;
      else if (rr <= __ldcg(b.tol2bb + k)) st = 1;
      else if (it + 1 >= b.max_it) st = 3;
      if (st == 2 && it == 0 && lane < b.tile_cnt[t]) {  // truncated at once: the preconditioned residual
        const int64_t o = 3 * (nbc + b.tile_node[t] + lane);
#pragma unroll
        for (int c = 0; c < 3; c++) x[o + c] = __ldcg(p + o + c);
      }
      if (st == 0 && lane < b.tile_cnt[t]) {
        const T beta = (T)(rzn / __ldcg(b.rz + cur * K + k));
        const int64_t o = 3 * (nbc + b.tile_node[t] + lane);
#pragma unroll
        for (int c = 0; c < 3; c++) p[o + c] = __ldcg(z + o + c) + beta * __ldcg(p + o + c);
      }
      if (lead) {
        b.done[nxt * K + k] = st;
        b.done[2 * K + k] = st;
        b.rz[nxt * K + k] = rzn;
        b.iters[k] = st == 2 ? it : it + 1;
        b.rr[k] = rr;
      }
    }
    if (!grid_sync_bounded(b.bar, b.err, b.wait_limit)) return;
    __shared__ int all_done;
    if (threadIdx.x == 0) {
      int a = 1;
      for (int k = 0; k < K && a; k++) a = __ldcg(b.done + nxt * K + k) != 0;
      all_done = a;
    }
    __syncthreads();
    if (all_done) break;
  }
}

template <typename T>
int launch_batched_pcg(int mat, const ElemView<T>& ev, NodeCsr csr, const BatchPcg& b, const T* u, const T* rhs, T* x,
                       T* r, T* z, T* p, T* q, const T* dinv, T* fe, cudaStream_t st) {
  void (*kern)(ElemView<T>, NodeCsr, BatchPcg, const T*, const T*, T*, T*, T*, T*, T*, const T*, T*) = nullptr;
  switch (mat) {
    case kLinear: kern = k_batched_pcg<T, kLinear>; break;
    case kStvk: kern = k_batched_pcg<T, kStvk>; break;
    case kNeoHookean: kern = k_batched_pcg<T, kNeoHookean>; break;
    default: return -1;
  }
  int dev = 0, sms = 0, per = 0, coop = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (!coop) return -2;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kThreads, 0);
  if (per < 1) return -2;
  const unsigned grid = (unsigned)(per * sms);
  ElemView<T> ev_ = ev;
  NodeCsr csr_ = csr;
  BatchPcg b_ = b;
  const T *u_ = u, *rhs_ = rhs, *dinv_ = dinv;
  T *x_ = x, *r_ = r, *z_ = z, *p_ = p, *q_ = q, *fe_ = fe;
  void* args[] = {&ev_, &csr_, &b_, &u_, &rhs_, &x_, &r_, &z_, &p_, &q_, &dinv_, &fe_};
  count_launch();
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(kThreads), args, 0, st) == cudaSuccess ? 0 : -3;
}
template int launch_batched_pcg<float>(int, const ElemView<float>&, NodeCsr, const BatchPcg&, const float*, const float*,
                                       float*, float*, float*, float*, float*, const float*, float*, cudaStream_t);
template int launch_batched_pcg<double>(int, const ElemView<double>&, NodeCsr, const BatchPcg&, const double*,
                                        const double*, double*, double*, double*, double*, double*, const double*,
                                        double*, cudaStream_t);

template <typename T>
__global__ void k_axpy_state(int64_t n, double a, const T* __restrict__ d, const double* __restrict__ base,
                             double* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = base[i] + a * (double)d[i];
}
template <typename T>
void launch_axpy_state(int64_t n, double a, const T* d, const double* base, double* x, cudaStream_t st) {
  count_launch();
  k_axpy_state<T><<<grid_for(n), kThreads, 0, st>>>(n, a, d, base, x);
}
template void launch_axpy_state<double>(int64_t, double, const double*, const double*, double*, cudaStream_t);
template void launch_axpy_state<float>(int64_t, double, const float*, const double*, double*, cudaStream_t);

__global__ void k_scale_copy(int64_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}
void launch_scale_copy(int64_t n, double a, const double* x, double* y, cudaStream_t st) {
  count_launch();
  k_scale_copy<<<grid_for(n), kThreads, 0, st>>>(n, a, x, y);
}

}  // namespace sfem
