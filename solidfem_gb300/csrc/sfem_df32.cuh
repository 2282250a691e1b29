// Two-term FP32 arithmetic ("double-float"): a value is hi + lo with |lo| <= ulp(hi) / 2, about 48
// significant bits, evaluated on the FP32 pipes.  GB300's FP64 rate is a small fraction of its FP32
// rate, so FP64-accurate element arithmetic runs faster this way.
//
// Building blocks (published error-free transformations, written here from their definitions):
//   two_sum        Knuth's TwoSum: s + e == a + b exactly, s = RN(a + b);
//   quick_two_sum  Dekker's Fast2Sum (|a| >= |b|);
//   two_prod       the FMA form of Dekker's product: p + e == a * b exactly, p = RN(a * b);
//   df_add         Joldes, Muller, Popescu (ACM TOMS 2017) "AccurateDWPlusDW": relative error
//                  below 3u^2 (u = 2^-24) even under cancellation;
//   df_mul         the same paper's DWTimesDW with one FMA for the cross terms;
//   df_rcp         one Newton step from the FP32 reciprocal, the residual 1 - y * r formed with FMA;
//   DfSum          compensated summation and dot products (Ogita, Rump, Oishi, SIAM J. Sci. Comput.
//                  2005, Sum2 / Dot2): the leading parts summed by TwoSum chains, every rounding
//                  error, the low parts and the cross products collected in a second FP32 sum.
// Every rounding-sensitive step uses the _rn intrinsics, which the compiler never contracts into
// FMAs, so the transformations stay exact.  Inputs come from FP64 through an integer split
// (no FP64 instructions); magnitudes below 2^-100 are taken as zero.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef __CUDACC__
#include <cuda_runtime.h>
#else  // plain C++ (the host check of this arithmetic)
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace sfem {
namespace df32 {

#ifdef __CUDA_ARCH__
#define SFEM_DF_ADD(a, b) __fadd_rn(a, b)
#define SFEM_DF_SUB(a, b) __fsub_rn(a, b)
#define SFEM_DF_MUL(a, b) __fmul_rn(a, b)
#define SFEM_DF_FMA(a, b, c) __fmaf_rn(a, b, c)
#define SFEM_DF_RCP(a) __frcp_rn(a)
#else
#define SFEM_DF_ADD(a, b) ((a) + (b))
#define SFEM_DF_SUB(a, b) ((a) - (b))
#define SFEM_DF_MUL(a, b) ((a) * (b))
#define SFEM_DF_FMA(a, b, c) fmaf(a, b, c)
#define SFEM_DF_RCP(a) (1.0f / (a))
#endif

struct df {
  float hi, lo;
};

__host__ __device__ __forceinline__ df two_sum(float a, float b) {
  const float s = SFEM_DF_ADD(a, b);
  const float bb = SFEM_DF_SUB(s, a);
  const float e = SFEM_DF_ADD(SFEM_DF_SUB(a, SFEM_DF_SUB(s, bb)), SFEM_DF_SUB(b, bb));
  return {s, e};
}
__host__ __device__ __forceinline__ df quick_two_sum(float a, float b) {
  const float s = SFEM_DF_ADD(a, b);
  return {s, SFEM_DF_SUB(b, SFEM_DF_SUB(s, a))};
}
__host__ __device__ __forceinline__ df two_prod(float a, float b) {
  const float p = SFEM_DF_MUL(a, b);
  return {p, SFEM_DF_FMA(a, b, -p)};
}

__host__ __device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__host__ __device__ __forceinline__ df df_scale2(df a, float p2) { return {a.hi * p2, a.lo * p2}; }  // p2 = 2^k

__host__ __device__ __forceinline__ df df_add(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  const df t = two_sum(x.lo, y.lo);
  const float c = SFEM_DF_ADD(s.lo, t.hi);
  const df v = quick_two_sum(s.hi, c);
  const float w = SFEM_DF_ADD(t.lo, v.lo);
  return quick_two_sum(v.hi, w);
}
// same-sign operands (no cancellation): the sloppy form is as accurate
__host__ __device__ __forceinline__ df df_add_same_sign(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  const float v = SFEM_DF_ADD(x.lo, y.lo);
  return quick_two_sum(s.hi, SFEM_DF_ADD(s.lo, v));
}
__host__ __device__ __forceinline__ df df_add_f(df x, float b) {
  const df s = two_sum(x.hi, b);
  const df v = quick_two_sum(s.hi, SFEM_DF_ADD(s.lo, x.lo));
  return v;
}
__host__ __device__ __forceinline__ df df_mul(df x, df y) {
  const df c = two_prod(x.hi, y.hi);
  const float t = SFEM_DF_MUL(x.hi, y.lo);
  const float cl = SFEM_DF_ADD(c.lo, SFEM_DF_FMA(x.lo, y.hi, t));
  return quick_two_sum(c.hi, cl);
}
__host__ __device__ __forceinline__ df df_mul_f(df x, float b) {
  const df c = two_prod(x.hi, b);
  return quick_two_sum(c.hi, SFEM_DF_FMA(x.lo, b, c.lo));
}
__host__ __device__ __forceinline__ df df_rcp(df y) {
  const float r = SFEM_DF_RCP(y.hi);
  // e = 1 - y r in two-term precision: 1 - y.hi r is exact with one FMA for r = RN(1 / y.hi)
  const float e = SFEM_DF_FMA(-y.lo, r, SFEM_DF_FMA(-y.hi, r, 1.0f));
  return quick_two_sum(r, SFEM_DF_MUL(r, e));
}
__host__ __device__ __forceinline__ df df_div(df x, df y) { return df_mul(x, df_rcp(y)); }

// compensated sum: s holds the running TwoSum chain of leading parts, c everything else
struct DfSum {
  float s = 0.0f, c = 0.0f;
  __host__ __device__ __forceinline__ void add(float a) {
    const df t = two_sum(s, a);
    s = t.hi;
    c = SFEM_DF_ADD(c, t.lo);
  }
  __host__ __device__ __forceinline__ void add(df a) {
    add(a.hi);
    c = SFEM_DF_ADD(c, a.lo);
  }
  __host__ __device__ __forceinline__ void sub(df a) { add(df_neg(a)); }
  // + a b (the low parts' product, below u^2 |a b|, left out)
  __host__ __device__ __forceinline__ void add_prod(df a, df b) {
    const df p = two_prod(a.hi, b.hi);
    add(p.hi);
    c = SFEM_DF_ADD(c, SFEM_DF_ADD(p.lo, SFEM_DF_FMA(a.hi, b.lo, SFEM_DF_MUL(a.lo, b.hi))));
  }
  __host__ __device__ __forceinline__ void sub_prod(df a, df b) { add_prod(df_neg(a), b); }
  __host__ __device__ __forceinline__ df value() const { return two_sum(s, c); }
};

// FP64 -> two-term FP32 by integer operations: hi takes the leading 24 significand bits
// (truncated), lo the next 29 (rounded to 24), then the pair is renormalised.
__host__ __device__ __forceinline__ df split_f64(double x) {
#ifdef __CUDA_ARCH__
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  memcpy(&b, &x, sizeof(b));
#endif
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const int e = (int)((hw >> 20) & 0x7ffu);
  if (e < 1023 - 100) return {0.0f, 0.0f};                         // zero, subnormal or below 2^-100
  if (e > 1023 + 127) {  // beyond FP32, infinite or NaN
    const float big = (e == 0x7ff && ((hw & 0xfffffu) | lw)) ? NAN : INFINITY;
    return {(hw >> 31) ? -big : big, 0.0f};
  }
  const unsigned sign = hw & 0x80000000u;
  const unsigned hb = sign | ((unsigned)(e - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
  float h;
#ifdef __CUDA_ARCH__
  h = __uint_as_float(hb);
#else
  memcpy(&h, &hb, sizeof(h));
#endif
  // the remaining 29 bits r weigh r 2^(E - 52), E = e - 1023: (r 2^-29) 2^(E - 23), E - 23 >= -123
  const unsigned r = lw & 0x1fffffffu;
  const unsigned pb = (unsigned)(e - 1023 - 23 + 127) << 23;
  float p;
#ifdef __CUDA_ARCH__
  p = __uint_as_float(pb);
#else
  memcpy(&p, &pb, sizeof(p));
#endif
  float l = SFEM_DF_MUL(SFEM_DF_MUL((float)r, 1.0f / 536870912.0f), p);
  if (sign) l = -l;
  return quick_two_sum(h, l);
}
__host__ __device__ __forceinline__ double to_f64(df a) { return (double)a.hi + (double)a.lo; }

// log(1 + x) for a two-term x > -1: 2 atanh(s), s = x / (2 + x), by its series s + s^3/3 + s^5/5 ...
// (all terms of one sign), up to 14 terms for |s| <= 1/4; outside that (J below 0.6 or above 1.67)
// from the FP64 log1p.  x <= -1 gives NaN (an inverted element).
__host__ __device__ __forceinline__ df log1p_df(df x) {
  if (!(x.hi > -1.0f)) return {NAN, 0.0f};
  const df s = df_div(x, df_add_f(x, 2.0f));
  if (fabsf(s.hi) > 0.25f) {
    const double l = log1p(to_f64(x));
    return split_f64(l);
  }
  const df s2 = df_mul(s, s);
  df sum = s, pw = s;
#pragma unroll
  for (int k = 1; k <= 14; k++) {
    pw = df_mul(pw, s2);
    const df term = df_mul(pw, df_rcp(df{(float)(2 * k + 1), 0.0f}));
    sum = df_add_same_sign(sum, term);
    if (fabsf(term.hi) <= 8.9e-16f * fabsf(sum.hi)) break;  // 2^-50
  }
  return df_scale2(sum, 2.0f);
}

// One neo-Hookean element (ElasticEnergy.cpp:170-186 stress, :80-86 energy) from D = [u1 - u0,
// u2 - u0, u3 - u0] (row-major, two-term), X = Dm^-1 (row-major), V, mu, lambda: the 12 nodal forces
// -V P X^T (node 0 first, components inner) and, with energy, V psi.  Formed on H = F - I:
//   cof(F) = I + G   (G: each cofactor's linear and quadratic terms in H),
//   J - 1 = H00 + G00 + H00 G00 + H01 G01 + H02 G02,   l = log1p(J - 1),
//   P = mu H + [(mu (J - 1) + lambda l) I + (lambda l - mu) G] / J,
//   psi = mu (tr H - l) + mu/2 |H|^2 + lambda/2 l^2,
// so that no term of order one cancels.  Returns true for an inverted element (J <= 0; the forces are
// then NaN, as log J is).
__host__ __device__ __forceinline__ bool nh_element(const df (&D)[9], const df (&X)[9], df vol, df mu, df la,
                                                    bool energy, df (&f)[12], df* psi_v) {
  df H[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      DfSum sm;
#pragma unroll
      for (int k = 0; k < 3; k++) sm.add_prod(D[3 * i + k], X[3 * k + j]);
      H[3 * i + j] = sm.value();
    }
  // G = cof(I + H) - I, entry (i, j) the cofactor of F_ij
  df G[9];
  {
    DfSum a, b, c;
    a.add(H[4]), a.add(H[8]), a.add_prod(H[4], H[8]), a.sub_prod(H[5], H[7]);
    b.add(H[0]), b.add(H[8]), b.add_prod(H[0], H[8]), b.sub_prod(H[2], H[6]);
    c.add(H[0]), c.add(H[4]), c.add_prod(H[0], H[4]), c.sub_prod(H[1], H[3]);
    G[0] = a.value(), G[4] = b.value(), G[8] = c.value();
  }
  {
    DfSum g1, g2, g3, g5, g6, g7;
    g1.add_prod(H[5], H[6]), g1.sub(H[3]), g1.sub_prod(H[3], H[8]);  // F12 F20 - F10 F22
    g2.add_prod(H[3], H[7]), g2.sub(H[6]), g2.sub_prod(H[4], H[6]);  // F10 F21 - F11 F20
    g3.add_prod(H[2], H[7]), g3.sub(H[1]), g3.sub_prod(H[1], H[8]);  // F02 F21 - F01 F22
    g5.add_prod(H[1], H[6]), g5.sub(H[7]), g5.sub_prod(H[0], H[7]);  // F01 F20 - F00 F21
    g6.add_prod(H[1], H[5]), g6.sub(H[2]), g6.sub_prod(H[2], H[4]);  // F01 F12 - F02 F11
    g7.add_prod(H[2], H[3]), g7.sub(H[5]), g7.sub_prod(H[0], H[5]);  // F02 F10 - F00 F12
    G[1] = g1.value(), G[2] = g2.value(), G[3] = g3.value();
    G[5] = g5.value(), G[6] = g6.value(), G[7] = g7.value();
  }
  df jm1;
  {
    DfSum s;
    s.add(H[0]), s.add(G[0]), s.add_prod(H[0], G[0]), s.add_prod(H[1], G[1]), s.add_prod(H[2], G[2]);
    jm1 = s.value();
  }
  const df J = df_add_f(jm1, 1.0f);
  const df l = log1p_df(jm1);
  const df iJ = df_rcp(J);
  const df lal = df_mul(la, l);
  const df A = df_mul(df_add(lal, df_neg(mu)), iJ);
  const df B = df_mul(df_add(df_mul(mu, jm1), lal), iJ);
  const df nvol = df_neg(vol);
  df Pv[9];  // -V P
#pragma unroll
  for (int q = 0; q < 9; q++) {
    DfSum sm;
    sm.add_prod(mu, H[q]);
    sm.add_prod(A, G[q]);
    if (q == 0 || q == 4 || q == 8) sm.add(B);
    Pv[q] = df_mul(sm.value(), nvol);
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      DfSum sm;
#pragma unroll
      for (int j = 0; j < 3; j++) sm.add_prod(Pv[3 * c + j], X[3 * k + j]);
      f[3 * (k + 1) + c] = sm.value();
    }
    DfSum s0;
    s0.sub(f[3 + c]), s0.sub(f[6 + c]), s0.sub(f[9 + c]);
    f[c] = s0.value();
  }
  if (energy) {
    DfSum tr, h2, psi;
    tr.add(H[0]), tr.add(H[4]), tr.add(H[8]), tr.sub(l);
#pragma unroll
    for (int q = 0; q < 9; q++) h2.add_prod(H[q], H[q]);
    psi.add_prod(mu, tr.value());
    psi.add_prod(df_scale2(mu, 0.5f), h2.value());
    psi.add_prod(df_scale2(la, 0.5f), df_mul(l, l));
    *psi_v = df_mul(psi.value(), vol);
  }
  return J.hi <= 0.0f;
}

#undef SFEM_DF_ADD
#undef SFEM_DF_SUB
#undef SFEM_DF_MUL
#undef SFEM_DF_FMA
#undef SFEM_DF_RCP

}  // namespace df32
}  // namespace sfem
