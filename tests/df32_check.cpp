// Host check of the two-term FP32 arithmetic (solidfem_gb300/csrc/sfem_df32.cuh) that the FP32
// handles' neo-Hookean residual runs on the GPU: the same header compiled as plain C++, against
// quad-precision evaluations (__float128 on x86-64, long double where that is IEEE quad).  Prints
// one "name value" line per measured quantity; the Python test (test_df32_host.py) holds the bounds.
//
//   g++ -O2 -ffp-contract=off -I solidfem_gb300/csrc tests/df32_check.cpp -o df32_check -lquadmath
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include <random>

#include "sfem_df32.cuh"

using sfem::df32::df;
#if defined(__x86_64__)
#include <quadmath.h>
typedef __float128 ld;
static ld fabsl(ld x) { return x < 0 ? -x : x; }
static ld fmaxl(ld a, ld b) { return a > b ? a : b; }
static ld logl(ld x) { return logq(x); }
static ld log1pl(ld x) { return log1pq(x); }
static ld ldexpl(ld x, int e) { return ldexpq(x, e); }
#else
typedef long double ld;
#endif

static ld val(df a) { return (ld)a.hi + (ld)a.lo; }
static df geo_split(double x) {  // the device's X / V split: hi = RN(x), lo = RN(x - hi)
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}

// neo-Hookean forces -V P X^T and V psi in quad precision, the naive formula of ElasticEnergy.cpp:170-186 / :80-86
static bool nh_ref(const double D[9], const double X[9], double vol, double mu, double la, ld f[12], ld* psi) {
  ld F[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      ld s = 0;
      for (int k = 0; k < 3; k++) s += (ld)D[3 * i + k] * (ld)X[3 * k + j];
      F[3 * i + j] = s + (i == j ? 1 : 0);
    }
  const ld C[9] = {F[4] * F[8] - F[5] * F[7], F[5] * F[6] - F[3] * F[8], F[3] * F[7] - F[4] * F[6],
                   F[2] * F[7] - F[1] * F[8], F[0] * F[8] - F[2] * F[6], F[1] * F[6] - F[0] * F[7],
                   F[1] * F[5] - F[2] * F[4], F[2] * F[3] - F[0] * F[5], F[0] * F[4] - F[1] * F[3]};
  const ld J = F[0] * C[0] + F[1] * C[1] + F[2] * C[2];
  if (J <= 0) return false;
  const ld l = logl(J);
  ld P[9];
  for (int q = 0; q < 9; q++) P[q] = mu * (F[q] - C[q] / J) + la * l * C[q] / J;
  for (int c = 0; c < 3; c++) {
    ld s0 = 0;
    for (int k = 0; k < 3; k++) {
      ld s = 0;
      for (int j = 0; j < 3; j++) s += P[3 * c + j] * (ld)X[3 * k + j];
      f[3 * (k + 1) + c] = -(ld)vol * s;
      s0 += f[3 * (k + 1) + c];
    }
    f[c] = -s0;
  }
  ld I1 = 0;
  for (int q = 0; q < 9; q++) I1 += F[q] * F[q];
  *psi = (ld)vol * (0.5L * mu * (I1 - 3) - mu * l + 0.5L * la * l * l);
  return true;
}

// the same forces with FP64 arithmetic (the FP64 element pass's formula), for scale
static void nh_f64(const double D[9], const double X[9], double vol, double mu, double la, double f[12], double* psi) {
  double F[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0;
      for (int k = 0; k < 3; k++) s += D[3 * i + k] * X[3 * k + j];
      F[3 * i + j] = s + (i == j ? 1 : 0);
    }
  const double C[9] = {F[4] * F[8] - F[5] * F[7], F[5] * F[6] - F[3] * F[8], F[3] * F[7] - F[4] * F[6],
                       F[2] * F[7] - F[1] * F[8], F[0] * F[8] - F[2] * F[6], F[1] * F[6] - F[0] * F[7],
                       F[1] * F[5] - F[2] * F[4], F[2] * F[3] - F[0] * F[5], F[0] * F[4] - F[1] * F[3]};
  const double J = F[0] * C[0] + F[1] * C[1] + F[2] * C[2];
  const double l = log(J);
  double P[9];
  for (int q = 0; q < 9; q++) P[q] = mu * (F[q] - C[q] / J) + la * l * C[q] / J;
  for (int c = 0; c < 3; c++) {
    double s0 = 0;
    for (int k = 0; k < 3; k++) {
      double s = 0;
      for (int j = 0; j < 3; j++) s += P[3 * c + j] * X[3 * k + j];
      f[3 * (k + 1) + c] = -vol * s;
      s0 += f[3 * (k + 1) + c];
    }
    f[c] = -s0;
  }
  double I1 = 0;
  for (int q = 0; q < 9; q++) I1 += F[q] * F[q];
  *psi = vol * (0.5 * mu * (I1 - 3) - mu * l + 0.5 * la * l * l);
}

int main() {
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> U(-1.0, 1.0);

  // 1. the FP64 split: |x - (hi + lo)| relative to |x|
  ld split_err = 0;
  for (int i = 0; i < 200000; i++) {
    const double x = U(rng) * pow(10.0, 25.0 * U(rng));
    const df s = sfem::df32::split_f64(x);
    const ld e = fabsl(val(s) - (ld)x) / fabsl((ld)x);
    if (e > split_err) split_err = e;
    if ((ld)fabsf(s.lo) > 0.5L * ldexpl(1.0L, ilogbf(s.hi) - 23)) split_err = 1;  // not normalised
  }
  printf("split_rel %.3e\n", (double)split_err);

  // 2. log1p over the series range and the FP64 fallback
  ld log_err = 0;
  for (int i = 0; i < 200000; i++) {
    const double x = (i % 2) ? 0.6 * U(rng) : 1e-3 * U(rng) * pow(10.0, -3.0 * fabs(U(rng)));
    const df xs = sfem::df32::split_f64(x);
    const ld r = log1pl(val(xs));
    const ld e = fabsl(val(sfem::df32::log1p_df(xs)) - r) / fabsl(r);
    if (e > log_err) log_err = e;
  }
  printf("log1p_rel %.3e\n", (double)log_err);

  // 3. neo-Hookean elements (nu = 0.49), strains from 1e-6 to 0.3: the largest force error relative to
  //    the element's largest force, and the energy's relative error, for the two-term and FP64 forms
  const double Eyoung = 1e5, nu = 0.49;
  const double mu = Eyoung / (2 * (1 + nu)), la = Eyoung * nu / ((1 + nu) * (1 - 2 * nu));
  ld fe_tt = 0, fe_64 = 0, pe_tt = 0, pe_64 = 0;
  int inverted_ok = 1;
  for (int i = 0; i < 100000; i++) {
    double X[9], D[9];
    const double h = pow(10.0, 2.0 * U(rng));  // element size 1e-2 .. 1e2
    for (int q = 0; q < 9; q++) X[q] = (q % 4 == 0 ? 1.0 : 0.0) / h + 0.3 * U(rng) / h;
    const double strain = pow(10.0, -6.0 + 5.5 * (0.5 + 0.5 * U(rng)));
    const double drift = 1e3 * h * U(rng);  // a large common displacement, removed by the differences
    for (int q = 0; q < 9; q++) {
      const double ua = drift + strain * h * U(rng), u0 = drift;
      D[q] = ua - u0;
    }
    const double vol = h * h * h / 6.0 * (1.0 + 0.2 * U(rng));
    ld fr[12], pr;
    if (!nh_ref(D, X, vol, mu, la, fr, &pr)) continue;
    df Dd[9], Xd[9], f[12], psi;
    for (int q = 0; q < 9; q++) Dd[q] = sfem::df32::split_f64(D[q]), Xd[q] = geo_split(X[q]);
    const bool inv = sfem::df32::nh_element(Dd, Xd, geo_split(vol), sfem::df32::split_f64(mu),
                                            sfem::df32::split_f64(la), true, f, &psi);
    if (inv) inverted_ok = 0;
    double f64[12], p64;
    nh_f64(D, X, vol, mu, la, f64, &p64);
    ld fmax = 0, et = 0, e6 = 0;
    for (int q = 0; q < 12; q++) {
      fmax = fmaxl(fmax, fabsl(fr[q]));
      et = fmaxl(et, fabsl(val(f[q]) - fr[q]));
      e6 = fmaxl(e6, fabsl((ld)f64[q] - fr[q]));
    }
    fe_tt = fmaxl(fe_tt, et / fmax);
    fe_64 = fmaxl(fe_64, e6 / fmax);
    pe_tt = fmaxl(pe_tt, fabsl(val(psi) - pr) / fabsl(pr));
    pe_64 = fmaxl(pe_64, fabsl((ld)p64 - pr) / fabsl(pr));
  }
  printf("force_rel_two_term %.3e\nforce_rel_fp64 %.3e\nenergy_rel_two_term %.3e\nenergy_rel_fp64 %.3e\n",
         (double)fe_tt, (double)fe_64, (double)pe_tt, (double)pe_64);

  // 4. node sums (the two-term gather): 24 element contributions that cancel to a small net force, added
  //    in order with the accurate two-term addition; error relative to the largest contribution, beside
  //    FP64 recursive summation of the same (FP64-rounded) contributions
  ld gs_tt = 0, gs_64 = 0;
  for (int i = 0; i < 100000; i++) {
    double v[24];
    double sum = 0;
    for (int k = 0; k < 23; k++) v[k] = U(rng) * pow(10.0, 2.0 * U(rng)), sum += v[k];
    v[23] = -sum + 1e-6 * U(rng);  // nearly in equilibrium
    df acc = {0.0f, 0.0f};
    double acc64 = 0;
    ld exact = 0, vmax = 0;
    for (int k = 0; k < 24; k++) {
      const df t = sfem::df32::split_f64(v[k]);
      acc = sfem::df32::df_add(acc, t);
      acc64 += v[k];
      exact += val(t);  // the two-term inputs exactly
      vmax = fmaxl(vmax, fabsl((ld)v[k]));
    }
    ld exact64 = 0;
    for (int k = 0; k < 24; k++) exact64 += (ld)v[k];
    gs_tt = fmaxl(gs_tt, fabsl(val(acc) - exact) / vmax);
    gs_64 = fmaxl(gs_64, fabsl((ld)acc64 - exact64) / vmax);
  }
  printf("node_sum_rel_two_term %.3e\nnode_sum_rel_fp64 %.3e\n", (double)gs_tt, (double)gs_64);

  // 5. an inverted element reports itself and gives non-finite forces
  {
    double X[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, D[9] = {-2, 0, 0, 0, 0, 0, 0, 0, 0};
    df Dd[9], Xd[9], f[12], psi;
    for (int q = 0; q < 9; q++) Dd[q] = sfem::df32::split_f64(D[q]), Xd[q] = geo_split(X[q]);
    const bool inv = sfem::df32::nh_element(Dd, Xd, geo_split(1.0 / 6), sfem::df32::split_f64(mu),
                                            sfem::df32::split_f64(la), true, f, &psi);
    printf("inverted_flag %d\nforces_nan %d\nvalid_not_flagged %d\n", inv ? 1 : 0, isnan(f[3].hi) ? 1 : 0,
           inverted_ok);
  }
  return 0;
}
