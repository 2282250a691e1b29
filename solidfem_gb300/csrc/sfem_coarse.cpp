// Coarse space of a two-level preconditioner for the Krylov inner solves, host side: the free
// nodes grouped into aggregates by the cells of a uniform grid, and the compact form of each
// aggregate's orthonormal rigid-body basis.  An extension: the reference's solver
// (SolveConjugateGradientMF, Math/IterativeSolvers.h:115-195) has no coarse space.
//
// Basis.  The rigid motions of an aggregate's nodes, three translations and three rotations about
// its centroid, are the columns of B (node i's 3 x 6 block B_i = [I, -[d_i]x], d_i the node's
// offset from the centroid).  The offsets sum to zero, so B^T B = diag(n I, J) with J the
// aggregate's inertia tensor sum(|d|^2 I - d d^T), and P = B R_a is orthonormal for
//   R_a = diag(I / sqrt(n), V L^-1/2),   J = V L V^T,
// keeping only rotations whose eigenvalue exceeds rtol times the largest (a single node keeps
// none, collinear nodes lose the rotation about their line); dropped columns of R_a are zero.
// Restriction and prolongation then need only d_i per node and R_a per aggregate:
//   P^T r = R_a^T (sum r_i, sum d_i x r_i),   (P y)_i = u_a + w_a x d_i,  (u_a, w_a) = R_a y_a.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "sfem.h"
#include "sfem_internal.h"

namespace {

// eigenpairs of a symmetric 3 x 3 matrix, A = V diag(w) V^T, by cyclic Jacobi rotations (each
// rotation zeroes one off-diagonal entry; the off-diagonal mass falls quadratically)
void symmetric_eigen3(double A[3][3], double w[3], double V[3][3]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) V[i][j] = i == j ? 1.0 : 0.0;
  const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int sweep = 0; sweep < 32; sweep++) {
    const double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
    const double dia = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
    if (off == 0.0 || off <= 1e-32 * dia) break;
    for (const auto& pq : pairs) {
      const int p = pq[0], q = pq[1];
      const double apq = A[p][q];
      if (apq == 0.0) continue;
      // tan of the rotation angle: the smaller root of t^2 + 2 theta t - 1 = 0
      const double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
      const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
      const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
      A[p][p] -= t * apq;
      A[q][q] += t * apq;
      A[p][q] = A[q][p] = 0.0;
      for (int k = 0; k < 3; k++) {
        if (k != p && k != q) {
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = A[p][k] = c * akp - s * akq;
          A[k][q] = A[q][k] = s * akp + c * akq;
        }
        const double vkp = V[k][p], vkq = V[k][q];
        V[k][p] = c * vkp - s * vkq;
        V[k][q] = s * vkp + c * vkq;
      }
    }
  }
  for (int i = 0; i < 3; i++) w[i] = A[i][i];
}

}  // namespace

extern "C" int sfem_coarse_factors(const double* X, int64_t n, double cell, double rtol, int32_t* aid, double* d,
                                   double* R, int64_t* n_agg) {
  if (!X || !aid || !d || !n_agg || n < 1 || n > INT32_MAX || !(cell > 0.0) || !std::isfinite(cell) ||
      !(rtol >= 0.0))
    return sfem::set_error(SFEM_ERR_INVALID, "sfem_coarse_factors: X, aid, d, n_agg, n >= 1, cell > 0, rtol >= 0");
  double lo[3] = {X[0], X[1], X[2]};
  for (int64_t i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) {
      if (!std::isfinite(X[3 * i + c])) return sfem::set_error(SFEM_ERR_INVALID, "sfem_coarse_factors: non-finite X");
      lo[c] = std::min(lo[c], X[3 * i + c]);
    }
  // grid cell of every node, numbered compactly in increasing key order
  std::vector<int64_t> g((size_t)3 * n);
  int64_t span[3] = {1, 1, 1};
  for (int64_t i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) {
      const double f = std::floor((X[3 * i + c] - lo[c]) / cell);
      if (!(f < 1e6)) return sfem::set_error(SFEM_ERR_INVALID, "sfem_coarse_factors: more than 1e6 cells per axis");
      g[3 * i + c] = (int64_t)f;
      span[c] = std::max(span[c], g[3 * i + c] + 1);
    }
  std::vector<int64_t> key((size_t)n);
  for (int64_t i = 0; i < n; i++) key[i] = (g[3 * i] * span[1] + g[3 * i + 1]) * span[2] + g[3 * i + 2];
  std::vector<int64_t> uniq(key);
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  const int64_t na = (int64_t)uniq.size();
  for (int64_t i = 0; i < n; i++) aid[i] = (int32_t)(std::lower_bound(uniq.begin(), uniq.end(), key[i]) - uniq.begin());
  *n_agg = na;

  // centroids and offsets (sums in node order)
  std::vector<double> cen((size_t)3 * na, 0.0), cnt((size_t)na, 0.0);
  for (int64_t i = 0; i < n; i++) {
    cnt[aid[i]] += 1.0;
    for (int c = 0; c < 3; c++) cen[3 * aid[i] + c] += X[3 * i + c];
  }
  for (int64_t a = 0; a < na; a++)
    for (int c = 0; c < 3; c++) cen[3 * a + c] /= cnt[a];
  for (int64_t i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) d[3 * i + c] = X[3 * i + c] - cen[3 * aid[i] + c];
  if (!R) return SFEM_OK;

  // inertia tensors, then R_a per aggregate (row-major 6 x 6)
  std::vector<double> J((size_t)9 * na, 0.0);
  for (int64_t i = 0; i < n; i++) {
    const double* di = d + 3 * i;
    const double dd = di[0] * di[0] + di[1] * di[1] + di[2] * di[2];
    double* Ja = J.data() + 9 * aid[i];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) Ja[3 * r + c] += (r == c ? dd : 0.0) - di[r] * di[c];
  }
  for (int64_t a = 0; a < na; a++) {
    double* Ra = R + 36 * a;
    std::fill(Ra, Ra + 36, 0.0);
    const double inv = 1.0 / std::sqrt(cnt[a]);
    for (int c = 0; c < 3; c++) Ra[6 * c + c] = inv;
    double A[3][3], w[3], V[3][3];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) A[r][c] = J[9 * a + 3 * r + c];
    symmetric_eigen3(A, w, V);
    int order[3] = {0, 1, 2};  // ascending eigenvalues
    std::sort(order, order + 3, [&](int x, int y) { return w[x] < w[y]; });
    const double wmax = std::max(w[order[2]], 0.0);
    int col = 3;
    for (int k : order) {
      if (!(w[k] > rtol * wmax)) continue;
      const double sc = 1.0 / std::sqrt(w[k]);
      for (int r = 0; r < 3; r++) Ra[6 * (3 + r) + col] = V[r][k] * sc;
      col++;
    }
  }
  return SFEM_OK;
}

// Polynomial modes: per aggregate and displacement component k, the F features of the node's offset
// (F = 4 for degree 1: 1, dx, dy, dz; F = 10 for degree 2: also dx^2, dy^2, dz^2, dx dy, dy dz, dz dx),
// column F k + m of B_i giving component k the feature f_m(d_i) (degree 1: the affine motions
// u = t + A d_i).  B^T B is block diagonal over the components with the features' Gram matrix
// G = sum f f^T in every block, so P = B R_a is orthonormal for R_a = I (x) V L^-1/2 from G's eigenpairs
// (L, V), eigenvalues <= max(rtol, 1e-3) times the largest dropped: column 3 j + k of R_a is component
// k of the j-th kept eigenvector (largest eigenvalue first), so the zero columns of dropped ones come
// last.  The floor drops nearly dependent modes (in an aggregate two node layers thick, the quadratic
// feature along the thin direction is almost a linear one): kept, they make W's entries large and
// cancelling, which its FP16 storage cannot carry (measured: 3,274 instead of ≈ 350 iterations).  The features are formed from d_i / h_a (h_a the aggregate's largest |d|) for the
// eigenproblem and the scaling is folded into R_a, which therefore acts on the unscaled features.
namespace {

// eigenpairs of a symmetric n x n matrix (n <= 10, row-major), A = V diag(w) V^T, by cyclic Jacobi
void symmetric_eigen(int n, double* A, double* w, double* V) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) V[n * i + j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 64; sweep++) {
    double off = 0.0, dia = 0.0;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) (i == j ? dia : off) += A[n * i + j] * A[n * i + j];
    if (off == 0.0 || off <= 1e-30 * dia) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = A[n * p + q];
        if (apq == 0.0) continue;
        const double theta = (A[n * q + q] - A[n * p + p]) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < n; k++) {  // columns p, q of A
          const double akp = A[n * k + p], akq = A[n * k + q];
          A[n * k + p] = c * akp - sn * akq;
          A[n * k + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {  // rows p, q
          const double apk = A[n * p + k], aqk = A[n * q + k];
          A[n * p + k] = c * apk - sn * aqk;
          A[n * q + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = V[n * k + p], vkq = V[n * k + q];
          V[n * k + p] = c * vkp - sn * vkq;
          V[n * k + q] = sn * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; i++) w[i] = A[n * i + i];
}

}  // namespace

// the F features of offset d (F = 4 or 10)
static inline void poly_features(const double* d, int F, double* f) {
  f[0] = 1.0;
  f[1] = d[0];
  f[2] = d[1];
  f[3] = d[2];
  if (F == 10) {
    f[4] = d[0] * d[0];
    f[5] = d[1] * d[1];
    f[6] = d[2] * d[2];
    f[7] = d[0] * d[1];
    f[8] = d[1] * d[2];
    f[9] = d[2] * d[0];
  }
}

constexpr double kPolyModeFloor = 1e-3;

extern "C" int sfem_coarse_factors_poly(const double* X, int64_t n, double cell, double rtol, int32_t degree,
                                        int32_t* aid, double* d, double* R, int64_t* n_agg) {
  if (degree != 1 && degree != 2) return sfem::set_error(SFEM_ERR_INVALID, "sfem_coarse_factors_poly: degree 1 or 2");
  const int st = sfem_coarse_factors(X, n, cell, rtol, aid, d, nullptr, n_agg);
  if (st != SFEM_OK || !R) return st;
  const int F = degree == 1 ? 4 : 10, nm = 3 * F;
  const int64_t na = *n_agg;
  std::vector<double> hs((size_t)na, 0.0);
  for (int64_t i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) hs[aid[i]] = std::max(hs[aid[i]], std::fabs(d[3 * i + c]));
  std::vector<double> G((size_t)F * F * na, 0.0);
  for (int64_t i = 0; i < n; i++) {
    const double h = hs[aid[i]] > 0.0 ? hs[aid[i]] : 1.0;
    const double e[3] = {d[3 * i] / h, d[3 * i + 1] / h, d[3 * i + 2] / h};
    double f[10];
    poly_features(e, F, f);
    double* Ga = G.data() + (size_t)F * F * aid[i];
    for (int r = 0; r < F; r++)
      for (int c = 0; c < F; c++) Ga[F * r + c] += f[r] * f[c];
  }
  for (int64_t a = 0; a < na; a++) {
    double* Ra = R + (size_t)nm * nm * a;
    std::fill(Ra, Ra + (size_t)nm * nm, 0.0);
    double A[100], w[10], V[100];
    std::copy(G.begin() + (size_t)F * F * a, G.begin() + (size_t)F * F * (a + 1), A);
    symmetric_eigen(F, A, w, V);
    int order[10];
    for (int k = 0; k < F; k++) order[k] = k;
    std::sort(order, order + F, [&](int x, int y) { return w[x] < w[y]; });
    const double wmax = std::max(w[order[F - 1]], 0.0), wtol = std::max(rtol, kPolyModeFloor) * wmax;
    // the scaling of feature m by h^-deg(m), folded into R (features act on the unscaled offsets)
    const double h = hs[a] > 0.0 ? hs[a] : 1.0;
    double fs[10];
    for (int m = 0; m < F; m++) fs[m] = m == 0 ? 1.0 : (m < 4 ? 1.0 / h : 1.0 / (h * h));
    int j = 0;
    for (int e = F - 1; e >= 0; e--) {  // the largest first, so that a dropped mode is always the last
      const int mm = order[e];
      if (!(w[mm] > wtol)) continue;
      const double sc = 1.0 / std::sqrt(w[mm]);
      for (int k = 0; k < 3; k++)
        for (int m = 0; m < F; m++) Ra[(size_t)nm * (F * k + m) + 3 * j + k] = V[F * m + mm] * sc * fs[m];
      j++;
    }
  }
  return SFEM_OK;
}
