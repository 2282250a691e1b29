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

// Affine modes (twelve per aggregate): u_i = t + A d_i, columns B_i = [I, L(d_i)] with L's column
// 3 + 3 k + l giving component k the coordinate d_i[l].  B^T B = diag(n I, S (x) I) blockwise per
// component, S = sum d d^T, so P = B R_a is orthonormal for the translations scaled by 1 / sqrt(n) and,
// per kept eigenpair (lambda_m, v_m) of S (ascending; lambda_m > rtol times the largest) and component
// k, the column 3 + 3 j + k (j: the pair's rank among the kept ones) with entries v_m[l] / sqrt(lambda_m)
// in rows 3 + 3 k + l.  R: 144 doubles per aggregate, row-major 12 x 12, dropped columns zero.
extern "C" int sfem_coarse_factors_affine(const double* X, int64_t n, double cell, double rtol, int32_t* aid,
                                          double* d, double* R, int64_t* n_agg) {
  const int st = sfem_coarse_factors(X, n, cell, rtol, aid, d, nullptr, n_agg);
  if (st != SFEM_OK || !R) return st;
  const int64_t na = *n_agg;
  std::vector<double> S((size_t)9 * na, 0.0), cnt((size_t)na, 0.0);
  for (int64_t i = 0; i < n; i++) {
    const double* di = d + 3 * i;
    double* Sa = S.data() + 9 * aid[i];
    cnt[aid[i]] += 1.0;
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) Sa[3 * r + c] += di[r] * di[c];
  }
  for (int64_t a = 0; a < na; a++) {
    double* Ra = R + 144 * a;
    std::fill(Ra, Ra + 144, 0.0);
    const double inv = 1.0 / std::sqrt(cnt[a]);
    for (int c = 0; c < 3; c++) Ra[12 * c + c] = inv;
    double A[3][3], w[3], V[3][3];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) A[r][c] = S[9 * a + 3 * r + c];
    symmetric_eigen3(A, w, V);
    int order[3] = {0, 1, 2};
    std::sort(order, order + 3, [&](int x, int y) { return w[x] < w[y]; });
    const double wmax = std::max(w[order[2]], 0.0);
    int j = 0;
    for (int m : order) {
      if (!(w[m] > rtol * wmax)) continue;
      const double sc = 1.0 / std::sqrt(w[m]);
      for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) Ra[12 * (3 + 3 * k + l) + 3 + 3 * j + k] = V[l][m] * sc;
      j++;
    }
  }
  return SFEM_OK;
}
