// Test infrastructure only: a C-ABI harness around the reference SolidFEM
// matrix-free physics, compiled together with the reference's own unmodified
// hot-path translation units (see oracle/Makefile.ref).  It is used in the
// development container to generate golden fixtures and to pin the C
// restatement in oracle/sfem_oracle.c.  Nothing in the product links it.
//
// The harness adds only what the reference's matrix-free class lacks for the
// benchmark configurations:
//   * dead-load nodal forces added to the residual of
//     FemPhysicsMatrixFree::ComputeGradients (Source/FemPhysicsMatrixFree.cpp:536-560),
//   * a per-DOF Jacobi diagonal built from
//     ElasticEnergy::ComputeLocalStiffnessMatrixFromDifferential (Source/ElasticEnergy.cpp:493-517),
//   * a Newton loop with an Eigen sparse LU inner solve around
//     ElasticEnergy::AssembleStiffnessMatrix (Source/ElasticEnergy.cpp:573-635)
//     so that equilibria with dead loads can be computed directly,
//   * the orientation fix of FemBody::Prepare (Source/FemBody.cpp:127-156).
#include <stdio.h>
#include <stdint.h>
#include <vector>
#include <cmath>
#include <algorithm>

FILE* out = NULL;  // the reference's Printf sink (FEMLibrary.cpp:35)

#include "FemPhysicsMatrixFree.h"
#include "ElasticEnergy.h"
#include "LinearSolver.h"
#include "NewtonSolver.h"
#include <Eigen/SparseLU>
#include <Eigen/LU>

using namespace FEM_SYSTEM;

namespace {

struct RefProblem : public FemPhysicsMatrixFree {
  std::vector<Vector3R> fext;  // dead loads, reshuffled free-node order

  RefProblem(const std::vector<Tet>& t, const std::vector<Node>& n, const FemConfig& c)
      : FemPhysicsMatrixFree(t, n, c) {}

  void SetForceFraction(real f) { mForceFraction = f; }
  void SetSim(int type, int steps) { mSimType = (SimulationType)type; mNumSteps = steps; }
  void SetTimeStep(real h) { mTimeStep = h; }
  uint32 NumBCs() const { return mNumBCs; }
  const std::vector<uint32>& Map() const { return mReshuffleMap; }
  std::vector<Node>& Nodes() { return nodes; }

  void Gradients(std::vector<Vector3R>& r) {
    ComputeGradients(r);
    if (!fext.empty())
      for (size_t i = 0; i < r.size(); i++) r[i] += mForceFraction * fext[i];
  }
  void MatVec(const std::vector<Vector3R>& d, std::vector<Vector3R>& out) const {
    MatrixVectorMultiply(d, out);
  }
};

struct Handle {
  RefProblem* phys;
  FemPhysicsMatrixFree::Config cfg;
};

std::vector<Vector3R> ToVec(const double* p, size_t n) {
  std::vector<Vector3R> v(n);
  for (size_t i = 0; i < n; i++) v[i] = Vector3R(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
  return v;
}
void FromVec(const std::vector<Vector3R>& v, double* p) {
  for (size_t i = 0; i < v.size(); i++) {
    p[3 * i] = v[i].x; p[3 * i + 1] = v[i].y; p[3 * i + 2] = v[i].z;
  }
}

}  // namespace

extern "C" {

// material: MaterialModelType; solver: NonlinearSolverType.
void* ref_create(const double* nodes, int n_nodes, const int* tets, int n_tets,
                 const int* fixed, int n_fixed, double young, double poisson,
                 double density, double gravity, int zup, int material, int solver,
                 int outer_iters, int inner_iters, double abs_tol) {
  std::vector<Node> nn(n_nodes);
  for (int i = 0; i < n_nodes; i++) {
    nn[i].pos = Vector3R(nodes[3 * i], nodes[3 * i + 1], nodes[3 * i + 2]);
    nn[i].pos0 = nn[i].pos;
  }
  std::vector<Tet> tt(n_tets);
  for (int e = 0; e < n_tets; e++) {
    for (int j = 0; j < 4; j++) tt[e].idx[j] = (uint32)tets[4 * e + j];
    // FemBody::Prepare: positive orientation by swapping the first two indices
    Vector3R x0 = nn[tt[e].idx[0]].pos0;
    Matrix3R m(nn[tt[e].idx[1]].pos0 - x0, nn[tt[e].idx[2]].pos0 - x0, nn[tt[e].idx[3]].pos0 - x0);
    if (m.Determinant() / 6.f < 0) std::swap(tt[e].idx[0], tt[e].idx[1]);
  }
  for (int i = 0; i < n_fixed; i++) nn[fixed[i]].invMass = 0;

  Handle* h = new Handle;
  h->cfg.mSolver = (NonlinearSolverType)solver;
  FemConfig c;
  c.mYoungsModulus = young;
  c.mPoissonRatio = poisson;
  c.mDensity = density;
  c.mGravity = gravity;
  c.mZUpAxis = zup != 0;
  c.mMaterial = (MaterialModelType)material;
  c.mSimType = ST_STATIC;
  c.mOuterIterations = outer_iters;
  c.mInnerIterations = inner_iters;
  c.mAbsNewtonRsidualThreshold = abs_tol;
  c.mVerbose = false;
  c.mCustomConfig = &h->cfg;
  h->phys = new RefProblem(tt, nn, c);
  return h;
}

void ref_destroy(void* hp) {
  Handle* h = (Handle*)hp;
  delete h->phys;
  delete h;
}

int ref_num_bcs(void* hp) { return (int)((Handle*)hp)->phys->NumBCs(); }
int ref_num_free(void* hp) { return (int)((Handle*)hp)->phys->GetNumFreeNodes(); }

void ref_reshuffle_map(void* hp, int* out_map) {
  const auto& m = ((Handle*)hp)->phys->Map();
  for (size_t i = 0; i < m.size(); i++) out_map[i] = (int)m[i];
}

// Element connectivity after the orientation fix, in reshuffled node indices.
void ref_tets(void* hp, int* out_tets) {
  RefProblem* p = ((Handle*)hp)->phys;
  for (uint32 e = 0; e < p->GetNumElements(); e++)
    for (int j = 0; j < 4; j++) out_tets[4 * e + j] = (int)p->GetGlobalIndex(e, j);
}

void ref_set_force_fraction(void* hp, double f) { ((Handle*)hp)->phys->SetForceFraction(f); }

// FemPhysicsMatrixFree::SetBoundaryConditionsSurface: triangles of original node indices
void ref_set_pressure_surface(void* hp, const int* tris, int n_tris, double pressure) {
  std::vector<uint32> tl(3 * (size_t)n_tris);
  for (size_t i = 0; i < tl.size(); i++) tl[i] = (uint32)tris[i];
  ((Handle*)hp)->phys->SetBoundaryConditionsSurface(tl, pressure);
}

// Dead loads given per original node index (only free nodes are used).
void ref_set_nodal_loads(void* hp, const double* f_orig) {
  RefProblem* p = ((Handle*)hp)->phys;
  uint32 nbc = p->NumBCs();
  p->fext.assign(p->GetNumFreeNodes(), Vector3R());
  const auto& m = p->Map();
  for (size_t i = 0; i < m.size(); i++) {
    if (m[i] >= nbc) p->fext[m[i] - nbc] = Vector3R(f_orig[3 * i], f_orig[3 * i + 1], f_orig[3 * i + 2]);
  }
}

// Positions of all nodes in reshuffled order (N x 3).
void ref_set_positions_shuffled(void* hp, const double* pos) {
  RefProblem* p = ((Handle*)hp)->phys;
  for (uint32 i = 0; i < p->GetNumNodes(); i++)
    p->Nodes()[i].pos = Vector3R(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
}
void ref_get_positions_shuffled(void* hp, double* pos) {
  RefProblem* p = ((Handle*)hp)->phys;
  for (uint32 i = 0; i < p->GetNumNodes(); i++) {
    const Vector3R& x = p->Nodes()[i].pos;
    pos[3 * i] = x.x; pos[3 * i + 1] = x.y; pos[3 * i + 2] = x.z;
  }
}
// Positions in original node order (what pysolidfem's get_nodes returns).
void ref_get_positions(void* hp, double* pos) {
  RefProblem* p = ((Handle*)hp)->phys;
  for (uint32 i = 0; i < p->GetNumNodes(); i++) {
    Vector3R x = p->GetDeformedPosition(i);
    pos[3 * i] = x.x; pos[3 * i + 1] = x.y; pos[3 * i + 2] = x.z;
  }
}

void ref_compute_gradients(void* hp, double* r) {
  RefProblem* p = ((Handle*)hp)->phys;
  std::vector<Vector3R> v(p->GetNumFreeNodes());
  p->Gradients(v);
  FromVec(v, r);
}

void ref_matvec(void* hp, const double* d, double* outp) {
  RefProblem* p = ((Handle*)hp)->phys;
  std::vector<Vector3R> dv = ToVec(d, p->GetNumFreeNodes());
  std::vector<Vector3R> ov(p->GetNumFreeNodes());
  p->MatVec(dv, ov);
  FromVec(ov, outp);
}

// Per-DOF diagonal of the tangent stiffness over free DOFs (3 N_f).
void ref_jacobi_diagonal(void* hp, double* diag) {
  RefProblem* p = ((Handle*)hp)->phys;
  p->ComputeDeformationGradients();
  uint32 nbc = p->NumBCs();
  std::fill(diag, diag + 3 * p->GetNumFreeNodes(), 0.0);
  for (uint32 e = 0; e < p->GetNumElements(); e++) {
    EigenMatrix K;
    ElasticEnergy::ComputeLocalStiffnessMatrixFromDifferential(p, e, K);
    for (int j = 0; j < 4; j++) {
      uint32 g = p->GetGlobalIndex(e, j);
      if (g < nbc) continue;
      for (int c = 0; c < 3; c++) diag[3 * (g - nbc) + c] += K(3 * j + c, 3 * j + c);
    }
  }
}

// PK1 stress of every element at the current positions (E x 9, row-major).
void ref_element_stress(void* hp, double* P) {
  RefProblem* p = ((Handle*)hp)->phys;
  p->ComputeDeformationGradients();
  for (uint32 e = 0; e < p->GetNumElements(); e++) {
    Matrix3R Pmu, Pl;
    Matrix3R S = ElasticEnergy::ComputeElementStress(p, e, Pmu, Pl, true);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) P[9 * e + 3 * i + j] = S.m[i][j];
  }
}

double ref_elastic_energy(void* hp) { return ((Handle*)hp)->phys->ComputeElasticEnergy(); }

// Free-DOF force parameter gradients (FemPhysicsBase::GetForceParamGrads).
void ref_force_param_grads(void* hp, double* gmu, double* glambda, double* grho) {
  RefProblem* p = ((Handle*)hp)->phys;
  p->ComputeDeformationGradients();
  EigenVector a, b, c;
  p->GetForceParamGrads(a, b, c);
  for (int i = 0; i < a.size(); i++) { gmu[i] = a(i); glambda[i] = b(i); grho[i] = c(i); }
}

// The reference's own static solve: Step(0) dispatching on the configured solver.
void ref_step(void* hp) { ((Handle*)hp)->phys->Step(0); }

// The reference's assembled tangent (ElasticEnergy::AssembleStiffnessMatrix,
// Source/ElasticEnergy.cpp:573-635) at the current positions, dense row-major
// 3 N_f x 3 N_f (small meshes only).
void ref_assemble_dense(void* hp, double* out) {
  RefProblem* p = ((Handle*)hp)->phys;
  p->ComputeDeformationGradients();
  SparseMatrix K;
  ElasticEnergy::AssembleStiffnessMatrix(p, K);
  const int n = (int)K.rows();
  EigenMatrix D(K);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) out[(size_t)i * n + j] = D(i, j);
}

// Dynamics: simulation type / substeps (FemPhysicsBase mSimType, mNumSteps), the time step
// of the implicit terms (mTimeStep), node velocities and step-start positions (pos0), in
// reshuffled order, and the reference's own Step(dt).
void ref_set_sim(void* hp, int type, int steps) { ((Handle*)hp)->phys->SetSim(type, steps); }
void ref_set_time_step(void* hp, double h) { ((Handle*)hp)->phys->SetTimeStep(h); }
void ref_set_velocities_shuffled(void* hp, const double* v) {
  RefProblem* p = ((Handle*)hp)->phys;
  for (uint32 i = 0; i < p->GetNumNodes(); i++) p->Nodes()[i].vel = Vector3R(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
}
void ref_get_velocities_shuffled(void* hp, double* v) {
  RefProblem* p = ((Handle*)hp)->phys;
  for (uint32 i = 0; i < p->GetNumNodes(); i++) {
    const Vector3R& a = p->Nodes()[i].vel;
    v[3 * i] = a.x; v[3 * i + 1] = a.y; v[3 * i + 2] = a.z;
  }
}
void ref_set_start_shuffled(void* hp, const double* x) {
  RefProblem* p = ((Handle*)hp)->phys;
  for (uint32 i = 0; i < p->GetNumNodes(); i++) p->Nodes()[i].pos0 = Vector3R(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
}
void ref_step_dt(void* hp, double dt) { ((Handle*)hp)->phys->Step(dt); }

// Harness Newton with a direct sparse LU inner solve over the assembled
// reference tangent; includes dead loads.  Residual-norm backtracking.
// Returns the number of Newton iterations; *res_out = final |r|.
int ref_newton_direct(void* hp, int max_iters, double rel_tol, double* res_out) {
  RefProblem* p = ((Handle*)hp)->phys;
  p->SetForceFraction(1);
  uint32 nf = p->GetNumFreeNodes(), nbc = p->NumBCs();
  std::vector<Vector3R> r(nf), r2(nf);
  p->Gradients(r);
  auto norm = [](const std::vector<Vector3R>& v) {
    double s = 0; for (auto& a : v) s += a.x * a.x + a.y * a.y + a.z * a.z; return std::sqrt(s);
  };
  double r0 = norm(r), rn = r0;
  int it = 0;
  for (; it < max_iters && rn > rel_tol * r0; it++) {
    p->ComputeDeformationGradients();
    SparseMatrix K;
    ElasticEnergy::AssembleStiffnessMatrix(p, K);
    Eigen::SparseLU<SparseMatrix> lu;
    lu.compute(K);
    EigenVector rhs(3 * nf);
    for (uint32 i = 0; i < nf; i++) { rhs(3 * i) = r[i].x; rhs(3 * i + 1) = r[i].y; rhs(3 * i + 2) = r[i].z; }
    EigenVector d = lu.solve(rhs);
    std::vector<Vector3R> x0(nf);
    for (uint32 i = 0; i < nf; i++) x0[i] = p->Nodes()[i + nbc].pos;
    double alpha = 1;
    for (int ls = 0; ls < 30; ls++) {
      for (uint32 i = 0; i < nf; i++)
        p->Nodes()[i + nbc].pos = x0[i] + alpha * Vector3R(d(3 * i), d(3 * i + 1), d(3 * i + 2));
      p->Gradients(r2);
      double n2 = norm(r2);
      if (std::isfinite(n2) && !p->CheckForInversion(0) && n2 < (1 - 1e-4 * alpha) * rn) { rn = n2; break; }
      alpha *= 0.5;
    }
    r = r2;
  }
  *res_out = rn;
  return it;
}

// Harness Newton with the finite-difference Jacobian of the reference residual
// (NewtonSolver::ComputeJacobianFD, Include/NewtonSolver.h:95-111: forward
// differences, eps = 1e-5) and a dense LU solve; includes dead loads.  For small
// meshes only.  Used where the reference's analytic tangent is inconsistent
// with its force (corotational).  Residual-norm backtracking as above.
int ref_newton_fd(void* hp, int max_iters, double rel_tol, double* res_out) {
  RefProblem* p = ((Handle*)hp)->phys;
  p->SetForceFraction(1);
  uint32 nf = p->GetNumFreeNodes(), nbc = p->NumBCs();
  const int n = 3 * nf;
  std::vector<Vector3R> r(nf), r2(nf);
  auto norm = [](const std::vector<Vector3R>& v) {
    double s = 0; for (auto& a : v) s += a.x * a.x + a.y * a.y + a.z * a.z; return std::sqrt(s);
  };
  auto getx = [&](int k) -> double& { Vector3R& x = p->Nodes()[k / 3 + nbc].pos; return k % 3 == 0 ? x.x : (k % 3 == 1 ? x.y : x.z); };
  p->Gradients(r);
  double r0 = norm(r), rn = r0;
  int it = 0;
  const double eps = 1e-5;
  for (; it < max_iters && rn > rel_tol * r0; it++) {
    EigenMatrix K(n, n);
    for (int j = 0; j < n; j++) {
      double keep = getx(j);
      getx(j) = keep + eps;
      p->Gradients(r2);
      getx(j) = keep;
      for (uint32 i = 0; i < nf; i++) {
        K(3 * i, j) = -(r2[i].x - r[i].x) / eps;
        K(3 * i + 1, j) = -(r2[i].y - r[i].y) / eps;
        K(3 * i + 2, j) = -(r2[i].z - r[i].z) / eps;
      }
    }
    EigenVector rhs(n);
    for (uint32 i = 0; i < nf; i++) { rhs(3 * i) = r[i].x; rhs(3 * i + 1) = r[i].y; rhs(3 * i + 2) = r[i].z; }
    EigenVector d = K.partialPivLu().solve(rhs);
    std::vector<Vector3R> x0(nf);
    for (uint32 i = 0; i < nf; i++) x0[i] = p->Nodes()[i + nbc].pos;
    double alpha = 1;
    bool ok = false;
    for (int ls = 0; ls < 30; ls++) {
      for (uint32 i = 0; i < nf; i++)
        p->Nodes()[i + nbc].pos = x0[i] + alpha * Vector3R(d(3 * i), d(3 * i + 1), d(3 * i + 2));
      p->Gradients(r2);
      double n2 = norm(r2);
      if (std::isfinite(n2) && !p->CheckForInversion(0) && n2 < (1 - 1e-4 * alpha) * rn) { rn = n2; ok = true; break; }
      alpha *= 0.5;
    }
    if (!ok) { for (uint32 i = 0; i < nf; i++) p->Nodes()[i + nbc].pos = x0[i]; p->Gradients(r); break; }
    r = r2;
  }
  *res_out = rn;
  return it;
}

// The reference's own NewtonSolverBackTrack (Include/NewtonSolver.h:179-348) with the default
// Bonet-Wood condition, exactly as FemPhysicsMatrixFree::SolveNewtonLS sets it up
// (Source/FemPhysicsMatrixFree.cpp:733-781, static case), over a problem that forwards every
// callback to the reference class and records each line-search trial: the Newton iteration it
// belongs to, its step length relative to the Newton direction, and the norm of its residual.
namespace {
struct TraceProblem {
  RefProblem* p;
  std::vector<int> it;
  std::vector<double> step, res;
  EigenVector base, delta, last;
  int iter = -1;
  double res0 = 0;
  EigenVector ComputeRhs(const EigenVector& sol) {
    EigenVector r = p->ComputeRhs(sol);
    if (iter < 0) {
      res0 = r.norm();
    } else {
      it.push_back(iter);
      step.push_back((sol - base).dot(delta) / delta.squaredNorm());
      res.push_back(r.norm());
    }
    last = sol;
    return r;
  }
  // FemPhysicsMatrixFree::ComputeSystemMatrix (:696-715) for a static problem without Dirichlet
  // penalties or cables: the assembled tangent at the state of the last ComputeRhs
  void ComputeSystemMatrix(const EigenVector&, const EigenVector&, SparseMatrix& K) {
    ElasticEnergy::AssembleStiffnessMatrix(p, K);
  }
  EigenVector SolveLinearSystem(SparseMatrix& K, const EigenVector& rhs, const EigenVector& s, const EigenVector& y) {
    EigenVector d = p->SolveLinearSystem(K, rhs, s, y);
    iter++;
    base = last;
    delta = d;
    return d;
  }
  real MeritResidual(const EigenVector& rhs) { return p->MeritResidual(rhs); }
};
}  // namespace

// Returns the number of recorded trials (at most cap); it/step/res per trial, *res0 the initial
// residual norm, *converged the solver's result.  Positions are left at the solver's solution.
int ref_newton_ls_trace(void* hp, int max_iters, double abs_tol, int* it, double* step, double* res, int cap,
                        double* res0, int* converged) {
  RefProblem* p = ((Handle*)hp)->phys;
  p->SetForceFraction(1);
  TraceProblem tp;
  tp.p = p;
  NewtonSolverBackTrack<TraceProblem, SparseMatrix> solver;
  solver.mNumIterations = max_iters;
  solver.mVerbose = VL_NONE;
  solver.mResidualThreshold = abs_tol;
  solver.mUseProblemSolver = true;
  const uint32 nf = p->GetNumFreeNodes(), nbc = p->NumBCs();
  EigenVector solution(3 * nf);
  for (uint32 i = 0; i < nf; i++) {
    const Vector3R& x = p->Nodes()[i + nbc].pos;
    solution(3 * i) = x.x; solution(3 * i + 1) = x.y; solution(3 * i + 2) = x.z;
  }
  *converged = solver.Solve(tp, 3 * nf, solution) ? 1 : 0;
  for (uint32 i = 0; i < nf; i++)
    p->Nodes()[i + nbc].pos = Vector3R(solution(3 * i), solution(3 * i + 1), solution(3 * i + 2));
  *res0 = tp.res0;
  const int n = std::min<int>(cap, (int)tp.it.size());
  for (int k = 0; k < n; k++) {
    it[k] = tp.it[k];
    step[k] = tp.step[k];
    res[k] = tp.res[k];
  }
  return n;
}

}  // extern "C"
