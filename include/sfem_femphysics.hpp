// C++ drop-in for SolidFEM's FemPhysicsMatrixFree on the GB300 library (libsfem_gb300.so).
//
// The reference's solvers are duck-typed templates over the physics class:
//   SolveConjugateGradientMF<Real, Vector, MatrixMultiplier>   (Math/IterativeSolvers.h:115-195)
//   NonlinearConjugateGradientMinimizer<PROBLEM, VECTOR>       (Include/NonlinearCG.h:38-114)
// FemPhysicsMatrixFreeGpu has the members they call, with the signatures of
// FemPhysicsMatrixFree (Include/FemPhysicsMatrixFree.h:61-90), so those templates run on the GPU
// unchanged.  Free-DOF vectors are std::vector<Vector3R> in the reference's reshuffled order (fixed
// nodes first removed, ReshuffleFixedNodes, Source/FemPhysicsMatrixFree.cpp:229-263); a Vector3R is
// three contiguous doubles, so &v[0].x is the 3 N_f array the C ABI takes.
//
// Add this header to SolidFEM's Include/ directory (it includes the reference's FemDataStructures.h)
// and link libsfem_gb300.so.  Errors of the C ABI are thrown as sfem_gpu_error with the ABI's status.
#pragma once

#include <stdint.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "FemDataStructures.h"
#include "sfem.h"

namespace FEM_SYSTEM {

class sfem_gpu_error : public std::runtime_error {
 public:
  sfem_gpu_error(int code, const char* msg) : std::runtime_error(msg ? msg : ""), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

class FemPhysicsMatrixFreeGpu {
 public:
  // FemPhysicsMatrixFree(const std::vector<Tet>&, const std::vector<Node>&, const FemConfig&)
  // (Include/FemPhysicsMatrixFree.h:61-62): fixed nodes are the ones with invMass == 0, as
  // FemBody::Prepare marks them; precision SFEM_FP64 or SFEM_FP32 (FP64 Newton residual either way).
  FemPhysicsMatrixFreeGpu(const std::vector<Tet>& tets, const std::vector<Node>& nodes, const FemConfig& cfg,
                          int32_t precision = SFEM_FP64, int32_t device = 0) {
    std::vector<double> x(3 * nodes.size());
    std::vector<int32_t> fixed, t(4 * tets.size());
    for (size_t i = 0; i < nodes.size(); i++) {
      x[3 * i] = nodes[i].pos.x;
      x[3 * i + 1] = nodes[i].pos.y;
      x[3 * i + 2] = nodes[i].pos.z;
      if (nodes[i].invMass == 0) fixed.push_back((int32_t)i);
    }
    for (size_t e = 0; e < tets.size(); e++)
      for (int j = 0; j < 4; j++) t[4 * e + j] = (int32_t)tets[e].idx[j];
    sfem_config c{};
    c.young = cfg.mYoungsModulus;
    c.poisson = cfg.mPoissonRatio;
    c.density = cfg.mDensity;
    c.gravity[cfg.mZUpAxis ? 2 : 1] = cfg.mGravity;
    c.material = (int32_t)cfg.mMaterial;
    c.precision = precision;
    c.device = device;
    c.tangent = SFEM_TANGENT_REFERENCE;
    check(sfem_create(x.data(), (int64_t)nodes.size(), t.data(), (int64_t)tets.size(),
                      fixed.empty() ? nullptr : fixed.data(), (int64_t)fixed.size(), &c, &h_));
    int64_t n = 0, nf = 0, ne = 0;
    check(sfem_sizes(h_, &n, &nf, &ne));
    n_ = (size_t)n;
    nf_ = (size_t)nf;
    ne_ = (size_t)ne;
    outer_ = cfg.mOuterIterations;
    abs_tol_ = cfg.mAbsNewtonRsidualThreshold;
  }
  ~FemPhysicsMatrixFreeGpu() {
    if (h_) sfem_destroy(h_);
  }
  FemPhysicsMatrixFreeGpu(const FemPhysicsMatrixFreeGpu&) = delete;
  FemPhysicsMatrixFreeGpu& operator=(const FemPhysicsMatrixFreeGpu&) = delete;

  // sizes (Include/FemPhysicsMatrixFree.h:74-77)
  uint32 GetNumNodes() const { return (uint32)n_; }
  uint32 GetNumFreeNodes() const { return (uint32)nf_; }
  uint32 GetNumElements() const { return (uint32)ne_; }

  // FemPhysicsMatrixFree::ComputeGradients (Source/FemPhysicsMatrixFree.cpp:536-560)
  void ComputeGradients(std::vector<Vector3R>& r) {
    r.resize(nf_);
    check(sfem_compute_gradients(h_, data(r), nullptr));
  }
  // FemPhysicsMatrixFree::MatrixVectorMultiply (:523-534); const like the reference's (the device
  // handle is not part of the object's logical state)
  void MatrixVectorMultiply(const std::vector<Vector3R>& d, std::vector<Vector3R>& out) const {
    out.resize(nf_);
    check(sfem_matvec(h_, data(d), data(out)));
  }
  // FemPhysicsMatrixFree::DotProduct (Include/FemPhysicsMatrixFree.h:89)
  real DotProduct(const std::vector<Vector3R>& a, const std::vector<Vector3R>& b) const {
    double s = 0;
    check(sfem_dot(h_, data(a), data(b), &s));
    return s;
  }
  // FemPhysicsMatrixFree::UpdatePosAndComputeGradients (:562-568)
  void UpdatePosAndComputeGradients(const std::vector<Vector3R>& pos, std::vector<Vector3R>& r) {
    check(sfem_set_free_positions(h_, data(pos)));
    ComputeGradients(r);
  }
  // FemPhysicsBase::CheckForInversion (Source/FemPhysicsBase.cpp:93-117)
  bool CheckForInversion() const {
    int64_t k = 0;
    check(sfem_count_inverted(h_, &k));
    return k > 0;
  }
  // Step(0) of ST_STATIC (Source/FemPhysicsMatrixFree.cpp:297-340): the whole static solve on the
  // device (inexact Newton with Jacobi-PCG inner solves), to the configuration's absolute residual
  // threshold or a relative 1e-10, at most mOuterIterations Newton steps
  void Step(real /*dt*/ = 0) {
    sfem_newton_opts o{};
    o.rel_tol = 1e-10;
    o.abs_tol = abs_tol_;
    o.max_newton = (int32_t)(outer_ > 0 ? outer_ : 50);
    o.precond = SFEM_PC_JACOBI;
    o.ls_condition = SFEM_LSC_ARMIJO;
    sfem_newton_stats st{};
    check(sfem_newton_solve(h_, &o, &st));
  }
  // node positions in the caller's order (FemPhysicsMatrixFree::GetDeformedPosition per node)
  std::vector<Vector3R> GetPositions() const {
    std::vector<Vector3R> p(n_);
    check(sfem_get_positions(h_, data(p)));
    return p;
  }

  sfem_handle* handle() const { return h_; }

 private:
  static void check(int s) {
    if (s < 0) throw sfem_gpu_error(s, sfem_last_error());
  }
  static double* data(std::vector<Vector3R>& v) { return v.empty() ? nullptr : &v[0].x; }
  static const double* data(const std::vector<Vector3R>& v) { return v.empty() ? nullptr : &v[0].x; }

  sfem_handle* h_ = nullptr;
  size_t n_ = 0, nf_ = 0, ne_ = 0;
  uint32 outer_ = 0;
  real abs_tol_ = 0;
};

}  // namespace FEM_SYSTEM
