// Internal declarations shared by the host driver (sfem_host.cpp) and the
// CUDA kernels (sfem_kernels.cu).  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sfem {

enum Mode {
  MODE_FORCE = 0,    // element internal forces (12 per element)
  MODE_HVP = 1,      // element force differential of a direction p
  MODE_DIAG = 2,     // diagonal of the element tangent (12 per element)
  MODE_ENERGY = 3,   // sum of V * Psi(F)
  MODE_STRESS = 4,   // PK1 stress (9 per element, 12-stride)
  MODE_PMU = 5,      // forces of the mu-part of the neo-Hookean stress
  MODE_PLAMBDA = 6,  // forces of the lambda-part
  MODE_NODALVOL = 7  // V/4 per element corner
};

// Element arrays on the device, structure-of-arrays.
//   tets:  E int4 of reshuffled node indices
//   X:     9 x E, X[k * E + e] = (Dm^-1)_{k/3, k%3} of element e
//   vol:   E signed rest volumes
//   scale: E per-element stiffness scales (E_e / E) or nullptr
template <typename T>
struct ElemView {
  const int4* tets;
  const T* X;
  const T* vol;
  const T* scale;
  int64_t E;
  T mu, lambda;
};

// Node-to-element CSR: for node g, entries ent[ptr[g] .. ptr[g+1]) hold
// (element << 2 | local slot), sorted by element, so every gather sums the
// element contributions in element order (deterministic, no atomics).
struct NodeCsr {
  const int64_t* ptr;  // N + 1
  const int64_t* ent;  // 4 E
};

// Scalars of one Krylov solve, resident on the device so that the iteration
// runs without host round trips.  All reductions finish in the last block of
// the producing kernel, in a fixed order (deterministic).
struct CgScalars {
  double rz;     // r . z
  double pq;     // p . A p
  double alpha;  // rz / pq
  double beta;
  double rr;     // r . r
  double bb;     // b . b
  double tol2;   // (rel_tol)^2 * bb
  int32_t it;
  int32_t max_it;
  int32_t done;
  int32_t status;  // 0 ok, 1 max iters, 2 negative curvature, -3 nan
};

struct Reduce {
  double* partials;   // >= kMaxBlocks * 4 doubles
  unsigned* counter;  // zero-initialised
};

unsigned long long launch_count();

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 2048;

// ---- element passes ----
template <typename T, int MAT>
void launch_element(int mode, const ElemView<T>& ev, const T* u, const T* p, T* fe, Reduce red,
                    double* result, int* n_inverted, const CgScalars* s, cudaStream_t st);

// ---- node gathers (FP64 residual / T HVP / T diagonal) ----
void launch_gather_force(int64_t nbc, int64_t N, NodeCsr csr, const double* fe, const double* mass,
                         const double* fext, const double* grav, double ff, double* r, Reduce red,
                         double* rr_out, cudaStream_t st);
template <typename T>
void launch_gather_hvp(int64_t nbc, int64_t N, NodeCsr csr, const T* fe, const T* p, T* q, Reduce red,
                       CgScalars* s, cudaStream_t st);
template <typename T>
void launch_gather_diag(int64_t nbc, int64_t N, NodeCsr csr, const T* fe, T* dinv, T* diag,
                        cudaStream_t st);
// per-element forces of the FP64 force pass in element-major 12-vectors are
// reused by the adjoint: g_e = sum_a lam_a . f_a / E_e
void launch_adjoint_elem(const int4* tets, int64_t E, int64_t nbc, const double* fe, const double* lam,
                         const double* young_e, double* dLdE, cudaStream_t st);

// ---- Krylov vector kernels (T = float or double) ----
template <typename T>
void launch_cg_init(int64_t n, const T* b, T* x, T* r, T* p, const T* dinv, Reduce red, CgScalars* s,
                    cudaStream_t st);
template <typename T>
void launch_cg_update(int64_t n, T* x, T* r, const T* p, const T* q, const T* dinv, Reduce red,
                      CgScalars* s, cudaStream_t st);
template <typename T>
void launch_cg_direction(int64_t n, const T* r, const T* dinv, T* p, const CgScalars* s, cudaStream_t st);

// ---- misc vector kernels ----
void launch_dot(int64_t n, const double* a, const double* b, Reduce red, double* out, cudaStream_t st);
void launch_potential(int64_t nbc, int64_t N, const double* x0, const double* u, const double* mass,
                      const double* fext, const double* grav, double ff, Reduce red, double* out,
                      cudaStream_t st);
template <typename Tin, typename Tout>
void launch_convert(int64_t n, const Tin* a, Tout* b, cudaStream_t st);
// x = x + a * d   (FP64 state += precision-T direction)
template <typename T>
void launch_axpy_state(int64_t n, double a, const T* d, const double* base, double* x, cudaStream_t st);
void launch_scale_copy(int64_t n, double a, const double* x, double* y, cudaStream_t st);

}  // namespace sfem
