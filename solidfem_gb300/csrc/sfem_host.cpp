// Host side of the C ABI (include/sfem.h): problem set-up, device memory, and
// the Krylov / Newton / nonlinear-CG drivers.  All arithmetic on problem data
// runs in the CUDA kernels of sfem_kernels.cu; the host only sequences launches
// and reads back a handful of scalars.
//
// Set-up mirrors FemPhysicsMatrixFree's constructor (Source/FemPhysicsMatrixFree.cpp:71-213):
// orientation fix (FemBody::Prepare, Source/FemBody.cpp:127-156), fixed nodes
// first (ReshuffleFixedNodes :229-263), Dm^-1 / signed volume / lumped masses
// per element in FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <type_traits>
#include <cmath>
#include <random>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "sfem.h"
#include "sfem_internal.h"

using namespace sfem;

namespace {

// internal status of pcg_device: CG stopped on non-positive curvature (truncated CG)
constexpr int SFEM_NEGATIVE_CURVATURE = 3;

thread_local std::string g_err = "";

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CU(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) {                                                                    \
      int code_ = (e_ == cudaErrorMemoryAllocation) ? SFEM_ERR_OOM : SFEM_ERR_CUDA;             \
      return fail(code_, "%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));       \
    }                                                                                           \
  } while (0)

#define TRY(x)            \
  do {                    \
    int s_ = (x);         \
    if (s_ < 0) return s_; \
  } while (0)

template <typename T>
int dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess)
    return fail(e == cudaErrorMemoryAllocation ? SFEM_ERR_OOM : SFEM_ERR_CUDA, "cudaMalloc(%zu bytes): %s",
                count * sizeof(T), cudaGetErrorString(e));
  return 0;
}

template <typename T>
struct KrylovWs {  // vectors of one precision, full length 3N (fixed-node entries stay 0)
  T *b = nullptr, *x = nullptr, *r = nullptr, *p = nullptr, *p2 = nullptr, *q = nullptr, *dinv = nullptr,
    *u = nullptr, *ones = nullptr;
};

struct GnnState;
void gnn_free(GnnState* g);

}  // namespace

int sfem::set_error(int code, const char* msg) {
  g_err = msg;
  return code;
}

struct sfem_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t N = 0, E = 0, nbc = 0, nf = 0;
  int material = SFEM_MMT_NEO_HOOKEAN;
  int precision = SFEM_FP64;
  int tangent = SFEM_TANGENT_REFERENCE;
  double young = 0, poisson = 0, mu = 0, lambda = 0, density = 0, grav[3] = {0, 0, 0}, ff = 1.0;
  std::vector<int32_t> map;  // original -> reshuffled
  int32_t* dmap = nullptr;   // the same on the device
  bool has_scale = false;

  // element data
  int4* tets = nullptr;
  double *X64 = nullptr, *vol64 = nullptr, *scale64 = nullptr, *young_e = nullptr, *scale_la64 = nullptr;
  float *X32 = nullptr, *vol32 = nullptr, *scale32 = nullptr, *scale_la32 = nullptr;
  bool has_scale_la = false;
  // two-term residual: the low parts of X (9 x E) and V (E) beside X32 / vol32, made on first use
  float* df_lo = nullptr;
  int32_t resid_arith = SFEM_RESIDUAL_TWO_TERM;
  // independent instances: free-DOF segments, per-instance activity and residual norms
  int n_inst = 0;
  int64_t* inst_seg = nullptr;   // device, n_inst + 1 (offsets into a free-DOF vector)
  int32_t* inst_active = nullptr;
  double* inst_norm = nullptr;
  std::vector<double> inst_r0, inst_rel;
  std::vector<int32_t> inst_its;
  // instances' own PCG recurrences in one persistent launch (launch_batched_pcg): element instance,
  // node tiles of at most 32 free nodes within one instance, per-tile partials and per-instance scalars
  int bt_mode = 1;  // 1: per-instance persistent PCG (materials 0, 1, 3); 0: one recurrence over all
  int bt_ntiles = 0;
  int32_t *bt_einst = nullptr, *bt_tile_node = nullptr, *bt_tile_cnt = nullptr, *bt_tile_inst = nullptr,
          *bt_inst_tile = nullptr;
  double *bt_part = nullptr, *bt_rz = nullptr, *bt_tol2bb = nullptr, *bt_rr = nullptr;
  int32_t *bt_done = nullptr, *bt_iters = nullptr, *bt_err = nullptr;
  unsigned* bt_bar = nullptr;
  long long bt_wait_limit = 20000000;  // polls of 64 ns or more: about a second at least
  int bt_wait_test = 0;
  std::vector<int32_t> bt_iters_h, bt_status_h;
  std::vector<double> bt_rr_h, bt_bb_h;
  // two-level preconditioner: the coarse-space correction of the learned flexible CG
  bool cs_on = false;
  int cs_n_agg = 0, cs_ld = 0, cs_nk = 0, cs_nm = 6;
  double cs_setup_s[3] = {0.0, 0.0, 0.0};
  int32_t* cs_aid = nullptr;
  float4* cs_d = nullptr;
  __half* cs_W = nullptr;
  float cs_w_inv_scale = 1.f;
  float *cs_s = nullptr, *cs_y = nullptr;
  int cs_n_runs = 0, cs_n_blocks = 0, cs_blk_off = 0;
  int32_t *cs_run_start = nullptr, *cs_blk_run = nullptr, *cs_agg_run_ptr = nullptr, *cs_agg_run = nullptr;
  float* cs_runpart = nullptr;
  // a second stream for the coarse chain's aggregate sums and product, which overlap the first five
  // polynomial passes; events fork and join it
  cudaStream_t cs_stream = nullptr;
  cudaEvent_t cs_fork = nullptr, cs_join = nullptr;
  CoarseView cv() const {
    return CoarseView{cs_n_agg,   cs_nm,     cs_ld,     nf,          cs_aid,       cs_d,           cs_W,           cs_w_inv_scale,
                      cs_s,       cs_y,      cs_n_runs, cs_n_blocks, cs_blk_off,   cs_run_start,   cs_blk_run,     cs_agg_run_ptr,
                      cs_agg_run, cs_runpart};
  }
  // node data (reshuffled, 3N)
  double *x0 = nullptr, *u = nullptr, *mass = nullptr, *fext = nullptr, *grav_d = nullptr;
  // dynamics (FemPhysicsMatrixFree mTimeStep, node vel, pos0 at the step start)
  double dt = 0.0;  // 0: static
  double *vel = nullptr, *ustart = nullptr;
  double* pm64 = nullptr;  // per patch-node slot mass share / h^2 (implicit dynamics)
  // neo-Hookean tangent cache of the running Krylov solve (12 E values per precision)
  double* nhc64 = nullptr;
  float* nhc32 = nullptr;
  bool nhc_on = false;
  // assembled tangent (block CSR over free nodes, built on first use)
  int64_t bsr_nnzb = -1;
  int32_t *bsr_rowptr = nullptr, *bsr_col = nullptr, *bsr_slot = nullptr, *bsr_dslot = nullptr;
  double* bsr_vals = nullptr;
  // FP32 Krylov operator: 0 = matrix-free patch product, 1 = the tangent assembled in sliced ELL
  // at the start of every FP32 Krylov solve (sell_on while its values match the current state)
  int32_t op_mode = 0;
  bool sell_on = false;
  int64_t sell_T = -1, sell_nnzb = 0;  // block-slots (with padding), blocks
  int64_t *sell_base = nullptr, *sell_cptr = nullptr;
  int32_t *sell_col = nullptr, *sell_dslot = nullptr;
  int16_t* sell_col16 = nullptr;  // the columns as differences to the row, when all fit (else sell_col)
  // symmetric tangents: only the diagonal and upper blocks are stored (the slots above); each row's
  // lower blocks are read transposed from their mirror rows: per slice of 32 rows, lower entry
  // (row r, position k) at lbase[r / 32] + 32 k + r % 32 holds the column j (difference j - r, or j)
  // and the block-slot of block (j, r) in row j (-1: padding)
  bool sell_sym = false;
  int64_t sell_nlow = 0;
  int64_t* sell_lbase = nullptr;
  int16_t* sell_lcol16 = nullptr;
  int32_t* sell_lcol = nullptr;
  int32_t* sell_lslot = nullptr;
  uint32_t* sell_code = nullptr;
  float *sell_vals32 = nullptr, *sell_ke32 = nullptr;
  double *sell_vals64 = nullptr, *sell_ke64 = nullptr;
  // device bytes the assembled operator holds, the caller's cap on them (0: none), and whether an
  // allocation failed (then the Krylov solves keep the matrix-free product until the operator is set again)
  int64_t sell_bytes = 0, sell_limit = 0;
  bool sell_oom = false;
  // optional record of every line-search trial of the Newton solves (caller-owned host memory)
  double* ls_trace = nullptr;
  int32_t ls_trace_cap = 0;
  int32_t* ls_trace_count = nullptr;
  int32_t prof_op = 0;  // operator of the sampled Krylov launches
  float* pm32 = nullptr;
  DynView dyn() const { return DynView{vel, ustart, 1.0 / dt, 1.0 / (dt * dt)}; }
  int64_t *csr_ptr = nullptr, *csr_ent = nullptr;
  // element patches (elements are stored in patch order; perm maps to the caller's order)
  std::vector<int32_t> perm_h;
  int32_t* perm = nullptr;
  int64_t n_patches = 0, n_slots = 0, n_shared = 0;
  int max_pnodes = 0;  // largest node count of a patch
  double* rec64 = nullptr;  // patch-product element records (12 values per element, see PatchView::rec)
  float* rec32 = nullptr;
  int64_t *elem_off = nullptr, *node_off = nullptr;
  int32_t *pnode = nullptr, *pdest = nullptr, *bnode = nullptr, *bptr = nullptr, *bidx = nullptr;
  int2* bslot = nullptr;  // per node: (first partial slot, count) of a shared node, (0, 0) otherwise
  uint16_t *lptr = nullptr, *lent = nullptr, *lent12 = nullptr;
  ushort4* lidx = nullptr;
  double* partial = nullptr;  // 3 * n_slots values (float passes use it as floats)
  double* etmp = nullptr;     // E scratch doubles
  GnnState* gnn = nullptr;    // learned preconditioner (sfem_gnn_init)
  // follower pressure surface (sfem_set_pressure_surface)
  int64_t n_tris = 0;
  int32_t *tri = nullptr, *tptr = nullptr, *tent = nullptr;
  double* ptf = nullptr;
  double pressure = 0.0;
  PressureView pres() const { return PressureView{n_tris, tri, tptr, tent, ptf, pressure}; }
  // scratch
  double* fe = nullptr;  // 12 E doubles (float passes use it as 12 E floats)
  double* partials = nullptr;
  unsigned* counter = nullptr;
  CgScalars* scal = nullptr;
  CgScalars* scal_h = nullptr;  // pinned mirror
  double* dres = nullptr;       // small device result slots
  double* dres_h = nullptr;     // pinned mirror
  int* ninv = nullptr;
  // Newton / misc work vectors (FP64, 3N)
  double *r64 = nullptr, *ubase = nullptr, *tmp64 = nullptr, *tmp64b = nullptr;
  KrylovWs<double> k64;
  KrylovWs<float> k32;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // profiling of the element Hessian-vector kernel inside Krylov solves
  bool profiling = false;
  cudaEvent_t pev[3] = {nullptr, nullptr, nullptr};
  double prof_elem_ms = 0, prof_gather_ms = 0;
  int64_t prof_samples = 0, prof_launches = 0;
  int prof_precision = 0;

  Reduce red() const { return Reduce{partials, counter}; }
  PatchBoundary pb() const { return PatchBoundary{n_shared, bnode, bptr}; }
  template <typename T>
  PatchView<T> pv(const T* X, const T* vol, const T* scale, const T* scale_la, T m, T l) const {
    const T* pm = nullptr;
    if (dt > 0) pm = reinterpret_cast<const T*>(sizeof(T) == 8 ? (const void*)pm64 : (const void*)pm32);
    const T* nhc = nullptr;
    if (nhc_on) nhc = reinterpret_cast<const T*>(sizeof(T) == 8 ? (const void*)nhc64 : (const void*)nhc32);
    const T* rec = reinterpret_cast<const T*>(sizeof(T) == 8 ? (const void*)rec64 : (const void*)rec32);
    return PatchView<T>{elem_off, node_off, pnode, pdest, lptr, lent, lidx, X, vol, scale, scale_la, E, n_patches,
                        nbc, m, l, pm, nhc, max_pnodes, rec, sizeof(T) == 4 ? lent12 : nullptr};
  }
  NodeCsr csr() const { return NodeCsr{csr_ptr, csr_ent}; }
  ElemView<double> ev64() const {
    return ElemView<double>{tets, X64, vol64, has_scale ? scale64 : nullptr,
                            has_scale && has_scale_la ? scale_la64 : nullptr, E, mu, lambda};
  }
  ElemView<float> ev32() const {
    return ElemView<float>{tets, X32, vol32, has_scale ? scale32 : nullptr,
                           has_scale && has_scale_la ? scale_la32 : nullptr, E, (float)mu, (float)lambda};
  }
};

namespace {

template <typename T>
int alloc_ws(sfem_handle* h, KrylovWs<T>& w) {
  if (w.b) return 0;
  size_t n = 3 * (size_t)h->N;
  T** ptrs[] = {&w.b, &w.x, &w.r, &w.p, &w.p2, &w.q, &w.dinv, &w.u, &w.ones};
  for (T** p : ptrs) {
    TRY(dalloc(p, n));
    CU(cudaMemsetAsync(*p, 0, n * sizeof(T), h->stream));
  }
  // identity "preconditioner" (1 on free DOFs, 0 on fixed ones) for unpreconditioned CG
  std::vector<T> ones(n, T(0));
  for (size_t i = 3 * (size_t)h->nbc; i < n; i++) ones[i] = T(1);
  CU(cudaMemcpyAsync(w.ones, ones.data(), n * sizeof(T), cudaMemcpyHostToDevice, h->stream));
  CU(cudaStreamSynchronize(h->stream));
  return 0;
}

template <typename T>
ElemView<T> ev_of(const sfem_handle* h);
template <>
ElemView<double> ev_of<double>(const sfem_handle* h) { return h->ev64(); }
template <>
ElemView<float> ev_of<float>(const sfem_handle* h) { return h->ev32(); }

template <typename T>
KrylovWs<T>& ws_of(sfem_handle* h);
template <>
KrylovWs<double>& ws_of<double>(sfem_handle* h) { return h->k64; }
template <>
KrylovWs<float>& ws_of<float>(sfem_handle* h) { return h->k32; }

// internal material id of the kernels: MaterialModelType 0..3, 4 = corotational with the exact
// tangent, m + 1 for the other MaterialModelType values m = 4..12 (FP64 handles only)
int mat_id(const sfem_handle* h) {
  if (h->material == SFEM_MMT_COROTATIONAL && h->tangent == SFEM_TANGENT_EXACT) return 4;
  return h->material <= 3 ? h->material : h->material + 1;
}

// call f(std::integral_constant<int, M>) for the handle's material id (variants in FP64 only)
template <typename T, typename Fn>
void with_mat(int mat, Fn&& f) {
  switch (mat) {
    case 0: f(std::integral_constant<int, 0>{}); return;
    case 1: f(std::integral_constant<int, 1>{}); return;
    case 2: f(std::integral_constant<int, 2>{}); return;
    case 3: f(std::integral_constant<int, 3>{}); return;
    case 4: f(std::integral_constant<int, 4>{}); return;
    default: break;
  }
  if constexpr (sizeof(T) == sizeof(double)) {
    switch (mat) {
      case 5: f(std::integral_constant<int, 5>{}); return;
      case 6: f(std::integral_constant<int, 6>{}); return;
      case 7: f(std::integral_constant<int, 7>{}); return;
      case 8: f(std::integral_constant<int, 8>{}); return;
      case 9: f(std::integral_constant<int, 9>{}); return;
      case 10: f(std::integral_constant<int, 10>{}); return;
      case 11: f(std::integral_constant<int, 11>{}); return;
      case 12: f(std::integral_constant<int, 12>{}); return;
      default: f(std::integral_constant<int, 13>{}); return;
    }
  }
}

template <typename T>
void element_pass(sfem_handle* h, int mode, const T* u, const T* p, T* fe, double* result, int* ninv,
                  const CgScalars* s) {
  const ElemView<T> ev = ev_of<T>(h);
  with_mat<T>(mat_id(h), [&](auto m) {
    launch_element<T, decltype(m)::value>(mode, ev, u, p, fe, h->red(), result, ninv, s, h->stream);
  });
}

// q = K p over the free DOFs with the fused patch kernel (+ p.q and alpha when s is given)
template <typename T>
void hvp(sfem_handle* h, const T* u, const T* p, T* q, CgScalars* s, cudaEvent_t mid = nullptr, const T* r = nullptr,
         const T* dinv = nullptr, T* p_new = nullptr, const T* z = nullptr) {
  const ElemView<T> ev = ev_of<T>(h);
  const PatchView<T> pv = h->pv<T>(ev.X, ev.vol, ev.scale, ev.scale_la, ev.mu, ev.lambda);
  T* part = reinterpret_cast<T*>(h->partial);
  with_mat<T>(mat_id(h), [&](auto m) {
    launch_patch_hvp<T, decltype(m)::value>(pv, h->pb(), u, p, q, part, h->red(), s, h->stream, mid, r, dinv, p_new,
                                            z);
  });
}

// the Krylov loops' product: the assembled FP32 tangent while it is current (sell_on), else the
// patch product; both form the direction on the fly (p_new) and finish p.q and alpha
template <typename T>
void krylov_hvp(sfem_handle* h, const T* u, const T* p, T* q, cudaEvent_t mid, const T* r, const T* dinv, T* p_new,
                const T* z = nullptr) {
  if (h->sell_on) {
    const T* vals;
    if constexpr (std::is_same<T, float>::value)
      vals = h->sell_vals32;
    else
      vals = h->sell_vals64;
    if (h->sell_sym)
      launch_ssell_hvp<T>(h->nbc, h->nf, h->sell_base, h->sell_col, h->sell_col16, h->sell_lbase, h->sell_lcol,
                          h->sell_lcol16, h->sell_lslot, vals, p, q, h->red(), h->scal, h->stream, r, dinv, p_new, z);
    else
      launch_sell_hvp<T>(h->nbc, h->nf, h->sell_base, h->sell_col, h->sell_col16, vals, p, q, h->red(), h->scal,
                         h->stream, r, dinv, p_new, z);
    if (mid) cudaEventRecord(mid, h->stream);
    return;
  }
  hvp<T>(h, u, p, q, h->scal, mid, r, dinv, p_new, z);
}
// shared-node partial slots of the patch product (none with the assembled tangent: q is complete)
template <typename T>
const int2* krylov_bslot(const sfem_handle* h) {
  return h->sell_on ? nullptr : h->bslot;
}

// displacement in precision T for the element passes
template <typename T>
const T* disp(sfem_handle* h);
template <>
const double* disp<double>(sfem_handle* h) { return h->u; }
template <>
const float* disp<float>(sfem_handle* h) {
  launch_convert<double, float>(3 * h->N, h->u, h->k32.u, h->stream);
  return h->k32.u;
}

int sync(sfem_handle* h) {
  CU(cudaStreamSynchronize(h->stream));
  CU(cudaGetLastError());
  return 0;
}

// FP64 residual r64 = f_int + m g ff + f_ext ff; returns |r| and the number of inverted elements.
// With energy (elastic, total), the element pass also sums the elastic energy and a node pass
// the potential of the loads (the values sfem_energy returns, from the same kernels' arithmetic).
// the FP32 handle's neo-Hookean residual in two-term FP32 arithmetic (FP64-accurate; k_element_nh_df)
bool residual_two_term(const sfem_handle* h) {
  return h->resid_arith == SFEM_RESIDUAL_TWO_TERM && h->precision == SFEM_FP32 && mat_id(h) == 3 && h->n_inst == 0;
}
int residual(sfem_handle* h, double* rnorm, int* n_inverted, double* energy = nullptr) {
  CU(cudaMemsetAsync(h->ninv, 0, sizeof(int), h->stream));
  bool tt = residual_two_term(h);
  if (tt && !h->df_lo) {
    const int64_t E = h->E;
    if (dalloc(&h->df_lo, 10 * (size_t)E) == 0) {
      launch_split_geom(9 * E, h->X64, h->X32, h->df_lo, h->stream);
      launch_split_geom(E, h->vol64, h->vol32, h->df_lo + 9 * E, h->stream);
    } else {  // without room for the low parts: the FP64 pass, for this handle from now on
      cudaGetLastError();
      h->df_lo = nullptr;
      h->resid_arith = SFEM_RESIDUAL_FP64;
      g_err.clear();
      tt = false;
    }
  }
  if (tt) {
    const int64_t E = h->E;
    const DfGeom dg{h->X32, h->df_lo, h->vol32, h->df_lo + 9 * E};
    launch_element_nh_df(energy != nullptr, h->ev64(), dg, h->u, reinterpret_cast<float2*>(h->fe), h->red(),
                         energy ? h->dres + 3 : nullptr, h->ninv, h->stream);
  } else {
    element_pass<double>(h, energy ? MODE_FORCE_ENERGY : MODE_FORCE, h->u, nullptr, h->fe,
                         energy ? h->dres + 3 : nullptr, h->ninv, nullptr);
  }
  const PressureView pv = h->pres();
  if (h->n_tris > 0) launch_pressure_tris(pv, h->x0, h->u, h->ff, h->stream);
  const DynView dv = h->dyn();
  launch_gather_force(h->nbc, h->N, h->csr(), h->fe, h->mass, h->fext, h->grav, h->ff, h->r64, h->red(),
                      h->dres, h->stream, h->n_tris > 0 ? &pv : nullptr, h->dt > 0 ? &dv : nullptr, h->u, tt);
  if (energy)
    launch_potential(h->nbc, h->N, h->x0, h->u, h->mass, h->fext, h->grav, h->ff, h->red(), h->dres + 4, h->stream,
                     h->dt > 0 ? &dv : nullptr);
  CU(cudaMemcpyAsync(h->dres_h, h->dres, (energy ? 5 : 1) * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  int ninv_h = 0;
  CU(cudaMemcpyAsync(&ninv_h, h->ninv, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  if (rnorm) *rnorm = std::sqrt(h->dres_h[0]);
  if (n_inverted) *n_inverted = ninv_h;
  if (energy) {
    energy[0] = h->dres_h[3];
    energy[1] = h->dres_h[3] + h->dres_h[4];
  }
  return 0;
}

// Jacobi diagonal (inverse) of the tangent at the current state, precision T.  With the assembled
// operator in use (and only the inverse asked for), from its diagonal blocks: the same sums, formed
// once by the assembly, instead of an element pass.
template <typename T>
int jacobi(sfem_handle* h, T* dinv, T* diag) {
  if (h->sell_on && dinv && !diag) {
    const T* vals;
    if constexpr (std::is_same<T, float>::value)
      vals = h->sell_vals32;
    else
      vals = h->sell_vals64;
    if (vals) {
      launch_sell_diag_inv<T>(h->nbc, h->nf, h->sell_dslot, vals, dinv, h->stream);
      CU(cudaGetLastError());
      return 0;
    }
  }
  const T* u = disp<T>(h);
  T* fe = reinterpret_cast<T*>(h->fe);
  element_pass<T>(h, MODE_DIAG, u, nullptr, fe, nullptr, nullptr, nullptr);
  launch_gather_diag<T>(h->nbc, h->N, h->csr(), fe, dinv, diag, h->stream, h->dt > 0 ? h->mass : nullptr,
                        h->dt > 0 ? 1.0 / (h->dt * h->dt) : 0.0);
  CU(cudaGetLastError());
  return 0;
}

// For a neo-Hookean FP64 solve, the tangent factors of the current state are computed once per
// Krylov solve (k_nh_cache) and the patch product reads them instead of re-forming F, F^-1 and
// log J per element and iteration; the guard switches the cache off when the solve returns.
// FP64 element arithmetic is bound by the FP64 pipe, so trading it for 96 bytes per element pays
// (measured: the FP64 Jacobi-PCG solve of the 6.3M-tet workload 35.5 s -> 23.4 s); the FP32
// product is bound by latency and issue, and the extra bytes made it slower (95 -> 113 us per
// 3.1M tets), so FP32 solves re-form the factors.
template <typename T>
struct NhCacheGuard {
  sfem_handle* h;
  NhCacheGuard(sfem_handle* hh, const T* u) : h(hh) {
    // not with the assembled operator, whose blocks already hold the tangent
    if (h->material != SFEM_MMT_NEO_HOOKEAN || sizeof(T) != sizeof(double) || h->sell_on) return;
    T** c = reinterpret_cast<T**>(sizeof(T) == 8 ? (void*)&h->nhc64 : (void*)&h->nhc32);
    if (!*c && dalloc(c, 12 * (size_t)h->E) != 0) return;  // without memory: the uncached product
    launch_nh_cache<T>(ev_of<T>(h), u, *c, h->stream);
    h->nhc_on = true;
  }
  ~NhCacheGuard() { h->nhc_on = false; }
};

// Preconditioned CG on K x = b (device vectors of the workspace, full length).
// The displacement used by the HVP must already be in ws.u (FP32) / h->u (FP64).
template <typename T>
int pcg_device(sfem_handle* h, const T* u, const T* b, T* x, const T* dinv, double tol, int max_it,
               int check_every, sfem_pcg_stats* st) {
  KrylovWs<T>& w = ws_of<T>(h);
  const int64_t o = 3 * h->nbc, n = 3 * h->nf;
  CgScalars s0;
  memset(&s0, 0, sizeof(s0));
  s0.tol2 = tol * tol;
  s0.max_it = max_it;
  *h->scal_h = s0;
  CU(cudaMemcpyAsync(h->scal, h->scal_h, sizeof(CgScalars), cudaMemcpyHostToDevice, h->stream));
  if (!dinv) dinv = w.ones;  // unpreconditioned CG: z = r
  NhCacheGuard<T> cache(h, u);
  launch_cg_init<T>(n, b + o, x + o, w.r + o, w.p + o, dinv + o, h->red(), h->scal, h->stream);
  // directions alternate between two buffers: iteration k reads p_{k-1} from pbuf[k % 2] and
  // the patch kernel writes p_k = dinv r + beta p_{k-1} into pbuf[(k + 1) % 2]
  T* pbuf[2] = {w.p, w.p2};
  if (check_every <= 0) check_every = 32;
  int it = 0;
  bool pending = false;
  if (h->profiling) {
    h->prof_precision = sizeof(T) == 4 ? SFEM_FP32 : SFEM_FP64;
    h->prof_op = krylov_bslot<T>(h) == nullptr ? 1 : 0;
  }
  for (;;) {
    CU(cudaMemcpyAsync(h->scal_h, h->scal, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    if (h->scal_h->done || it >= max_it) break;
    if (pending) {  // events of the previous chunk's sampled iteration have completed
      float a = 0, b = 0;
      cudaEventElapsedTime(&a, h->pev[0], h->pev[1]);
      cudaEventElapsedTime(&b, h->pev[1], h->pev[2]);
      h->prof_elem_ms += a;
      h->prof_gather_ms += b;
      h->prof_samples++;
      pending = false;
    }
    for (int k = 0; k < check_every && it < max_it; k++, it++) {
      const bool sample = h->profiling && k == 0;
      if (sample) CU(cudaEventRecord(h->pev[0], h->stream));
      T* pold = pbuf[it % 2];
      T* pnew = pbuf[(it + 1) % 2];
      krylov_hvp<T>(h, u, pold, w.q, sample ? h->pev[1] : nullptr, w.r, dinv, pnew);
      if (sample) {
        CU(cudaEventRecord(h->pev[2], h->stream));
        pending = true;
      }
      if (h->profiling) h->prof_launches++;
      launch_cg_update_patch<T>(h->nbc, h->N, krylov_bslot<T>(h), reinterpret_cast<const T*>(h->partial), x, w.r,
                                pnew, w.q, dinv, h->red(), h->scal, h->stream);
    }
  }
  if (pending) {
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, h->pev[0], h->pev[1]);
    cudaEventElapsedTime(&b, h->pev[1], h->pev[2]);
    h->prof_elem_ms += a;
    h->prof_gather_ms += b;
    h->prof_samples++;
  }
  const CgScalars& s = *h->scal_h;
  if (st) {
    st->iters = s.it;
    st->status = s.status;
    st->rel_res = s.bb > 0 ? std::sqrt(s.rr / s.bb) : 0.0;
  }
  if (s.status == -3) return fail(SFEM_ERR_NAN, "non-finite value in the Krylov recurrence");
  if (s.status == 2) {
    // Negative curvature (truncated CG, as in Newton-CG for minimisation): keep the iterate
    // reached so far; at the first iteration return the preconditioned residual direction.
    if (s.it == 0) CU(cudaMemcpyAsync(x + o, pbuf[1] + o, n * sizeof(T), cudaMemcpyDeviceToDevice, h->stream));
    fail(SFEM_ERR_BREAKDOWN, "non-positive curvature p.Ap = %g in CG at iteration %d", s.pq, s.it);
    return SFEM_NEGATIVE_CURVATURE;
  }
  return s.status == 1 ? SFEM_NOT_CONVERGED : SFEM_OK;
}

// Morton order of element centroids, cut greedily into patches of at most
// kPatchElems elements and kPatchNodes distinct nodes.
struct PatchBuild {
  std::vector<int32_t> perm;  // patch position -> caller's element index
  std::vector<int64_t> elem_off, node_off;
  std::vector<int32_t> pnode, pdest, bnode, bptr;
  std::vector<uint16_t> lptr, lent;
  std::vector<ushort4> lidx;
  int max_nodes = 0;
};

uint32_t spread3(uint32_t v) {  // 10 bits -> every third bit
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

void build_patches(const std::vector<int4>& tt, const std::vector<double>& x0, int64_t N, int64_t nbc, PatchBuild& pb) {
  const size_t E = tt.size();
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t i = 0; i < N; i++)
    for (int c = 0; c < 3; c++) {
      lo[c] = std::min(lo[c], x0[3 * i + c]);
      hi[c] = std::max(hi[c], x0[3 * i + c]);
    }
  std::vector<uint32_t> key(E);
  for (size_t e = 0; e < E; e++) {
    const int32_t t[4] = {tt[e].x, tt[e].y, tt[e].z, tt[e].w};
    uint32_t q[3];
    for (int c = 0; c < 3; c++) {
      double m = 0.25 * (x0[3 * (size_t)t[0] + c] + x0[3 * (size_t)t[1] + c] + x0[3 * (size_t)t[2] + c] +
                         x0[3 * (size_t)t[3] + c]);
      double f = hi[c] > lo[c] ? (m - lo[c]) / (hi[c] - lo[c]) : 0.0;
      q[c] = (uint32_t)std::min(1023.0, std::max(0.0, f * 1024.0));
    }
    key[e] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
  }
  std::vector<int32_t> order(E);
  for (size_t e = 0; e < E; e++) order[e] = (int32_t)e;
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });

  std::vector<int32_t> mark(N, -1), local(N, 0), cnt(N, 0);
  pb.perm.clear();
  pb.elem_off.assign(1, 0);
  pb.node_off.assign(1, 0);
  pb.pnode.clear();
  pb.lptr.clear();
  pb.lent.assign(4 * E, 0);
  pb.lidx.assign(E, make_ushort4(0, 0, 0, 0));
  pb.perm.reserve(E);
  size_t k = 0;
  int32_t c = 0;
  std::vector<int32_t> nodes;
  while (k < E) {
    nodes.clear();
    const size_t e0 = k;
    while (k < E && (int64_t)(k - e0) < kPatchElems) {
      const int4 t4 = tt[order[k]];
      const int32_t t[4] = {t4.x, t4.y, t4.z, t4.w};
      int fresh = 0;
      for (int j = 0; j < 4; j++)
        if (mark[t[j]] != c) {
          bool dup = false;
          for (int i = 0; i < j; i++) dup |= (t[i] == t[j]);
          fresh += dup ? 0 : 1;
        }
      if ((int64_t)nodes.size() + fresh > kPatchNodes) break;
      for (int j = 0; j < 4; j++)
        if (mark[t[j]] != c) {
          mark[t[j]] = c;
          nodes.push_back(t[j]);
        }
      pb.perm.push_back(order[k]);
      k++;
    }
    std::sort(nodes.begin(), nodes.end());
    for (size_t j = 0; j < nodes.size(); j++) {
      local[nodes[j]] = (int32_t)j;
      cnt[nodes[j]]++;
    }
    // local corner ids and the local node -> (element, corner) CSR in element order
    const size_t ne = k - e0, nn = nodes.size();
    std::vector<uint16_t> deg(nn + 1, 0);
    for (size_t i = 0; i < ne; i++) {
      const int4 t4 = tt[pb.perm[e0 + i]];
      ushort4 l = make_ushort4((unsigned short)local[t4.x], (unsigned short)local[t4.y], (unsigned short)local[t4.z],
                               (unsigned short)local[t4.w]);
      pb.lidx[e0 + i] = l;
      deg[l.x + 1]++; deg[l.y + 1]++; deg[l.z + 1]++; deg[l.w + 1]++;
    }
    for (size_t j = 0; j < nn; j++) deg[j + 1] += deg[j];
    std::vector<uint16_t> fill(deg.begin(), deg.end() - 1);
    // entries are the shared-memory offsets of (element i, corner j) in the kernel's
    // element-result rows: kFeStride * i + 3 * j
    for (size_t i = 0; i < ne; i++) {
      const ushort4 l = pb.lidx[e0 + i];
      const unsigned short li[4] = {l.x, l.y, l.z, l.w};
      for (int j = 0; j < 4; j++) pb.lent[4 * e0 + fill[li[j]]++] = (uint16_t)(kFeStride * i + 3 * j);
    }
    pb.max_nodes = std::max<int>(pb.max_nodes, (int)nn);
    for (size_t j = 0; j <= nn; j++) pb.lptr.push_back(deg[j]);
    for (size_t j = 0; j < nn; j++) pb.pnode.push_back(nodes[j]);
    pb.elem_off.push_back((int64_t)k);
    pb.node_off.push_back((int64_t)pb.pnode.size());
    c++;
  }
  // shared nodes: flagged in pnode; the partials of a shared free node are stored
  // contiguously (in patch order) for the boundary pass: pdest[slot] is the position
  std::vector<std::vector<int64_t>> slots_of;
  std::vector<int64_t> bid(N, -1);
  pb.bnode.clear();
  pb.pdest.assign(pb.pnode.size(), -1);
  for (size_t sl = 0; sl < pb.pnode.size(); sl++) {
    const int32_t g = pb.pnode[sl];
    if (cnt[g] > 1) {
      pb.pnode[sl] = ~g;
      if (g >= nbc) {
        if (bid[g] < 0) {
          bid[g] = (int64_t)pb.bnode.size();
          pb.bnode.push_back(g);
          slots_of.emplace_back();
        }
        slots_of[bid[g]].push_back((int64_t)sl);
      }
    }
  }
  pb.bptr.assign(1, 0);
  int32_t pos = 0;
  for (auto& v : slots_of) {
    for (int64_t sl : v) pb.pdest[sl] = pos++;
    pb.bptr.push_back(pos);
  }
}

int check_handle(const sfem_handle* h) {
  if (!h) return fail(SFEM_ERR_INVALID, "null handle");
  return 0;
}

int set_device(const sfem_handle* h) {
  CU(cudaSetDevice(h->device));
  return 0;
}

// host original-order N x 3 -> device reshuffled 3N
// one contiguous copy of a node array in the caller's order, permuted on the device
int upload_nodes(sfem_handle* h, const double* src, double* dst) {
  CU(cudaMemcpyAsync(h->tmp64b, src, 3 * (size_t)h->N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_nodes_in(h->N, h->dmap, h->tmp64b, nullptr, 0, dst, h->stream);
  return sync(h);
}

void batch_release(sfem_handle* h);
void coarse_release(sfem_handle* h);
template <typename T>
int batched_pcg(sfem_handle* h, const T* u, const T* rhs, KrylovWs<T>& w, const T* dinv, double tol, int max_it,
                int* its);
}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" {

const char* sfem_last_error(void) { return g_err.c_str(); }

int sfem_create(const double* nodes, int64_t n_nodes, const int32_t* tets_in, int64_t n_tets, const int32_t* fixed,
                int64_t n_fixed, const sfem_config* cfg, sfem_handle** out) {
  if (!out) return fail(SFEM_ERR_INVALID, "out is null");
  *out = nullptr;
  if (!nodes || !tets_in || !cfg || n_nodes <= 0 || n_tets <= 0 || (n_fixed > 0 && !fixed))
    return fail(SFEM_ERR_INVALID, "invalid arguments to sfem_create");
  if (n_nodes >= (1ll << 31) || n_tets >= (1ll << 29)) return fail(SFEM_ERR_INVALID, "mesh too large");
  if (cfg->material < 0 || cfg->material > 12) return fail(SFEM_ERR_INVALID, "unsupported material %d", cfg->material);
  if (cfg->material > 3 && cfg->precision != SFEM_FP64)
    return fail(SFEM_ERR_INVALID, "material %d is available in FP64 handles", cfg->material);
  if (cfg->precision != SFEM_FP64 && cfg->precision != SFEM_FP32)
    return fail(SFEM_ERR_INVALID, "unsupported precision %d", cfg->precision);
  for (int64_t i = 0; i < 4 * n_tets; i++)
    if (tets_in[i] < 0 || tets_in[i] >= n_nodes) return fail(SFEM_ERR_INVALID, "tet index out of range at %lld", (long long)i);
  for (int64_t i = 0; i < n_fixed; i++)
    if (fixed[i] < 0 || fixed[i] >= n_nodes) return fail(SFEM_ERR_INVALID, "fixed index out of range");
  if (!(cfg->young > 0) || !(cfg->poisson > -1.0 && cfg->poisson < 0.5) || !(cfg->density >= 0))
    return fail(SFEM_ERR_INVALID, "invalid material parameters (E > 0, -1 < nu < 0.5, rho >= 0)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(SFEM_ERR_NO_DEVICE, "no CUDA device");

  sfem_handle* h = new sfem_handle();
  h->device = cfg->device;
  h->N = n_nodes;
  h->E = n_tets;
  h->material = cfg->material;
  h->precision = cfg->precision;
  h->tangent = cfg->tangent;
  h->young = cfg->young;
  h->poisson = cfg->poisson;
  h->density = cfg->density;
  for (int c = 0; c < 3; c++) h->grav[c] = cfg->gravity[c];
  // Lame parameters, Source/FemPhysicsBase.cpp:38-39
  h->lambda = cfg->young * cfg->poisson / (1.0 + cfg->poisson) / (1.0 - 2.0 * cfg->poisson);
  h->mu = 0.5 * cfg->young / (1.0 + cfg->poisson);

  auto bail = [&](int code) {
    sfem_destroy(h);
    return code;
  };
  if (cudaSetDevice(h->device) != cudaSuccess) return bail(fail(SFEM_ERR_NO_DEVICE, "cannot select device %d", h->device));
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(SFEM_ERR_CUDA, "stream creation failed"));
  h->own_stream = true;

  // ---- reshuffle: fixed nodes first ----
  std::vector<char> isfix(n_nodes, 0);
  for (int64_t i = 0; i < n_fixed; i++) isfix[fixed[i]] = 1;
  h->map.resize(n_nodes);
  int64_t k = 0;
  for (int64_t i = 0; i < n_nodes; i++)
    if (isfix[i]) h->map[i] = (int32_t)k++;
  h->nbc = k;
  for (int64_t i = 0; i < n_nodes; i++)
    if (!isfix[i]) h->map[i] = (int32_t)k++;
  h->nf = h->N - h->nbc;
  if (h->nf <= 0) return bail(fail(SFEM_ERR_INVALID, "all nodes are fixed"));

  std::vector<double> x0(3 * (size_t)n_nodes);
  for (int64_t i = 0; i < n_nodes; i++)
    for (int c = 0; c < 3; c++) x0[3 * (size_t)h->map[i] + c] = nodes[3 * (size_t)i + c];

  // ---- element precompute (FP64) ----
  const size_t E = (size_t)n_tets;
  std::vector<int4> tt(E);
  std::vector<double> X(9 * E), vol(E), mass(n_nodes, 0.0);
  for (size_t e = 0; e < E; e++) {
    int32_t t[4] = {tets_in[4 * e], tets_in[4 * e + 1], tets_in[4 * e + 2], tets_in[4 * e + 3]};
    for (int j = 0; j < 4; j++) t[j] = h->map[t[j]];
    double D[9];
    for (int pass = 0; pass < 2; pass++) {
      const double* a0 = &x0[3 * (size_t)t[0]];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) D[3 * i + j] = x0[3 * (size_t)t[j + 1] + i] - a0[i];
      double det = D[0] * (D[4] * D[8] - D[5] * D[7]) + D[1] * (D[5] * D[6] - D[3] * D[8]) +
                   D[2] * (D[3] * D[7] - D[4] * D[6]);
      if (pass == 0 && det < 0) {
        std::swap(t[0], t[1]);  // FemBody::Prepare: make the volume positive
        continue;
      }
      if (det == 0) return bail(fail(SFEM_ERR_INVALID, "degenerate element %zu", e));
      double inv[9];
      inv[0] = D[4] * D[8] - D[5] * D[7];
      inv[3] = D[5] * D[6] - D[3] * D[8];
      inv[6] = D[3] * D[7] - D[4] * D[6];
      inv[1] = D[2] * D[7] - D[1] * D[8];
      inv[4] = D[0] * D[8] - D[2] * D[6];
      inv[7] = D[1] * D[6] - D[0] * D[7];
      inv[2] = D[1] * D[5] - D[2] * D[4];
      inv[5] = D[2] * D[3] - D[0] * D[5];
      inv[8] = D[0] * D[4] - D[1] * D[3];
      for (int q = 0; q < 9; q++) X[q * E + e] = inv[q] / det;
      vol[e] = det / 6.0;
      break;
    }
    tt[e] = make_int4(t[0], t[1], t[2], t[3]);
    double lm = 0.25 * vol[e] * h->density;
    for (int j = 0; j < 4; j++) mass[t[j]] += lm;
  }
  // lumped masses as the reference stores them (mass = 1 / (1 / m)), fixed nodes 0
  for (int64_t i = 0; i < n_nodes; i++) mass[i] = (i < h->nbc || mass[i] == 0) ? 0.0 : 1.0 / (1.0 / mass[i]);

  // ---- element patches: Morton order, elements stored in patch order from here on ----
  PatchBuild pbld;
  build_patches(tt, x0, n_nodes, h->nbc, pbld);
  {
    std::vector<int4> ttp(E);
    std::vector<double> Xp(9 * E), volp(E);
    for (size_t k2 = 0; k2 < E; k2++) {
      const int32_t e = pbld.perm[k2];
      ttp[k2] = tt[e];
      volp[k2] = vol[e];
      for (int q = 0; q < 9; q++) Xp[q * E + k2] = X[q * E + e];
    }
    tt.swap(ttp);
    X.swap(Xp);
    vol.swap(volp);
  }
  h->perm_h = pbld.perm;
  h->n_patches = (int64_t)pbld.elem_off.size() - 1;
  h->n_slots = (int64_t)pbld.pnode.size();
  h->max_pnodes = std::max(pbld.max_nodes, 1);
  h->n_shared = (int64_t)pbld.bnode.size();

  // ---- node -> element CSR (entries in element order) ----
  std::vector<int64_t> ptr(n_nodes + 1, 0), ent(4 * E);
  for (size_t e = 0; e < E; e++) {
    ptr[tt[e].x + 1]++; ptr[tt[e].y + 1]++; ptr[tt[e].z + 1]++; ptr[tt[e].w + 1]++;
  }
  for (int64_t i = 0; i < n_nodes; i++) ptr[i + 1] += ptr[i];
  {
    std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
    for (size_t e = 0; e < E; e++) {
      const int32_t t[4] = {tt[e].x, tt[e].y, tt[e].z, tt[e].w};
      for (int j = 0; j < 4; j++) ent[fill[t[j]]++] = ((int64_t)e << 2) | j;
    }
  }

  // ---- device buffers ----
  const size_t N3 = 3 * (size_t)n_nodes;
  int st = 0;
  if ((st = dalloc(&h->tets, E)) || (st = dalloc(&h->X64, 9 * E)) || (st = dalloc(&h->vol64, E)) ||
      (st = dalloc(&h->X32, 9 * E)) || (st = dalloc(&h->vol32, E)) || (st = dalloc(&h->x0, N3)) ||
      (st = dalloc(&h->u, N3)) || (st = dalloc(&h->mass, (size_t)n_nodes)) || (st = dalloc(&h->fext, N3)) ||
      (st = dalloc(&h->vel, N3)) || (st = dalloc(&h->ustart, N3)) ||
      (st = dalloc(&h->grav_d, 3)) || (st = dalloc(&h->csr_ptr, (size_t)n_nodes + 1)) ||
      (st = dalloc(&h->csr_ent, 4 * E)) || (st = dalloc(&h->fe, 12 * E)) ||
      (st = dalloc(&h->partials, std::max<size_t>(4 * (size_t)kMaxBlocks, (size_t)h->n_patches + kMaxBlocks))) ||
      (st = dalloc(&h->counter, 1)) || (st = dalloc(&h->perm, E)) || (st = dalloc(&h->etmp, E)) ||
      (st = dalloc(&h->elem_off, (size_t)h->n_patches + 1)) || (st = dalloc(&h->node_off, (size_t)h->n_patches + 1)) ||
      (st = dalloc(&h->pnode, (size_t)h->n_slots)) || (st = dalloc(&h->pdest, (size_t)h->n_slots)) ||
      (st = dalloc(&h->lptr, (size_t)(h->n_slots + h->n_patches))) ||
      (st = dalloc(&h->lent, 4 * E)) || (st = dalloc(&h->lent12, 4 * E)) || (st = dalloc(&h->lidx, E)) || (st = dalloc(&h->partial, 3 * (size_t)h->n_slots)) ||
      (st = dalloc(&h->bnode, (size_t)h->n_shared)) || (st = dalloc(&h->bptr, (size_t)h->n_shared + 1)) ||
      (st = dalloc(&h->bidx, (size_t)n_nodes)) || (st = dalloc(&h->dmap, (size_t)n_nodes)) ||
      (st = dalloc(&h->bslot, (size_t)n_nodes)) ||
      (st = dalloc(&h->scal, 1)) || (st = dalloc(&h->dres, 8)) || (st = dalloc(&h->ninv, 1)) ||
      (st = dalloc(&h->r64, N3)) || (st = dalloc(&h->ubase, N3)) || (st = dalloc(&h->tmp64, N3)) ||
      (st = dalloc(&h->tmp64b, N3)) || (st = dalloc(&h->rec64, 12 * E)) || (st = dalloc(&h->rec32, 12 * E)))
    return bail(st);
  if (cudaMallocHost((void**)&h->scal_h, sizeof(CgScalars)) != cudaSuccess ||
      cudaMallocHost((void**)&h->dres_h, 8 * sizeof(double)) != cudaSuccess)
    return bail(fail(SFEM_ERR_OOM, "pinned allocation failed"));
  std::vector<float> X32(9 * E), vol32(E);
  for (size_t i = 0; i < 9 * E; i++) X32[i] = (float)X[i];
  for (size_t i = 0; i < E; i++) vol32[i] = (float)vol[i];
  cudaStream_t s = h->stream;
#define UP(dst, src, bytes)                                                                \
  if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)          \
    return bail(fail(SFEM_ERR_CUDA, "upload failed: %s", cudaGetErrorString(cudaGetLastError())));
  UP(h->tets, tt.data(), E * sizeof(int4));
  UP(h->dmap, h->map.data(), (size_t)n_nodes * sizeof(int32_t));
  UP(h->X64, X.data(), 9 * E * sizeof(double));
  UP(h->vol64, vol.data(), E * sizeof(double));
  UP(h->X32, X32.data(), 9 * E * sizeof(float));
  UP(h->vol32, vol32.data(), E * sizeof(float));
  {  // element records of the patch product: one 16-byte-aligned row per element
    std::vector<double> r64(12 * E, 0.0);
    std::vector<float> r32(12 * E, 0.f);
    for (size_t e = 0; e < E; e++) {
      for (int q9 = 0; q9 < 9; q9++) {
        r64[12 * e + q9] = X[q9 * E + e];
        r32[12 * e + q9] = X32[q9 * E + e];
      }
      r64[12 * e + 9] = vol[e];
      r32[12 * e + 9] = vol32[e];
      memcpy(&r64[12 * e + 10], &pbld.lidx[e], sizeof(ushort4));
      memcpy(&r32[12 * e + 10], &pbld.lidx[e], sizeof(ushort4));
    }
    UP(h->rec64, r64.data(), 12 * E * sizeof(double));
    UP(h->rec32, r32.data(), 12 * E * sizeof(float));
  }
  UP(h->x0, x0.data(), N3 * sizeof(double));
  UP(h->mass, mass.data(), (size_t)n_nodes * sizeof(double));
  UP(h->grav_d, h->grav, 3 * sizeof(double));
  UP(h->csr_ptr, ptr.data(), ptr.size() * sizeof(int64_t));
  UP(h->csr_ent, ent.data(), ent.size() * sizeof(int64_t));
  UP(h->perm, pbld.perm.data(), E * sizeof(int32_t));
  UP(h->elem_off, pbld.elem_off.data(), pbld.elem_off.size() * sizeof(int64_t));
  UP(h->node_off, pbld.node_off.data(), pbld.node_off.size() * sizeof(int64_t));
  UP(h->pnode, pbld.pnode.data(), pbld.pnode.size() * sizeof(int32_t));
  UP(h->lptr, pbld.lptr.data(), pbld.lptr.size() * sizeof(uint16_t));
  UP(h->lent, pbld.lent.data(), pbld.lent.size() * sizeof(uint16_t));
  {  // the same entries for 12-value result rows (kFeStride i + 3 j -> 12 i + 3 j)
    std::vector<uint16_t> l12(pbld.lent.size());
    for (size_t t = 0; t < l12.size(); t++) l12[t] = (uint16_t)(pbld.lent[t] - pbld.lent[t] / kFeStride);
    UP(h->lent12, l12.data(), l12.size() * sizeof(uint16_t));
    TRY(sync(h));
  }
  UP(h->lidx, pbld.lidx.data(), pbld.lidx.size() * sizeof(ushort4));
  UP(h->pdest, pbld.pdest.data(), pbld.pdest.size() * sizeof(int32_t));
  if (h->n_shared > 0) UP(h->bnode, pbld.bnode.data(), pbld.bnode.size() * sizeof(int32_t));
  UP(h->bptr, pbld.bptr.data(), pbld.bptr.size() * sizeof(int32_t));
  std::vector<int32_t> bidx_h((size_t)n_nodes, -1);
  std::vector<int2> bslot_h((size_t)n_nodes, make_int2(0, 0));
  for (size_t i = 0; i < pbld.bnode.size(); i++) {
    bidx_h[pbld.bnode[i]] = (int32_t)i;
    bslot_h[pbld.bnode[i]] = make_int2(pbld.bptr[i], pbld.bptr[i + 1] - pbld.bptr[i]);
  }
  UP(h->bidx, bidx_h.data(), bidx_h.size() * sizeof(int32_t));
  UP(h->bslot, bslot_h.data(), bslot_h.size() * sizeof(int2));
#undef UP
  double* zero_bufs[] = {h->u, h->fext, h->r64, h->ubase, h->tmp64, h->tmp64b, h->vel, h->ustart};
  for (double* z : zero_bufs)
    if (cudaMemsetAsync(z, 0, N3 * sizeof(double), s) != cudaSuccess) return bail(fail(SFEM_ERR_CUDA, "memset failed"));
  if (cudaMemsetAsync(h->counter, 0, sizeof(unsigned), s) != cudaSuccess) return bail(fail(SFEM_ERR_CUDA, "memset failed"));
  if (alloc_ws(h, h->k64) < 0) return bail(SFEM_ERR_OOM);
  if (h->precision == SFEM_FP32 && alloc_ws(h, h->k32) < 0) return bail(SFEM_ERR_OOM);
  if (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
    return bail(fail(SFEM_ERR_CUDA, "event creation failed"));
  if (cudaStreamSynchronize(s) != cudaSuccess) return bail(fail(SFEM_ERR_CUDA, "set-up failed: %s", cudaGetErrorString(cudaGetLastError())));
  *out = h;
  return SFEM_OK;
}

int sfem_destroy(sfem_handle* h) {
  if (!h) return SFEM_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  batch_release(h);
  coarse_release(h);
  if (h->cs_stream) {
    cudaStreamSynchronize(h->cs_stream);
    cudaStreamDestroy(h->cs_stream);
  }
  if (h->cs_fork) cudaEventDestroy(h->cs_fork);
  if (h->cs_join) cudaEventDestroy(h->cs_join);
  void* ibufs[] = {h->scale_la64, h->scale_la32, h->inst_seg, h->inst_active, h->inst_norm, h->tri, h->tptr, h->tent,
                   h->ptf, h->vel, h->ustart, h->pm64, h->pm32, h->bsr_rowptr, h->bsr_col, h->bsr_slot,
                   h->bsr_dslot, h->bsr_vals, h->nhc64, h->nhc32, h->rec64, h->rec32, h->sell_base,
                   h->sell_cptr, h->sell_col, h->sell_dslot, h->sell_code, h->sell_vals32, h->sell_ke32,
                   h->sell_col16, h->sell_vals64, h->sell_ke64, h->sell_lbase, h->sell_lcol16, h->sell_lcol,
                   h->sell_lslot};
  for (void* b : ibufs)
    if (b) cudaFree(b);
  void* pbufs[] = {h->perm, h->etmp, h->elem_off, h->node_off, h->pnode, h->pdest, h->lptr, h->lent, h->lent12, h->lidx,
                   h->partial, h->bnode, h->bptr, h->bidx, h->dmap, h->bslot};
  for (void* b : pbufs)
    if (b) cudaFree(b);
  void* bufs[] = {h->tets, h->X64, h->vol64, h->scale64, h->young_e, h->X32, h->vol32, h->scale32, h->x0, h->u,
                  h->mass, h->fext, h->grav_d, h->csr_ptr, h->csr_ent, h->fe, h->partials, h->counter, h->scal,
                  h->dres, h->ninv, h->r64, h->ubase, h->tmp64, h->tmp64b, h->k64.b, h->k64.x, h->k64.r, h->k64.p,
                  h->k64.q, h->k64.dinv, h->k64.u, h->k32.b, h->k32.x, h->k32.r, h->k32.p, h->k32.q, h->k32.dinv,
                  h->k32.u, h->k64.p2, h->k64.ones, h->k32.p2, h->k32.ones, h->df_lo};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (h->scal_h) cudaFreeHost(h->scal_h);
  if (h->dres_h) cudaFreeHost(h->dres_h);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  for (cudaEvent_t e : h->pev)
    if (e) cudaEventDestroy(e);
  if (h->gnn) gnn_free(h->gnn);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return SFEM_OK;
}

int sfem_set_profiling(sfem_handle* h, int32_t enable) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (enable && !h->pev[0])
    for (cudaEvent_t& e : h->pev) CU(cudaEventCreate(&e));
  h->profiling = enable != 0;
  h->prof_elem_ms = h->prof_gather_ms = 0;
  h->prof_samples = h->prof_launches = 0;
  return SFEM_OK;
}

int sfem_get_profile(const sfem_handle* h, sfem_profile* out) {
  TRY(check_handle(h));
  if (!out) return fail(SFEM_ERR_INVALID, "out is null");
  out->hvp_elem_ms = h->prof_elem_ms;
  out->hvp_gather_ms = h->prof_gather_ms;
  out->samples = h->prof_samples;
  out->hvp_launches = h->prof_launches;
  const double sz = h->prof_precision == SFEM_FP32 ? 4.0 : 8.0;
  if (h->prof_op == 1)  // assembled tangent: blocks and their column indices, and per free node the
                        // direction inputs (z or r, p_old) and outputs (p, q)
    out->algo_bytes_hvp = (double)h->sell_nnzb * (9.0 * sz + (h->sell_col16 ? 2.0 : 4.0)) +
                          (double)h->sell_nlow * ((h->sell_col16 ? 2.0 : 4.0) + 4.0) + (double)h->nf * 12.0 * sz;
  else
    out->algo_bytes_hvp = (double)h->E * (16.0 + 10.0 * sz) + (double)h->N * 9.0 * sz;
  out->precision = h->prof_precision;
  out->reserved = 0;
  return SFEM_OK;
}

int sfem_kernel_launches(int64_t* count) {
  if (!count) return fail(SFEM_ERR_INVALID, "count is null");
  *count = (int64_t)sfem::launch_count();
  return SFEM_OK;
}

int sfem_sizes(const sfem_handle* h, int64_t* n_nodes, int64_t* n_free, int64_t* n_tets) {
  TRY(check_handle(h));
  if (n_nodes) *n_nodes = h->N;
  if (n_free) *n_free = h->nf;
  if (n_tets) *n_tets = h->E;
  return SFEM_OK;
}

int sfem_reshuffle_map(const sfem_handle* h, int32_t* map) {
  TRY(check_handle(h));
  if (!map) return fail(SFEM_ERR_INVALID, "map is null");
  memcpy(map, h->map.data(), h->map.size() * sizeof(int32_t));
  return SFEM_OK;
}

int sfem_get_stream(const sfem_handle* h, void** stream) {
  TRY(check_handle(h));
  *stream = (void*)h->stream;
  return SFEM_OK;
}

int sfem_set_stream(sfem_handle* h, void* stream) {
  TRY(check_handle(h));
  TRY(set_device(h));
  CU(cudaStreamSynchronize(h->stream));
  if (h->own_stream) CU(cudaStreamDestroy(h->stream));
  h->own_stream = false;
  h->stream = (cudaStream_t)stream;
  return SFEM_OK;
}

extern "C++" {
// rows [0, n) split over the host's threads
template <typename F>
static void parallel_rows(int64_t n, F&& f, int64_t min_rows = 4096) {
  const int nt = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  if (nt == 1 || n < min_rows) {
    f((int64_t)0, n);
    return;
  }
  std::vector<std::thread> pool;
  const int64_t chunk = (n + nt - 1) / nt;
  for (int k = 0; k < nt; k++) {
    const int64_t a = k * chunk, b = std::min(n, a + chunk);
    if (a < b) pool.emplace_back([&f, a, b] { f(a, b); });
  }
  for (auto& th : pool) th.join();
}

// items [0, n) handed out to the host's threads in chunks of `grain` as they finish (for work
// that grows along the range); each item's result does not depend on which thread ran it
template <typename F>
static void parallel_dynamic(int64_t n, int64_t grain, F&& f) {
  const int nt = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  if (nt == 1 || n <= grain) {
    f((int64_t)0, n);
    return;
  }
  std::atomic<int64_t> next{0};
  auto work = [&] {
    for (;;) {
      const int64_t a = next.fetch_add(grain);
      if (a >= n) return;
      f(a, std::min(n, a + grain));
    }
  };
  std::vector<std::thread> pool;
  for (int k = 0; k < nt; k++) pool.emplace_back(work);
  for (auto& th : pool) th.join();
}

// the sorted free columns of free row r: r and the free corners of the elements at node nbc + r
// (cp / ce: the node->element CSR, entries 4 e + corner)
static void row_columns(int64_t r, int64_t nbc, const std::vector<int4>& tt, const std::vector<int64_t>& cp,
                        const std::vector<int64_t>& ce, std::vector<int32_t>& cols) {
  cols.clear();
  cols.push_back((int32_t)r);
  for (int64_t k = cp[nbc + r]; k < cp[nbc + r + 1]; k++) {
    const int4 t4 = tt[ce[k] >> 2];
    const int32_t v[4] = {t4.x, t4.y, t4.z, t4.w};
    for (int b = 0; b < 4; b++)
      if (v[b] >= nbc) cols.push_back((int32_t)(v[b] - nbc));
  }
  std::sort(cols.begin(), cols.end());
  cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
}
}

// ---- assembled tangent (ElasticEnergy::AssembleStiffnessMatrix, Source/ElasticEnergy.cpp:573-635) ----
// block-CSR pattern of the tangent over the free nodes (sorted columns per row), the block of
// every (element, corner a, corner b) with both corners free (-1 otherwise) and each row's diagonal
static int tangent_pattern(sfem_handle* h, std::vector<int32_t>& rowptr, std::vector<int32_t>& col,
                           std::vector<int32_t>& slot, std::vector<int32_t>& dslot) {
  const int64_t E = h->E, N = h->N, nbc = h->nbc, nf = h->nf;
  std::vector<int4> tt((size_t)E);
  std::vector<int64_t> cp((size_t)N + 1), ce((size_t)4 * E);
  CU(cudaMemcpyAsync(tt.data(), h->tets, tt.size() * sizeof(int4), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(cp.data(), h->csr_ptr, cp.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(ce.data(), h->csr_ent, ce.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  // row lengths, then (rows in parallel) each row's columns, its diagonal and the blocks of the
  // (element, corner) entries at its node: every (e, a) belongs to exactly one row
  std::vector<int64_t> len((size_t)nf + 1, 0);
  parallel_rows(nf, [&](int64_t a, int64_t b) {
    std::vector<int32_t> cols;
    for (int64_t r = a; r < b; r++) {
      row_columns(r, nbc, tt, cp, ce, cols);
      len[r + 1] = (int64_t)cols.size();
    }
  });
  for (int64_t i = 0; i < nf; i++) len[i + 1] += len[i];
  if (len[nf] > (int64_t)INT32_MAX) return fail(SFEM_ERR_INVALID, "tangent too large for 32-bit block indices");
  rowptr.resize((size_t)nf + 1);
  for (int64_t i = 0; i <= nf; i++) rowptr[i] = (int32_t)len[i];
  col.resize((size_t)len[nf]);
  slot.assign((size_t)E * 16, -1);
  dslot.resize((size_t)nf);
  parallel_rows(nf, [&](int64_t a, int64_t b) {
    std::vector<int32_t> cols;
    for (int64_t r = a; r < b; r++) {
      row_columns(r, nbc, tt, cp, ce, cols);
      const int32_t base = rowptr[r];
      std::copy(cols.begin(), cols.end(), col.begin() + base);
      auto find = [&](int32_t c) { return base + (int32_t)(std::lower_bound(cols.begin(), cols.end(), c) - cols.begin()); };
      dslot[r] = find((int32_t)r);
      for (int64_t k = cp[nbc + r]; k < cp[nbc + r + 1]; k++) {
        const int64_t e = ce[k] >> 2;
        const int corner = (int)(ce[k] & 3);
        const int32_t v[4] = {tt[e].x, tt[e].y, tt[e].z, tt[e].w};
        for (int q = 0; q < 4; q++)
          if (v[q] >= nbc) slot[16 * e + 4 * corner + q] = find(v[q] - (int32_t)nbc);
      }
    }
  });
  return 0;
}

static int bsr_structure(sfem_handle* h) {
  if (h->bsr_nnzb >= 0) return 0;
  const int64_t nf = h->nf;
  std::vector<int32_t> rowptr, col, slot, dslot;
  TRY(tangent_pattern(h, rowptr, col, slot, dslot));
  TRY(dalloc(&h->bsr_rowptr, rowptr.size()));
  TRY(dalloc(&h->bsr_col, std::max<size_t>(col.size(), 1)));
  TRY(dalloc(&h->bsr_slot, slot.size()));
  TRY(dalloc(&h->bsr_dslot, std::max<size_t>(dslot.size(), 1)));
  TRY(dalloc(&h->bsr_vals, std::max<size_t>(9 * col.size(), 1)));
  CU(cudaMemcpyAsync(h->bsr_rowptr, rowptr.data(), rowptr.size() * 4, cudaMemcpyHostToDevice, h->stream));
  if (!col.empty()) CU(cudaMemcpyAsync(h->bsr_col, col.data(), col.size() * 4, cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->bsr_slot, slot.data(), slot.size() * 4, cudaMemcpyHostToDevice, h->stream));
  if (nf > 0) CU(cudaMemcpyAsync(h->bsr_dslot, dslot.data(), dslot.size() * 4, cudaMemcpyHostToDevice, h->stream));
  TRY(sync(h));
  h->bsr_nnzb = (int64_t)col.size();
  return 0;
}

// The tangent's pattern in sliced ELL, built row by row from the node->element CSR: a free row's
// columns are the free nodes of its elements (sorted; the diagonal always present); slices of 32
// rows are padded to their longest row (padding blocks point at the row itself and stay zero);
// block (row r, position k) is block-slot base[r / 32] + 32 k + r % 32.  Each block-slot lists
// its contributions 16 e + 4 a + b (block (a, b) of element e, a the row's corner) in the order of
// the row's element entries, so the assembly is a deterministic gather.
// device allocation for the assembled operator, counted against the handle's cap (sell_limit)
extern "C++" {
template <typename T>
static int sell_alloc(sfem_handle* h, T** p, size_t count) {
  *p = nullptr;
  const int64_t bytes = (int64_t)(std::max<size_t>(count, 1) * sizeof(T));
  if (h->sell_limit > 0 && h->sell_bytes + bytes > h->sell_limit)
    return fail(SFEM_ERR_OOM, "assembled operator: %lld more bytes exceed the limit of %lld", (long long)bytes,
                (long long)h->sell_limit);
  TRY(dalloc(p, count));
  h->sell_bytes += bytes;
  return 0;
}
}

// free every buffer of the assembled operator (also the ones a failed build left behind)
static void sell_release(sfem_handle* h) {
  void* bufs[] = {h->sell_base, h->sell_cptr, h->sell_col, h->sell_dslot, h->sell_code, h->sell_vals32,
                  h->sell_ke32, h->sell_col16, h->sell_vals64, h->sell_ke64, h->sell_lbase, h->sell_lcol16,
                  h->sell_lcol, h->sell_lslot};
  for (void* b : bufs)
    if (b) cudaFree(b);
  h->sell_lbase = nullptr;
  h->sell_lcol16 = nullptr;
  h->sell_lcol = nullptr;
  h->sell_lslot = nullptr;
  h->sell_sym = false;
  h->sell_nlow = 0;
  h->sell_base = h->sell_cptr = nullptr;
  h->sell_col = h->sell_dslot = nullptr;
  h->sell_code = nullptr;
  h->sell_vals32 = h->sell_ke32 = nullptr;
  h->sell_col16 = nullptr;
  h->sell_vals64 = h->sell_ke64 = nullptr;
  h->sell_T = -1;
  h->sell_nnzb = 0;
  h->sell_bytes = 0;
}

static int sell_structure(sfem_handle* h) {
  if (h->sell_T >= 0) return 0;
  // the symmetric tangents (linear, StVK, neo-Hookean) store the diagonal and upper blocks only
  const int mat = mat_id(h);
  bool sym = mat == 0 || mat == 1 || mat == 3;
  const int64_t E = h->E, N = h->N, nbc = h->nbc, nf = h->nf, ns = (nf + 31) / 32;
  if (E >= (int64_t(1) << 28)) return fail(SFEM_ERR_INVALID, "too many elements for the assembled operator");
  std::vector<int4> tt((size_t)E);
  std::vector<int64_t> cp((size_t)N + 1), ce((size_t)4 * E);
  CU(cudaMemcpyAsync(tt.data(), h->tets, tt.size() * sizeof(int4), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(cp.data(), h->csr_ptr, cp.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(ce.data(), h->csr_ent, ce.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  auto columns = [&](int64_t r, std::vector<int32_t>& cols) { row_columns(r, nbc, tt, cp, ce, cols); };
  // the blocks a row stores: all of its columns, or (symmetric) those >= the row, the diagonal first
  auto stored = [&](int64_t r, std::vector<int32_t>& cols) {
    columns(r, cols);
    if (sym) cols.erase(cols.begin(), std::lower_bound(cols.begin(), cols.end(), (int32_t)r));
  };
  std::vector<int32_t> len((size_t)nf);
  parallel_rows(nf, [&](int64_t a, int64_t b) {
    std::vector<int32_t> cols;
    for (int64_t r = a; r < b; r++) {
      columns(r, cols);
      len[r] = (int32_t)cols.size();
    }
  });
  if (sym)
    parallel_rows(nf, [&](int64_t a, int64_t b) {
      std::vector<int32_t> cols;
      for (int64_t r = a; r < b; r++) {
        stored(r, cols);
        len[r] = (int32_t)cols.size();
      }
    });
  std::vector<int64_t> base((size_t)ns + 1, 0);
  int64_t nnzb = 0;
  for (int64_t sl = 0; sl < ns; sl++) {
    int64_t w = 0;
    for (int64_t r = 32 * sl; r < std::min(nf, 32 * sl + 32); r++) {
      w = std::max<int64_t>(w, len[r]);
      nnzb += len[r];
    }
    base[sl + 1] = base[sl] + 32 * w;
  }
  const int64_t T = base[ns];
  if (T > (int64_t)INT32_MAX) return fail(SFEM_ERR_INVALID, "tangent too large for 32-bit block-slots");
  std::vector<int32_t> scol((size_t)T, 0), dslot((size_t)nf);
  std::vector<int64_t> cnt((size_t)T + 1, 0);
  // contributions per block-slot (each slot belongs to one row: rows fill theirs independently)
  auto for_contrib = [&](int64_t r, const std::vector<int32_t>& cols, auto&& emit) {
    const int64_t sl = r / 32, l = r % 32;
    for (int64_t k = cp[nbc + r]; k < cp[nbc + r + 1]; k++) {
      const int64_t ent = ce[k], e = ent >> 2;
      const int a = (int)(ent & 3);
      const int32_t v[4] = {tt[e].x, tt[e].y, tt[e].z, tt[e].w};
      for (int b = 0; b < 4; b++) {
        if (v[b] < nbc || (sym && v[b] - nbc < r)) continue;  // fixed node, or a block stored by its mirror
        const int64_t pos = std::lower_bound(cols.begin(), cols.end(), v[b] - (int32_t)nbc) - cols.begin();
        emit(base[sl] + 32 * pos + l, (uint32_t)(16 * e + 4 * a + b));
      }
    }
  };
  parallel_rows(nf, [&](int64_t a, int64_t b) {
    std::vector<int32_t> cols;
    for (int64_t r = a; r < b; r++) {
      stored(r, cols);
      const int64_t sl = r / 32, l = r % 32, w = (base[sl + 1] - base[sl]) / 32;
      for (int64_t k = 0; k < w; k++) {
        const int64_t t = base[sl] + 32 * k + l;
        scol[t] = k < (int64_t)cols.size() ? cols[k] : (int32_t)r;
        if (k < (int64_t)cols.size() && cols[k] == (int32_t)r) dslot[r] = (int32_t)t;
      }
      for_contrib(r, cols, [&](int64_t t, uint32_t) { cnt[t + 1]++; });
    }
  });
  for (int64_t t = 0; t < T; t++) cnt[t + 1] += cnt[t];
  std::vector<uint32_t> code((size_t)cnt[T]);
  parallel_rows(nf, [&](int64_t a, int64_t b) {
    std::vector<int32_t> cols;
    std::vector<int64_t> fill;
    for (int64_t r = a; r < b; r++) {
      stored(r, cols);
      for_contrib(r, cols, [&](int64_t t, uint32_t c) {
        // slots of one row are visited only by this thread: cnt[t] advances as the slot's cursor
        code[cnt[t]++] = c;
      });
    }
  });
  // the fill advanced cnt[t] to the end of slot t's list: shift back to start offsets
  for (int64_t t = T; t > 0; t--) cnt[t] = cnt[t - 1];
  cnt[0] = 0;
  // symmetric: the lower entries, each naming its column j and the block-slot of its mirror (j, r)
  std::vector<int64_t> lbase((size_t)ns + 1, 0);
  std::vector<int32_t> lcol, lslot;
  int64_t nlow = 0;
  if (sym) {
    std::vector<int32_t> llen((size_t)nf);
    parallel_rows(nf, [&](int64_t a, int64_t b) {
      std::vector<int32_t> cols;
      for (int64_t r = a; r < b; r++) {
        columns(r, cols);
        llen[r] = (int32_t)(std::lower_bound(cols.begin(), cols.end(), (int32_t)r) - cols.begin());
      }
    });
    for (int64_t sl = 0; sl < ns; sl++) {
      int64_t w = 0;
      for (int64_t r = 32 * sl; r < std::min(nf, 32 * sl + 32); r++) {
        w = std::max<int64_t>(w, llen[r]);
        nlow += llen[r];
      }
      lbase[sl + 1] = lbase[sl] + 32 * w;
    }
    const int64_t L = lbase[ns];
    lcol.assign((size_t)L, 0);
    lslot.assign((size_t)L, -1);
    parallel_rows(nf, [&](int64_t a, int64_t b) {
      std::vector<int32_t> cols;
      for (int64_t r = a; r < b; r++) {
        columns(r, cols);
        const int64_t sl = r / 32, l = r % 32, w = (lbase[sl + 1] - lbase[sl]) / 32;
        for (int64_t k = 0; k < w; k++) {
          const int64_t t = lbase[sl] + 32 * k + l;
          if (k < llen[r]) {
            const int32_t jc = cols[k];
            // row jc's stored columns ascend over its first len[jc] positions
            const int64_t js = jc / 32, jl = jc % 32;
            int lo = 0, hi = len[jc];
            while (lo < hi) {
              const int mid = (lo + hi) / 2;
              if (scol[base[js] + 32 * mid + jl] < (int32_t)r) lo = mid + 1; else hi = mid;
            }
            lcol[t] = jc;
            lslot[t] = (int32_t)(base[js] + 32 * lo + jl);
          } else {
            lcol[t] = (int32_t)r;  // padding (slot -1): skipped
          }
        }
      }
    });
  }
  // 16-bit column differences (2 instead of 4 bytes per block) when every |column - row| fits
  bool fits16 = true;
  for (int64_t r = 0; r < nf && fits16 && sym; r++) {
    const int64_t sl = r / 32, l = r % 32, w = (lbase[sl + 1] - lbase[sl]) / 32;
    for (int64_t k = 0; k < w; k++)
      if ((int64_t)lcol[lbase[sl] + 32 * k + l] - r < -32768) {
        fits16 = false;
        break;
      }
  }
  for (int64_t r = 0; r < nf && fits16; r++) {
    const int64_t sl = r / 32, l = r % 32, w = (base[sl + 1] - base[sl]) / 32;
    for (int64_t k = 0; k < w; k++) {
      const int64_t d = (int64_t)scol[base[sl] + 32 * k + l] - r;
      if (d < -32768 || d > 32767) {
        fits16 = false;
        break;
      }
    }
  }
  TRY(sell_alloc(h, &h->sell_base, base.size()));
  if (fits16) {
    std::vector<int16_t> d16((size_t)T, 0);
    for (int64_t r = 0; r < nf; r++) {
      const int64_t sl = r / 32, l = r % 32, w = (base[sl + 1] - base[sl]) / 32;
      for (int64_t k = 0; k < w; k++) {
        const int64_t t = base[sl] + 32 * k + l;
        d16[t] = (int16_t)((int64_t)scol[t] - r);
      }
    }
    TRY(sell_alloc(h, &h->sell_col16, std::max<size_t>(d16.size(), 1)));
    if (T > 0) CU(cudaMemcpyAsync(h->sell_col16, d16.data(), d16.size() * 2, cudaMemcpyHostToDevice, h->stream));
    TRY(sync(h));
  }
  if (!fits16) TRY(sell_alloc(h, &h->sell_col, std::max<size_t>(scol.size(), 1)));
  TRY(sell_alloc(h, &h->sell_cptr, cnt.size()));
  TRY(sell_alloc(h, &h->sell_code, std::max<size_t>(code.size(), 1)));
  TRY(sell_alloc(h, &h->sell_dslot, std::max<size_t>(dslot.size(), 1)));

  CU(cudaMemcpyAsync(h->sell_base, base.data(), base.size() * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
  if (!fits16 && T > 0)
    CU(cudaMemcpyAsync(h->sell_col, scol.data(), scol.size() * 4, cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->sell_cptr, cnt.data(), cnt.size() * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
  if (!code.empty())
    CU(cudaMemcpyAsync(h->sell_code, code.data(), code.size() * 4, cudaMemcpyHostToDevice, h->stream));
  if (nf > 0) CU(cudaMemcpyAsync(h->sell_dslot, dslot.data(), dslot.size() * 4, cudaMemcpyHostToDevice, h->stream));

  if (sym) {
    const int64_t L = lbase[ns];
    TRY(sell_alloc(h, &h->sell_lbase, lbase.size()));
    TRY(sell_alloc(h, &h->sell_lslot, std::max<size_t>(lslot.size(), 1)));
    CU(cudaMemcpyAsync(h->sell_lbase, lbase.data(), lbase.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                       h->stream));
    if (L > 0) CU(cudaMemcpyAsync(h->sell_lslot, lslot.data(), lslot.size() * 4, cudaMemcpyHostToDevice, h->stream));
    if (fits16) {
      std::vector<int16_t> d16((size_t)L, 0);
      for (int64_t r = 0; r < nf; r++) {
        const int64_t sl = r / 32, l = r % 32, w = (lbase[sl + 1] - lbase[sl]) / 32;
        for (int64_t k = 0; k < w; k++) {
          const int64_t t = lbase[sl] + 32 * k + l;
          d16[t] = (int16_t)((int64_t)lcol[t] - r);
        }
      }
      TRY(sell_alloc(h, &h->sell_lcol16, std::max<size_t>(d16.size(), 1)));
      if (L > 0) CU(cudaMemcpyAsync(h->sell_lcol16, d16.data(), d16.size() * 2, cudaMemcpyHostToDevice, h->stream));
      TRY(sync(h));
    } else {
      TRY(sell_alloc(h, &h->sell_lcol, std::max<size_t>(lcol.size(), 1)));
      if (L > 0) CU(cudaMemcpyAsync(h->sell_lcol, lcol.data(), lcol.size() * 4, cudaMemcpyHostToDevice, h->stream));
    }
  }
  TRY(sync(h));
  h->sell_T = T;
  h->sell_nnzb = nnzb;
  h->sell_sym = sym;
  h->sell_nlow = nlow;
  return 0;
}

extern "C++" {
// assemble the tangent at the current state into the sliced-ELL values of precision T
template <typename T>
static int sell_assemble(sfem_handle* h) {
  TRY(sell_structure(h));
  T** vals = reinterpret_cast<T**>(sizeof(T) == 4 ? (void*)&h->sell_vals32 : (void*)&h->sell_vals64);
  T** ke = reinterpret_cast<T**>(sizeof(T) == 4 ? (void*)&h->sell_ke32 : (void*)&h->sell_ke64);
  if (!*vals) TRY(sell_alloc(h, vals, std::max<size_t>(9 * (size_t)h->sell_T, 1)));
  const int mat = mat_id(h);
  if (mat > 4) return fail(SFEM_ERR_INVALID, "the assembled operator covers materials 0-3");
  const T* uT = disp<T>(h);
  const ElemView<T> ev = ev_of<T>(h);
  if constexpr (sizeof(T) == 4) {
    if (mat == 3) {  // FP32 neo-Hookean: 24 factors per element instead of ten 12-slot blocks
      if (!*ke) TRY(sell_alloc(h, ke, (size_t)h->E * kNhFactorsHost));
      launch_assemble_sell_nh32(ev, uT, *ke, h->sell_T, h->sell_cptr, h->sell_code, h->nbc, h->nf, h->sell_dslot,
                                h->dt > 0 ? h->mass : nullptr, h->dt > 0 ? 1.0 / (h->dt * h->dt) : 0.0, *vals,
                                h->stream);
      CU(cudaGetLastError());
      return 0;
    }
  }
  // 12-slot blocks per element: 16 for the corotational tangents (not symmetric), 10 otherwise
  const int nb_alloc = (h->material == SFEM_MMT_COROTATIONAL) ? 16 : 10;
  if (!*ke) TRY(sell_alloc(h, ke, (size_t)h->E * 12 * nb_alloc));
  int nb = 10;
  with_mat<float>(mat, [&](auto m) {  // the materials 0-4 (dispatch list shared by both precisions)
    nb = launch_element_stiffness_sym<T, decltype(m)::value>(ev, uT, *ke, h->stream);
  });
  launch_assemble_sell<T>(h->sell_T, h->sell_cptr, h->sell_code, *ke, nb, h->nbc, h->nf, h->sell_dslot,
                          h->dt > 0 ? h->mass : nullptr, h->dt > 0 ? 1.0 / (h->dt * h->dt) : 0.0, *vals, h->stream);
  CU(cudaGetLastError());
  return 0;
}
}

// The Krylov solves' operator for their duration: with op_mode 1 (materials 0-3, no batched
// instances) the tangent is assembled at the current state in the handle's precision and the
// loops use it; the patch product otherwise.
struct OperatorScope {
  sfem_handle* h;
  int st = 0;
  explicit OperatorScope(sfem_handle* hh) : h(hh) {
    if (h->op_mode == 1 && h->n_inst == 0 && mat_id(h) <= 4 && !h->sell_oom) {
      st = h->precision == SFEM_FP32 ? sell_assemble<float>(h) : sell_assemble<double>(h);
      h->sell_on = st == 0;
      if (st == SFEM_ERR_OOM) {
        // without the memory: free what the failed build holds, remember the failure so that later
        // Newton steps go straight to the matrix-free product, and report success
        cudaGetLastError();
        sell_release(h);
        h->sell_oom = true;
        g_err.clear();
        st = 0;
      }
    }
  }
  ~OperatorScope() { h->sell_on = false; }
};

// assemble the FP64 tangent at the current state into h->bsr_vals
static int bsr_assemble(sfem_handle* h) {
  TRY(bsr_structure(h));
  double* Ke = nullptr;
  TRY(dalloc(&Ke, (size_t)h->E * 144));
  const ElemView<double> ev = h->ev64();
  with_mat<double>(mat_id(h), [&](auto m) { launch_element_stiffness<double, decltype(m)::value>(ev, h->u, Ke, h->stream); });
  CU(cudaMemsetAsync(h->bsr_vals, 0, 9 * (size_t)h->bsr_nnzb * sizeof(double), h->stream));
  launch_assemble_bsr(h->nbc, h->N, h->csr(), Ke, h->bsr_slot, h->bsr_dslot, h->dt > 0 ? h->mass : nullptr,
                      h->dt > 0 ? 1.0 / (h->dt * h->dt) : 0.0, h->bsr_vals, h->stream);
  const int st = sync(h);
  cudaFree(Ke);
  return st;
}

int sfem_set_operator(sfem_handle* h, int32_t op) {
  TRY(check_handle(h));
  if (op != SFEM_OP_MATRIX_FREE && op != SFEM_OP_ASSEMBLED)
    return fail(SFEM_ERR_INVALID, "operator is SFEM_OP_MATRIX_FREE (0) or SFEM_OP_ASSEMBLED (1)");
  h->op_mode = op;
  h->sell_oom = false;  // setting the operator again retries the assembly
  if (op == SFEM_OP_MATRIX_FREE && h->sell_T >= 0) {  // release the assembled operator's memory
    TRY(set_device(h));
    TRY(sync(h));
    sell_release(h);
  }
  return SFEM_OK;
}

}  // extern "C"

extern "C++" {
// In-place Cholesky A = L L^T of a dense symmetric positive definite n x n matrix (row-major; L in
// the lower triangle), right-looking in blocks of 64: the diagonal block, then the panel below it
// (rows in parallel), then the trailing update A22 -= P P^T as 4 x 8 register tiles over the panel
// packed transposed (tiles in parallel, the order of every sum fixed).  False if a pivot is not
// positive.
static bool cholesky_lower(std::vector<double>& A, int n) {
  const int bs = 64;
  std::vector<double> Pt;
  for (int k0 = 0; k0 < n; k0 += bs) {
    const int k1 = std::min(n, k0 + bs), w = k1 - k0;
    for (int k = k0; k < k1; k++) {
      double d = A[(size_t)k * n + k];
      for (int p = k0; p < k; p++) d -= A[(size_t)k * n + p] * A[(size_t)k * n + p];
      if (!(d > 0.0) || !std::isfinite(d)) return false;
      d = std::sqrt(d);
      A[(size_t)k * n + k] = d;
      for (int i = k + 1; i < k1; i++) {
        double t = A[(size_t)i * n + k];
        for (int p = k0; p < k; p++) t -= A[(size_t)i * n + p] * A[(size_t)k * n + p];
        A[(size_t)i * n + k] = t / d;
      }
    }
    const int m = n - k1;
    if (m <= 0) break;
    parallel_rows(m, [&](int64_t a, int64_t b) {
      for (int64_t i = k1 + a; i < k1 + b; i++) {
        double* Ai = &A[(size_t)i * n];
        for (int k = k0; k < k1; k++) {
          const double* Ak = &A[(size_t)k * n];
          double t = Ai[k];
          for (int p = k0; p < k; p++) t -= Ai[p] * Ak[p];
          Ai[k] = t / Ak[k];
        }
      }
    }, 64);
    // P^T: Pt[p][r] = A[k1 + r][k0 + p], rows padded with zeros past every tile read (8 beyond m, to a
    // multiple of 8)
    const int mp = (m + 7) / 8 * 8 + 8;
    Pt.assign((size_t)w * mp, 0.0);
    parallel_rows(m, [&](int64_t a, int64_t b) {
      for (int64_t r = a; r < b; r++)
        for (int p = 0; p < w; p++) Pt[(size_t)p * mp + r] = A[(size_t)(k1 + r) * n + k0 + p];
    }, 256);
    // the lower trailing block in tiles of 4 rows x 8 columns (j <= i), row tiles handed out dynamically
    const int nti = (m + 3) / 4;
    parallel_dynamic(nti, 4, [&](int64_t t0, int64_t t1) {
      for (int64_t ti = t0; ti < t1; ti++) {
        const int i0 = (int)(4 * ti);
        const int jmax = std::min(m, i0 + 4);  // columns 0 .. jmax - 1 reach the tile's rows
        for (int j0 = 0; j0 < jmax; j0 += 8) {
          double acc[4][8];
          for (int r = 0; r < 4; r++)
            for (int c = 0; c < 8; c++) acc[r][c] = 0.0;
          for (int p = 0; p < w; p++) {
            const double* pr = &Pt[(size_t)p * mp];
            const double a0 = pr[i0], a1 = pr[i0 + 1], a2 = pr[i0 + 2], a3 = pr[i0 + 3];
            const double* pb = pr + j0;
            for (int c = 0; c < 8; c++) {
              const double bv = pb[c];
              acc[0][c] += a0 * bv;
              acc[1][c] += a1 * bv;
              acc[2][c] += a2 * bv;
              acc[3][c] += a3 * bv;
            }
          }
          for (int r = 0; r < 4 && i0 + r < m; r++) {
            double* Ai = &A[(size_t)(k1 + i0 + r) * n + k1];
            for (int c = 0; c < 8 && j0 + c <= i0 + r; c++) Ai[j0 + c] -= acc[r][c];
          }
        }
      }
    });
  }
  return true;
}

// The inverse of A = L L^T (L from cholesky_lower, lower triangle of a row-major n x n array) into
// Ainv (n x n, full, exactly symmetric).  Columns in groups of 8, each group on one host thread: the
// forward substitution L y = e_c from the group's first row down, then the backward substitution
// L^T x = y from row n - 1 up to the group's first row (the rows of x at and below it are the lower
// triangle's entries; the rest come from the symmetry).  Both run over rows in tiles of 4: the terms
// of rows already solved as 4 x 8 register tiles (four rows share every load of y or x), then the
// tile's own 4 x 4 triangle in order.  Every sum has a fixed order.
static void cholesky_inverse(const std::vector<double>& L, int n, std::vector<double>& Ainv) {
  constexpr int G = 8;
  std::vector<double> U((size_t)n * n);  // L^T row-major: column i of L contiguous
  parallel_rows(n, [&](int64_t a, int64_t b) {
    for (int64_t j = a; j < b; j++)
      for (int64_t i = j; i < n; i++) U[(size_t)j * n + i] = L[(size_t)i * n + j];
  }, 64);
  Ainv.assign((size_t)n * n, 0.0);
  const int64_t ng = (n + G - 1) / G;
  parallel_dynamic(ng, 1, [&](int64_t g0, int64_t g1) {
    std::vector<double> Y((size_t)n * G);
    for (int64_t g = g0; g < g1; g++) {
      const int c0 = (int)(g * G), w = std::min(G, n - c0);
      std::fill(Y.begin() + (size_t)c0 * G, Y.end(), 0.0);
      // L y = e_c, rows c0 .. n - 1 in tiles of 4 going down
      for (int i0 = c0; i0 < n; i0 += 4) {
        const int ni = std::min(4, n - i0);
        double acc[4][G];
        for (int r = 0; r < 4; r++)
          for (int k = 0; k < G; k++) acc[r][k] = (i0 + r == c0 + k) ? 1.0 : 0.0;
        const double* R0 = &L[(size_t)i0 * n];
        const double* R1 = ni > 1 ? R0 + n : R0;
        const double* R2 = ni > 2 ? R0 + 2 * (size_t)n : R0;
        const double* R3 = ni > 3 ? R0 + 3 * (size_t)n : R0;
        for (int p = c0; p < i0; p++) {
          const double l0 = R0[p], l1 = R1[p], l2 = R2[p], l3 = R3[p];
          const double* yp = &Y[(size_t)p * G];
          for (int k = 0; k < G; k++) {
            const double yv = yp[k];
            acc[0][k] -= l0 * yv;
            acc[1][k] -= l1 * yv;
            acc[2][k] -= l2 * yv;
            acc[3][k] -= l3 * yv;
          }
        }
        for (int r = 0; r < ni; r++) {
          const double* Lr = &L[(size_t)(i0 + r) * n];
          for (int q = 0; q < r; q++) {
            const double l = Lr[i0 + q];
            for (int k = 0; k < G; k++) acc[r][k] -= l * Y[(size_t)(i0 + q) * G + k];
          }
          const double inv = 1.0 / Lr[i0 + r];
          for (int k = 0; k < G; k++) Y[(size_t)(i0 + r) * G + k] = acc[r][k] * inv;
        }
      }
      // L^T x = y, rows n - 1 .. c0 in tiles of 4 going up (x overwrites y)
      for (int i1 = n - 1; i1 >= c0; i1 -= 4) {  // the tile's rows i1, i1 - 1, ... (at most 4, >= c0)
        const int ni = std::min(4, i1 - c0 + 1);
        double acc[4][G];
        for (int r = 0; r < 4; r++)
          for (int k = 0; k < G; k++) acc[r][k] = r < ni ? Y[(size_t)(i1 - r) * G + k] : 0.0;
        const double* R0 = &U[(size_t)i1 * n];
        const double* R1 = ni > 1 ? R0 - n : R0;
        const double* R2 = ni > 2 ? R0 - 2 * (size_t)n : R0;
        const double* R3 = ni > 3 ? R0 - 3 * (size_t)n : R0;
        for (int p = i1 + 1; p < n; p++) {
          const double u0 = R0[p], u1 = R1[p], u2 = R2[p], u3 = R3[p];
          const double* xp = &Y[(size_t)p * G];
          for (int k = 0; k < G; k++) {
            const double xv = xp[k];
            acc[0][k] -= u0 * xv;
            acc[1][k] -= u1 * xv;
            acc[2][k] -= u2 * xv;
            acc[3][k] -= u3 * xv;
          }
        }
        for (int r = 0; r < ni; r++) {  // row i1 - r needs the rows i1 - r + 1 .. i1 of this tile
          const int i = i1 - r;
          const double* Ur = &U[(size_t)i * n];
          for (int q = 0; q < r; q++) {
            const double u = Ur[i1 - q];
            for (int k = 0; k < G; k++) acc[r][k] -= u * Y[(size_t)(i1 - q) * G + k];
          }
          const double inv = 1.0 / Ur[i];
          for (int k = 0; k < G; k++) Y[(size_t)i * G + k] = acc[r][k] * inv;
        }
      }
      for (int k = 0; k < w; k++) {
        const int c = c0 + k;
        for (int i = c; i < n; i++) {
          const double v = Y[(size_t)i * G + k];
          Ainv[(size_t)i * n + c] = v;
          Ainv[(size_t)c * n + i] = v;
        }
      }
    }
  });
}
}

extern "C" {

int sfem_set_coarse_space(sfem_handle* h, double cell, double rtol) { return sfem_set_coarse_space_modes(h, cell, rtol, 6); }

int sfem_set_coarse_space_modes(sfem_handle* h, double cell, double rtol, int32_t modes) {
  TRY(check_handle(h));
  TRY(set_device(h));
  TRY(sync(h));
  coarse_release(h);
  if (!(cell > 0.0)) return SFEM_OK;  // off
  if (h->precision != SFEM_FP32) return fail(SFEM_ERR_INVALID, "the coarse space serves the FP32 flexible CG");
  if (!(rtol >= 0.0)) return fail(SFEM_ERR_INVALID, "rtol >= 0");
  if (modes != 6 && modes != 12 && modes != 30)
    return fail(SFEM_ERR_INVALID, "modes is 6 (rigid), 12 (affine) or 30 (quadratic)");
  const int nm = modes;
  const int64_t nf = h->nf, nbc = h->nbc;
  if (nf == 0) return SFEM_OK;
  // aggregates of the free nodes' rest positions and their modes' factors
  std::vector<double> X((size_t)3 * nf);
  CU(cudaMemcpyAsync(X.data(), h->x0 + 3 * nbc, X.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  std::vector<int32_t> aid((size_t)nf);
  std::vector<double> d((size_t)3 * nf);
  int64_t na = 0;
  TRY(sfem_coarse_factors(X.data(), nf, cell, rtol, aid.data(), d.data(), nullptr, &na));
  // the dense factorisation costs ~(nm n_agg)^3 / 2 multiply-adds on the host and W (nm n_agg)^2 halves:
  // at most 2048 aggregates and 12,288 modes
  if (na > 2048 || na * nm > 12288)
    return fail(SFEM_ERR_INVALID, "the coarse space has %lld aggregates of %d modes (at most 2048 and 12,288 modes)",
                (long long)na, nm);
  std::vector<double> R((size_t)nm * nm * na);
  if (nm == 6)
    TRY(sfem_coarse_factors(X.data(), nf, cell, rtol, aid.data(), d.data(), R.data(), &na));
  else
    TRY(sfem_coarse_factors_poly(X.data(), nf, cell, rtol, nm == 12 ? 1 : 2, aid.data(), d.data(), R.data(), &na));
  using clk = std::chrono::steady_clock;
  auto secs = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); };
  const clk::time_point t0 = clk::now();
  // the FP64 tangent at the rest state, as block CSR over the free nodes
  std::vector<double> u_save((size_t)3 * h->N);
  CU(cudaMemcpyAsync(u_save.data(), h->u, u_save.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemsetAsync(h->u, 0, u_save.size() * sizeof(double), h->stream));
  const int ast = bsr_assemble(h);
  CU(cudaMemcpyAsync(h->u, u_save.data(), u_save.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TRY(sync(h));
  TRY(ast);
  std::vector<int32_t> rowptr((size_t)nf + 1), col((size_t)h->bsr_nnzb);
  std::vector<double> vals((size_t)9 * h->bsr_nnzb);
  CU(cudaMemcpyAsync(rowptr.data(), h->bsr_rowptr, rowptr.size() * 4, cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(col.data(), h->bsr_col, col.size() * 4, cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(vals.data(), h->bsr_vals, vals.size() * 8, cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  const clk::time_point t1 = clk::now();
  // kept (non-zero) columns of every R_a and their positions in the compact coarse index
  std::vector<std::vector<int>> kc((size_t)na);
  std::vector<int> first((size_t)na + 1, 0);
  const int nm2 = nm * nm;
  for (int64_t a = 0; a < na; a++) {
    for (int c = 0; c < nm; c++) {
      double nz = 0.0;
      for (int r = 0; r < nm; r++) nz += std::fabs(R[nm2 * a + nm * r + c]);
      if (nz > 0.0) kc[a].push_back(c);
    }
    first[a + 1] = first[a] + (int)kc[a].size();
  }
  const int nk = first[na];
  // aggregate node lists (free-node indices, increasing)
  std::vector<int32_t> aptr((size_t)na + 1, 0), anode((size_t)nf);
  for (int64_t i = 0; i < nf; i++) aptr[aid[i] + 1]++;
  for (int64_t a = 0; a < na; a++) aptr[a + 1] += aptr[a];
  {
    std::vector<int32_t> fill(aptr.begin(), aptr.end() - 1);
    for (int64_t i = 0; i < nf; i++) anode[fill[aid[i]]++] = (int32_t)i;
  }
  // Kc = R^T (B^T K B) R by aggregate pairs: row aggregate a sums B_i^T K_ij B_j over its nodes i
  // and their blocks j in a fixed order (one thread per aggregate row: deterministic)
  std::vector<double> Kc((size_t)nk * nk, 0.0);
  auto Bmat = [&](int64_t i, double (&B)[3][30]) {  // [I, -[d]x] (rigid) or I (x) features (polynomial)
    const double* di = &d[3 * i];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < nm; c++) B[r][c] = (nm == 6 && c == r) ? 1.0 : 0.0;
    if (nm == 6) {
      B[1][3] = -di[2]; B[2][3] = di[1];
      B[2][4] = -di[0]; B[0][4] = di[2];
      B[0][5] = -di[1]; B[1][5] = di[0];
    } else {
      const int F = nm / 3;
      const double f[10] = {1.0, di[0], di[1], di[2], di[0] * di[0], di[1] * di[1], di[2] * di[2],
                            di[0] * di[1], di[1] * di[2], di[2] * di[0]};
      for (int k = 0; k < 3; k++)
        for (int m = 0; m < F; m++) B[k][F * k + m] = f[m];
    }
  };
  parallel_rows(na, [&](int64_t a0, int64_t a1) {
    std::vector<int> slot((size_t)na, -1);
    std::vector<int> touched;
    std::vector<double> G, Tg((size_t)nm * nm);
    for (int64_t a = a0; a < a1; a++) {
      touched.clear();
      G.clear();
      for (int32_t k = aptr[a]; k < aptr[a + 1]; k++) {
        const int64_t i = anode[k];
        double Bi[3][30];
        Bmat(i, Bi);
        for (int32_t e = rowptr[i]; e < rowptr[i + 1]; e++) {
          const int64_t j = col[e];
          const int b = aid[j];
          if (slot[b] < 0) {
            slot[b] = (int)touched.size();
            touched.push_back(b);
            G.resize(G.size() + nm2, 0.0);
          }
          const double* Kij = &vals[9 * (size_t)e];
          double* g = &G[nm2 * (size_t)slot[b]];
          if (nm == 6) {
            double Bj[3][30], KB[3][30];
            Bmat(j, Bj);
            for (int r = 0; r < 3; r++)
              for (int c = 0; c < nm; c++)
                KB[r][c] = Kij[3 * r] * Bj[0][c] + Kij[3 * r + 1] * Bj[1][c] + Kij[3 * r + 2] * Bj[2][c];
            for (int x = 0; x < nm; x++)
              for (int c = 0; c < nm; c++) g[nm * x + c] += Bi[0][x] * KB[0][c] + Bi[1][x] * KB[1][c] + Bi[2][x] * KB[2][c];
          } else {
            // polynomial modes: B_i = I (x) f(d_i), so (B_i^T K_ij B_j)[F r + m][F s + l] = f_m(d_i) K_ij[r][s] f_l(d_j)
            const int F = nm / 3;
            const double* dj = &d[3 * j];
            const double fj[10] = {1.0, dj[0], dj[1], dj[2], dj[0] * dj[0], dj[1] * dj[1], dj[2] * dj[2],
                                   dj[0] * dj[1], dj[1] * dj[2], dj[2] * dj[0]};
            double KB[3][30];
            for (int r = 0; r < 3; r++)
              for (int s2 = 0; s2 < 3; s2++)
                for (int l = 0; l < F; l++) KB[r][F * s2 + l] = Kij[3 * r + s2] * fj[l];
            for (int r = 0; r < 3; r++)
              for (int m = 0; m < F; m++) {
                const double fm = Bi[r][F * r + m];
                double* gr = g + (size_t)nm * (F * r + m);
                for (int c = 0; c < nm; c++) gr[c] += fm * KB[r][c];
              }
          }
        }
      }
      for (size_t t = 0; t < touched.size(); t++) {
        const int b = touched[t];
        const double* g = &G[nm2 * t];
        const double* Ra = &R[nm2 * a];
        const double* Rb = &R[nm2 * (size_t)b];
        const int kpa = (int)kc[a].size(), kqb = (int)kc[b].size();
        // Kc_ab = R_a^T g R_b in two products: T = g R_b (nm x kept of b), then R_a^T T
        for (int x = 0; x < nm; x++)
          for (int q = 0; q < kqb; q++) {
            double v = 0.0;
            for (int y = 0; y < nm; y++) v += g[nm * x + y] * Rb[nm * y + kc[b][q]];
            Tg[(size_t)nm * x + q] = v;
          }
        for (int p2 = 0; p2 < kpa; p2++)
          for (int q = 0; q < kqb; q++) {
            double v = 0.0;
            for (int x = 0; x < nm; x++) v += Ra[nm * x + kc[a][p2]] * Tg[(size_t)nm * x + q];
            Kc[(size_t)(first[a] + p2) * nk + first[b] + q] = v;
          }
        slot[b] = -1;
      }
    }
  }, 1);
  const clk::time_point t2 = clk::now();
  // Kc^-1 by Cholesky
  if (!cholesky_lower(Kc, nk)) return fail(SFEM_ERR_INVALID, "the coarse matrix is not positive definite");
  std::vector<double> Kinv;
  cholesky_inverse(Kc, nk, Kinv);
  // W = R Kc^-1 R^T in the modes' basis (nm n_agg square, rows padded to a multiple of 8)
  const int nc = (int)(nm * na), ld = (nc + 7) / 8 * 8;
  std::vector<float> W((size_t)nc * ld, 0.f);
  // per aggregate pair (a, b): T = Kinv_ab R_b^T (kept columns of a x nm), then W_ab = R_a T
  parallel_dynamic(na, 1, [&](int64_t a0, int64_t a1) {
    std::vector<double> T((size_t)nm * nm);
    for (int64_t a = a0; a < a1; a++) {
      const double* Ra = &R[nm2 * a];
      const int kpa = (int)kc[a].size();
      for (int64_t b = 0; b < na; b++) {
        const double* Rb = &R[nm2 * b];
        const int kqb = (int)kc[b].size();
        for (int p = 0; p < kpa; p++) {
          const double* Ki = &Kinv[(size_t)(first[a] + p) * nk + first[b]];
          for (int y = 0; y < nm; y++) {
            double v = 0.0;
            for (int q = 0; q < kqb; q++) v += Ki[q] * Rb[nm * y + kc[b][q]];
            T[(size_t)nm * p + y] = v;
          }
        }
        for (int x = 0; x < nm; x++) {
          float* Wr = &W[(size_t)(nm * a + x) * ld + nm * b];
          for (int y = 0; y < nm; y++) {
            double v = 0.0;
            for (int p = 0; p < kpa; p++) v += Ra[nm * x + kc[a][p]] * T[(size_t)nm * p + y];
            Wr[y] = (float)v;
          }
        }
      }
    }
  });
  // stored in FP16 (11-bit significand) times 2^k, k putting the largest magnitude in [2^13, 2^14): half
  // the bytes of the per-iteration product, relative rounding <= 2^-11 on every entry above 2^-14 / 2^k
  float wmax = 0.f;
  for (float v : W) wmax = std::max(wmax, std::fabs(v));
  const int wexp = wmax > 0.f ? 13 - std::ilogb(wmax) : 0;
  std::vector<__half> Wh(W.size());
  parallel_rows((int64_t)W.size(), [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; i++) Wh[i] = __float2half_rn(std::ldexp(W[i], wexp));
  });
  h->cs_w_inv_scale = std::ldexp(1.f, -wexp);
  const clk::time_point t3 = clk::now();
  // restriction runs: the blocks of the flexible-CG update's CTAs (coarse_block_start), split where
  // the aggregate changes and after kCoarseRun nodes; then every aggregate's runs in increasing order
  const int64_t N = h->N, g0a = (nbc + 3) & ~(int64_t)3, g0 = g0a < N ? g0a : N, ngrp = (N - g0) / 4;
  const int64_t nblk = std::max<int64_t>(1, (ngrp + 255) / 256);
  const int blk_off = (int)(g0 - nbc);
  std::vector<int32_t> rstart, rblk((size_t)nblk + 1, 0), ragg;
  for (int64_t b = 0; b < nblk; b++) {
    const int64_t i0 = coarse_block_start(b, nblk, blk_off, nf), i1 = coarse_block_start(b + 1, nblk, blk_off, nf);
    for (int64_t i = i0; i < i1; i++)
      if (i == i0 || aid[i] != aid[i - 1] || i - rstart.back() == kCoarseRun) {
        rstart.push_back((int32_t)i);
        ragg.push_back(aid[i]);
      }
    rblk[b + 1] = (int32_t)rstart.size();
  }
  const int64_t nrun = (int64_t)rstart.size();
  rstart.push_back((int32_t)nf);
  std::vector<int32_t> arptr((size_t)na + 1, 0), arun((size_t)nrun);
  for (int64_t k = 0; k < nrun; k++) arptr[ragg[k] + 1]++;
  for (int64_t a = 0; a < na; a++) arptr[a + 1] += arptr[a];
  {
    std::vector<int32_t> fill(arptr.begin(), arptr.end() - 1);
    for (int64_t k = 0; k < nrun; k++) arun[fill[ragg[k]]++] = (int32_t)k;
  }
  // device copies
  std::vector<float4> d4((size_t)nf);
  for (int64_t i = 0; i < nf; i++) d4[i] = make_float4((float)d[3 * i], (float)d[3 * i + 1], (float)d[3 * i + 2], 0.f);
  TRY(dalloc(&h->cs_aid, aid.size()));
  TRY(dalloc(&h->cs_d, d4.size()));
  TRY(dalloc(&h->cs_W, Wh.size()));
  TRY(dalloc(&h->cs_s, (size_t)ld));
  TRY(dalloc(&h->cs_y, (size_t)ld));
  TRY(dalloc(&h->cs_run_start, rstart.size()));
  TRY(dalloc(&h->cs_blk_run, rblk.size()));
  TRY(dalloc(&h->cs_agg_run_ptr, arptr.size()));
  TRY(dalloc(&h->cs_agg_run, std::max<size_t>(arun.size(), 1)));
  TRY(dalloc(&h->cs_runpart, std::max<size_t>((size_t)nm * nrun, 1)));
  CU(cudaMemcpyAsync(h->cs_aid, aid.data(), aid.size() * 4, cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->cs_d, d4.data(), d4.size() * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->cs_W, Wh.data(), Wh.size() * sizeof(__half), cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemsetAsync(h->cs_s, 0, (size_t)ld * 4, h->stream));
  CU(cudaMemsetAsync(h->cs_y, 0, (size_t)ld * 4, h->stream));
  CU(cudaMemcpyAsync(h->cs_run_start, rstart.data(), rstart.size() * 4, cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->cs_blk_run, rblk.data(), rblk.size() * 4, cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->cs_agg_run_ptr, arptr.data(), arptr.size() * 4, cudaMemcpyHostToDevice, h->stream));
  if (nrun > 0) CU(cudaMemcpyAsync(h->cs_agg_run, arun.data(), arun.size() * 4, cudaMemcpyHostToDevice, h->stream));
  h->cs_n_runs = (int)nrun;
  h->cs_n_blocks = (int)nblk;
  if (!h->cs_stream) CU(cudaStreamCreateWithFlags(&h->cs_stream, cudaStreamNonBlocking));
  if (!h->cs_fork) CU(cudaEventCreateWithFlags(&h->cs_fork, cudaEventDisableTiming));
  if (!h->cs_join) CU(cudaEventCreateWithFlags(&h->cs_join, cudaEventDisableTiming));
  h->cs_blk_off = blk_off;
  TRY(sync(h));
  h->cs_n_agg = (int)na;
  h->cs_ld = ld;
  h->cs_nk = nk;
  h->cs_nm = nm;
  h->cs_setup_s[0] = secs(t0, t1);
  h->cs_setup_s[1] = secs(t1, t2);
  h->cs_setup_s[2] = secs(t2, t3);
  h->cs_on = true;
  return SFEM_OK;
}

int sfem_coarse_info(sfem_handle* h, int32_t* n_agg, int32_t* n_coarse, double* seconds) {
  TRY(check_handle(h));
  if (n_agg) *n_agg = h->cs_on ? h->cs_n_agg : 0;
  if (n_coarse) *n_coarse = h->cs_on ? h->cs_nk : 0;
  if (seconds)
    for (int k = 0; k < 3; k++) seconds[k] = h->cs_on ? h->cs_setup_s[k] : 0.0;
  return SFEM_OK;
}

int sfem_coarse_apply(sfem_handle* h, const double* r, double* z) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!r || !z) return fail(SFEM_ERR_INVALID, "null");
  if (!h->cs_on) return fail(SFEM_ERR_INVALID, "no coarse space (sfem_set_coarse_space)");
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  TRY(alloc_ws(h, h->k32));
  KrylovWs<float>& w = h->k32;
  CU(cudaMemcpyAsync(h->tmp64 + o, r, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_convert<double, float>((int64_t)n, h->tmp64 + o, w.b + o, h->stream);
  CU(cudaMemsetAsync(w.q + o, 0, n * sizeof(float), h->stream));
  launch_coarse_apply(h->cv(), w.b + o, w.q + o, h->stream);
  launch_convert<float, double>((int64_t)n, w.q + o, h->tmp64 + o, h->stream);
  CU(cudaMemcpyAsync(z, h->tmp64 + o, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int sfem_set_newton_trace(sfem_handle* h, double* trace, int32_t cap, int32_t* count) {
  TRY(check_handle(h));
  if (trace && (cap < 0 || !count)) return fail(SFEM_ERR_INVALID, "trace needs a capacity and a count");
  h->ls_trace = trace;
  h->ls_trace_cap = trace ? cap : 0;
  h->ls_trace_count = trace ? count : nullptr;
  if (count) *count = 0;
  return SFEM_OK;
}

int sfem_set_operator_memory_limit(sfem_handle* h, int64_t bytes) {
  TRY(check_handle(h));
  if (bytes < 0) return fail(SFEM_ERR_INVALID, "the limit is a byte count (0: no limit)");
  h->sell_limit = bytes;
  h->sell_oom = false;
  return SFEM_OK;
}

int sfem_set_residual_arithmetic(sfem_handle* h, int32_t mode) {
  TRY(check_handle(h));
  if (mode != SFEM_RESIDUAL_FP64 && mode != SFEM_RESIDUAL_TWO_TERM)
    return fail(SFEM_ERR_INVALID, "residual arithmetic %d (0: FP64, 1: two-term FP32)", (int)mode);
  h->resid_arith = mode;
  return SFEM_OK;
}

int sfem_operator_info(sfem_handle* h, int64_t* bytes, int32_t* fallback) {
  TRY(check_handle(h));
  if (bytes) *bytes = h->sell_bytes;
  if (fallback) *fallback = h->sell_oom ? 1 : 0;
  return SFEM_OK;
}

int sfem_tangent_nnz(sfem_handle* h, int64_t* nnzb) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!nnzb) return fail(SFEM_ERR_INVALID, "null");
  TRY(bsr_structure(h));
  *nnzb = h->bsr_nnzb;
  return SFEM_OK;
}

int sfem_assemble_tangent(sfem_handle* h, int32_t* rowptr, int32_t* colidx, double* vals) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!rowptr || !colidx || !vals) return fail(SFEM_ERR_INVALID, "null");
  TRY(bsr_assemble(h));
  CU(cudaMemcpyAsync(rowptr, h->bsr_rowptr, ((size_t)h->nf + 1) * 4, cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(colidx, h->bsr_col, (size_t)h->bsr_nnzb * 4, cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(vals, h->bsr_vals, 9 * (size_t)h->bsr_nnzb * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int sfem_tangent_matvec(sfem_handle* h, const double* d_free, double* out_free) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!d_free || !out_free) return fail(SFEM_ERR_INVALID, "null");
  TRY(bsr_assemble(h));
  const size_t n = 3 * (size_t)h->nf;
  CU(cudaMemcpyAsync(h->tmp64, d_free, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_bsr_spmv(h->nf, h->bsr_rowptr, h->bsr_col, h->bsr_vals, h->tmp64, h->tmp64b, h->stream);
  CU(cudaMemcpyAsync(out_free, h->tmp64b, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

// ---- dynamics (FemPhysicsMatrixFree::Step :297-324, SubStep :371-387, Solve :589-597) ----
int sfem_set_time_step(sfem_handle* h, double dt) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!(dt >= 0.0) || !std::isfinite(dt)) return fail(SFEM_ERR_INVALID, "time step must be finite and >= 0");
  h->dt = dt;
  if (dt == 0.0) return SFEM_OK;
  if (!h->pm64) TRY(dalloc(&h->pm64, (size_t)h->n_slots));
  if (h->precision == SFEM_FP32 && !h->pm32) TRY(dalloc(&h->pm32, (size_t)h->n_slots));
  const double inv_h2 = 1.0 / (dt * dt);
  launch_patch_mass<double>(h->n_slots, h->nbc, h->pnode, h->bidx, h->pb(), h->mass, inv_h2, h->pm64, h->stream);
  if (h->pm32)
    launch_patch_mass<float>(h->n_slots, h->nbc, h->pnode, h->bidx, h->pb(), h->mass, inv_h2, h->pm32, h->stream);
  return sync(h);
}

int sfem_get_time_step(sfem_handle* h, double* dt) {
  TRY(check_handle(h));
  if (!dt) return fail(SFEM_ERR_INVALID, "null");
  *dt = h->dt;
  return SFEM_OK;
}

static int node_vec_io(sfem_handle* h, double* dev, const double* in, double* out) {
  const size_t N3 = 3 * (size_t)h->N;
  if (in) {
    CU(cudaMemcpyAsync(h->tmp64b, in, N3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_nodes_in(h->N, h->dmap, h->tmp64b, nullptr, h->nbc, dev, h->stream);  // fixed nodes do not move
    return sync(h);
  }
  launch_nodes_out(h->N, h->dmap, dev, nullptr, h->tmp64, h->stream);
  CU(cudaMemcpyAsync(out, h->tmp64, N3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int sfem_set_velocities(sfem_handle* h, const double* vel) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!vel) return fail(SFEM_ERR_INVALID, "null");
  return node_vec_io(h, h->vel, vel, nullptr);
}

int sfem_get_velocities(sfem_handle* h, double* vel) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!vel) return fail(SFEM_ERR_INVALID, "null");
  return node_vec_io(h, h->vel, nullptr, vel);
}

int sfem_begin_step(sfem_handle* h) {
  TRY(check_handle(h));
  TRY(set_device(h));
  CU(cudaMemcpyAsync(h->ustart, h->u, 3 * (size_t)h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  return sync(h);
}

int sfem_step(sfem_handle* h, double dt, int32_t sim_type, int32_t substeps, const sfem_newton_opts* opts,
              sfem_newton_stats* stats) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (substeps < 1) return fail(SFEM_ERR_INVALID, "substeps must be >= 1");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(SFEM_ERR_INVALID, "dt must be finite and > 0");
  const double hs = dt / substeps;
  if (stats) memset(stats, 0, sizeof(*stats));
  if (sim_type == SFEM_SIM_EXPLICIT) {
    // internal forces only (no gravity scaling, no loads), then symplectic Euler with h g
    const double ff = h->ff;
    const double dt_keep = h->dt;
    for (int i = 0; i < substeps; i++) {
      CU(cudaMemsetAsync(h->ninv, 0, sizeof(int), h->stream));
      element_pass<double>(h, MODE_FORCE, h->u, nullptr, h->fe, nullptr, h->ninv, nullptr);
      h->dt = 0.0;
      launch_gather_force(h->nbc, h->N, h->csr(), h->fe, h->mass, h->fext, h->grav, 0.0, h->r64, h->red(), nullptr,
                          h->stream);
      h->dt = dt_keep;
      launch_explicit_substep(h->nbc, h->N, h->r64, h->mass, h->grav, hs, h->vel, h->u, h->stream);
    }
    h->ff = ff;
    CU(cudaGetLastError());
    return sync(h);
  }
  if (sim_type != SFEM_SIM_IMPLICIT) return fail(SFEM_ERR_INVALID, "sim_type is SFEM_SIM_EXPLICIT or SFEM_SIM_IMPLICIT");
  if (!opts) return fail(SFEM_ERR_INVALID, "opts is null");
  // positions at the start of the step (the reference overwrites pos0 once per Step)
  TRY(sfem_begin_step(h));
  TRY(sfem_set_time_step(h, hs));
  h->ff = 1.0;
  int worst = SFEM_OK;
  for (int i = 0; i < substeps; i++) {
    sfem_newton_stats st{};
    const int rc = sfem_newton_solve(h, opts, &st);
    if (rc < 0) return rc;
    if (rc > worst) worst = rc;
    launch_velocity_update(h->nbc, h->N, h->u, h->ustart, 1.0 / hs, h->vel, h->stream);
    if (stats) {
      stats->newton_iters += st.newton_iters;
      stats->cg_iters += st.cg_iters;
      stats->line_search_cuts += st.line_search_cuts;
      stats->status = st.status > stats->status ? st.status : stats->status;
      stats->r0 = i == 0 ? st.r0 : stats->r0;
      stats->rel_res = st.rel_res;
      stats->seconds += st.seconds;
    }
  }
  TRY(sync(h));
  return worst;
}

int sfem_get_positions(sfem_handle* h, double* pos) {
  TRY(check_handle(h));
  TRY(set_device(h));
  launch_nodes_out(h->N, h->dmap, h->x0, h->u, h->tmp64, h->stream);
  CU(cudaMemcpyAsync(pos, h->tmp64, 3 * (size_t)h->N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int sfem_set_positions(sfem_handle* h, const double* pos) {
  TRY(check_handle(h));
  TRY(set_device(h));
  CU(cudaMemcpyAsync(h->tmp64b, pos, 3 * (size_t)h->N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_nodes_in(h->N, h->dmap, h->tmp64b, h->x0, 0, h->u, h->stream);
  return sync(h);
}

int sfem_get_free_positions(sfem_handle* h, double* pos_free) {
  TRY(check_handle(h));
  TRY(set_device(h));
  TRY(sfem_get_free_positions_dev(h, h->tmp64));
  CU(cudaMemcpyAsync(pos_free, h->tmp64, 3 * (size_t)h->nf * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int sfem_set_free_positions(sfem_handle* h, const double* pos_free) {
  TRY(check_handle(h));
  TRY(set_device(h));
  CU(cudaMemcpyAsync(h->tmp64b, pos_free, 3 * (size_t)h->nf * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TRY(sfem_set_free_positions_dev(h, h->tmp64b));
  return sync(h);
}

int sfem_get_free_positions_dev(sfem_handle* h, double* pos_dev) {
  TRY(check_handle(h));
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  // pos = x0 + u over the free block
  launch_axpy_state<double>((int64_t)n, 1.0, h->u + o, h->x0 + o, pos_dev, h->stream);
  CU(cudaGetLastError());
  return SFEM_OK;
}

int sfem_set_free_positions_dev(sfem_handle* h, const double* pos_dev) {
  TRY(check_handle(h));
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  // u = pos - x0 over the free block
  launch_axpy_state<double>((int64_t)n, -1.0, h->x0 + o, pos_dev, h->u + o, h->stream);
  CU(cudaGetLastError());
  return SFEM_OK;
}

int sfem_set_lame_params(sfem_handle* h, double mu, double lambda) {
  TRY(check_handle(h));
  h->mu = mu;
  h->lambda = lambda;
  // SetLameParams, Include/FemPhysicsBase.h:106-114
  h->young = mu * (3 * lambda + 2 * mu) / (mu + lambda);
  h->poisson = 0.5 * lambda / (mu + lambda);
  return SFEM_OK;
}

int sfem_set_force_fraction(sfem_handle* h, double f) {
  TRY(check_handle(h));
  h->ff = f;
  return SFEM_OK;
}

int sfem_set_element_youngs(sfem_handle* h, const double* young_e) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!young_e) {
    h->has_scale = false;
    return SFEM_OK;
  }
  if (!h->young_e) {
    TRY(dalloc(&h->young_e, (size_t)h->E));
    TRY(dalloc(&h->scale64, (size_t)h->E));
    TRY(dalloc(&h->scale32, (size_t)h->E));
  }
  CU(cudaMemcpyAsync(h->etmp, young_e, (size_t)h->E * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TRY(sfem_set_element_youngs_dev(h, h->etmp));
  return sync(h);
}

int sfem_set_element_youngs_dev(sfem_handle* h, const double* young_e_dev) {
  TRY(check_handle(h));
  if (!h->young_e) {
    TRY(dalloc(&h->young_e, (size_t)h->E));
    TRY(dalloc(&h->scale64, (size_t)h->E));
    TRY(dalloc(&h->scale32, (size_t)h->E));
  }
  // caller's element order -> patch order
  launch_permute(h->E, h->perm, young_e_dev, h->young_e, h->stream);
  launch_scale_copy(h->E, 1.0 / h->young, h->young_e, h->scale64, h->stream);
  launch_convert<double, float>(h->E, h->scale64, h->scale32, h->stream);
  h->has_scale = true;
  h->has_scale_la = false;
  CU(cudaGetLastError());
  return SFEM_OK;
}

int sfem_set_element_lame(sfem_handle* h, const double* mu_e, const double* lambda_e) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!mu_e || !lambda_e) {
    h->has_scale = h->has_scale_la = false;
    return SFEM_OK;
  }
  const size_t E = (size_t)h->E;
  if (!h->young_e) {
    TRY(dalloc(&h->young_e, E));
    TRY(dalloc(&h->scale64, E));
    TRY(dalloc(&h->scale32, E));
  }
  if (!h->scale_la64) {
    TRY(dalloc(&h->scale_la64, E));
    TRY(dalloc(&h->scale_la32, E));
  }
  std::vector<double> sm(E), sl(E);
  for (size_t k = 0; k < E; k++) {
    const int32_t e = h->perm_h[k];
    sm[k] = mu_e[e] / h->mu;
    sl[k] = lambda_e[e] / h->lambda;
  }
  CU(cudaMemcpyAsync(h->scale64, sm.data(), E * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->scale_la64, sl.data(), E * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_convert<double, float>(h->E, h->scale64, h->scale32, h->stream);
  launch_convert<double, float>(h->E, h->scale_la64, h->scale_la32, h->stream);
  h->has_scale = true;
  h->has_scale_la = true;
  return sync(h);
}

int sfem_set_pressure_surface(sfem_handle* h, const int32_t* tris, int64_t n_tris, double pressure) {
  TRY(check_handle(h));
  TRY(set_device(h));
  int32_t** bufs[] = {&h->tri, &h->tptr, &h->tent};
  for (int32_t** b : bufs)
    if (*b) {
      cudaFree(*b);
      *b = nullptr;
    }
  if (h->ptf) cudaFree(h->ptf);
  h->ptf = nullptr;
  h->n_tris = 0;
  h->pressure = pressure;
  if (!tris || n_tris <= 0) return SFEM_OK;
  std::vector<int32_t> t(3 * (size_t)n_tris), ptr((size_t)h->N + 1, 0), ent(3 * (size_t)n_tris);
  for (int64_t i = 0; i < 3 * n_tris; i++) {
    if (tris[i] < 0 || tris[i] >= h->N) return fail(SFEM_ERR_INVALID, "pressure triangle index out of range");
    t[i] = h->map[tris[i]];
    ptr[t[i] + 1]++;
  }
  for (int64_t i = 0; i < h->N; i++) ptr[i + 1] += ptr[i];
  {
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int64_t i = 0; i < 3 * n_tris; i++) ent[fill[t[i]]++] = (int32_t)(i / 3);
  }
  TRY(dalloc(&h->tri, t.size()));
  TRY(dalloc(&h->tptr, ptr.size()));
  TRY(dalloc(&h->tent, ent.size()));
  TRY(dalloc(&h->ptf, 3 * (size_t)n_tris));
  CU(cudaMemcpyAsync(h->tri, t.data(), t.size() * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->tptr, ptr.data(), ptr.size() * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->tent, ent.data(), ent.size() * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  h->n_tris = n_tris;
  return sync(h);
}

int sfem_set_instances(sfem_handle* h, int32_t k, const int64_t* node_offsets) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (k <= 0 || !node_offsets) {
    h->n_inst = 0;
    return SFEM_OK;
  }
  if (node_offsets[0] != 0 || node_offsets[k] != h->N) return fail(SFEM_ERR_INVALID, "instance offsets must span [0, N)");
  std::vector<int64_t> seg(k + 1, 0);
  for (int q = 0; q < k; q++) {
    if (node_offsets[q + 1] < node_offsets[q]) return fail(SFEM_ERR_INVALID, "instance offsets must increase");
    int64_t nfree = 0;
    for (int64_t i = node_offsets[q]; i < node_offsets[q + 1]; i++) nfree += h->map[i] >= h->nbc ? 1 : 0;
    seg[q + 1] = seg[q] + 3 * nfree;
  }
  // free nodes keep their relative order, so each instance is one contiguous free-DOF segment
  for (int q = 0; q < k; q++)
    for (int64_t i = node_offsets[q]; i < node_offsets[q + 1]; i++)
      if (h->map[i] >= h->nbc && (3 * (h->map[i] - h->nbc) < seg[q] || 3 * (h->map[i] - h->nbc) >= seg[q + 1]))
        return fail(SFEM_ERR_INVALID, "instance nodes are not contiguous");
  if (h->inst_seg) cudaFree(h->inst_seg);
  if (h->inst_active) cudaFree(h->inst_active);
  if (h->inst_norm) cudaFree(h->inst_norm);
  h->inst_seg = nullptr;
  h->inst_active = nullptr;
  h->inst_norm = nullptr;
  TRY(dalloc(&h->inst_seg, (size_t)k + 1));
  TRY(dalloc(&h->inst_active, (size_t)k));
  TRY(dalloc(&h->inst_norm, (size_t)k));
  CU(cudaMemcpyAsync(h->inst_seg, seg.data(), seg.size() * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
  std::vector<int32_t> act(k, 1);
  CU(cudaMemcpyAsync(h->inst_active, act.data(), k * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  h->n_inst = k;
  h->inst_rel.assign(k, 1.0);
  h->inst_its.assign(k, 0);
  // the persistent per-instance PCG: each element's instance (from its first corner), free-node tiles
  TRY(sync(h));
  batch_release(h);
  {
    std::vector<int32_t> inst_of((size_t)h->N, 0);  // reshuffled node -> instance
    for (int q = 0; q < k; q++)
      for (int64_t i = node_offsets[q]; i < node_offsets[q + 1]; i++) inst_of[h->map[i]] = q;
    std::vector<int4> tt((size_t)h->E);
    CU(cudaMemcpyAsync(tt.data(), h->tets, tt.size() * sizeof(int4), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    std::vector<int32_t> einst((size_t)h->E);
    for (int64_t e = 0; e < h->E; e++) einst[e] = inst_of[tt[e].x];
    std::vector<int32_t> tnode, tcnt, tinst, itile(k + 1, 0);
    for (int q = 0; q < k; q++) {
      const int64_t a = seg[q] / 3, b = seg[q + 1] / 3;
      for (int64_t f = a; f < b; f += 32) {
        tnode.push_back((int32_t)f);
        tcnt.push_back((int32_t)std::min<int64_t>(32, b - f));
        tinst.push_back(q);
      }
      itile[q + 1] = (int32_t)tnode.size();
    }
    const int nt = (int)tnode.size();
    TRY(dalloc(&h->bt_einst, (size_t)h->E));
    TRY(dalloc(&h->bt_tile_node, std::max(nt, 1)));
    TRY(dalloc(&h->bt_tile_cnt, std::max(nt, 1)));
    TRY(dalloc(&h->bt_tile_inst, std::max(nt, 1)));
    TRY(dalloc(&h->bt_inst_tile, (size_t)k + 1));
    TRY(dalloc(&h->bt_part, 3 * (size_t)std::max(nt, 1)));
    TRY(dalloc(&h->bt_rz, 2 * (size_t)k));
    TRY(dalloc(&h->bt_tol2bb, (size_t)k));
    TRY(dalloc(&h->bt_rr, (size_t)k));
    TRY(dalloc(&h->bt_done, 3 * (size_t)k));
    TRY(dalloc(&h->bt_iters, (size_t)k));
    TRY(dalloc(&h->bt_err, 1));
    TRY(dalloc(&h->bt_bar, 4));
    CU(cudaMemcpyAsync(h->bt_einst, einst.data(), einst.size() * 4, cudaMemcpyHostToDevice, h->stream));
    if (nt > 0) {
      CU(cudaMemcpyAsync(h->bt_tile_node, tnode.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, h->stream));
      CU(cudaMemcpyAsync(h->bt_tile_cnt, tcnt.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, h->stream));
      CU(cudaMemcpyAsync(h->bt_tile_inst, tinst.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, h->stream));
    }
    CU(cudaMemcpyAsync(h->bt_inst_tile, itile.data(), itile.size() * 4, cudaMemcpyHostToDevice, h->stream));
    h->bt_ntiles = nt;
  }
  return sync(h);
}

int sfem_set_batched_pcg(sfem_handle* h, int32_t mode) {
  TRY(check_handle(h));
  if (mode != 0 && mode != 1) return fail(SFEM_ERR_INVALID, "mode is 0 (one recurrence) or 1 (per instance)");
  h->bt_mode = mode;
  return SFEM_OK;
}

int sfem_set_device_wait(sfem_handle* h, int64_t limit, int32_t test) {
  TRY(check_handle(h));
  if (limit < 1) return fail(SFEM_ERR_INVALID, "the wait limit is a positive poll count");
  h->bt_wait_limit = limit;
  h->bt_wait_test = test ? 1 : 0;
  return SFEM_OK;
}

int sfem_instance_pcg_stats(const sfem_handle* h, int32_t* iters, int32_t* status, double* rel_res) {
  TRY(check_handle(h));
  for (size_t q = 0; q < h->bt_iters_h.size(); q++) {
    if (iters) iters[q] = h->bt_iters_h[q];
    if (status) status[q] = h->bt_status_h[q];
    if (rel_res) rel_res[q] = h->bt_bb_h[q] > 0 ? std::sqrt(h->bt_rr_h[q] / h->bt_bb_h[q]) : 0.0;
  }
  return SFEM_OK;
}

int sfem_instance_stats(const sfem_handle* h, double* rel_res, int32_t* newton_iters) {
  TRY(check_handle(h));
  for (int q = 0; q < h->n_inst; q++) {
    if (rel_res) rel_res[q] = h->inst_rel[q];
    if (newton_iters) newton_iters[q] = h->inst_its[q];
  }
  return SFEM_OK;
}

int sfem_set_nodal_loads(sfem_handle* h, const double* f) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!f) {
    CU(cudaMemsetAsync(h->fext, 0, 3 * (size_t)h->N * sizeof(double), h->stream));
    return sync(h);
  }
  return upload_nodes(h, f, h->fext);
}

int sfem_set_nodal_loads_free_dev(sfem_handle* h, const double* f_free_dev) {
  TRY(check_handle(h));
  CU(cudaMemcpyAsync(h->fext + 3 * h->nbc, f_free_dev, 3 * (size_t)h->nf * sizeof(double), cudaMemcpyDeviceToDevice,
                     h->stream));
  return SFEM_OK;
}

int sfem_compute_gradients_dev(sfem_handle* h, double* r_dev) {
  TRY(check_handle(h));
  double rn;
  TRY(residual(h, &rn, nullptr));
  CU(cudaMemcpyAsync(r_dev, h->r64 + 3 * h->nbc, 3 * (size_t)h->nf * sizeof(double), cudaMemcpyDeviceToDevice,
                     h->stream));
  return SFEM_OK;
}

int sfem_compute_gradients(sfem_handle* h, double* r, double* norm) {
  TRY(check_handle(h));
  TRY(set_device(h));
  double rn;
  TRY(residual(h, &rn, nullptr));
  if (r)
    CU(cudaMemcpyAsync(r, h->r64 + 3 * h->nbc, 3 * (size_t)h->nf * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  if (norm) *norm = rn;
  return SFEM_OK;
}

int sfem_matvec_dev(sfem_handle* h, const double* d_dev, double* Kd_dev) {
  TRY(check_handle(h));
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  // direction with zero fixed-node block
  CU(cudaMemsetAsync(h->tmp64, 0, o * sizeof(double), h->stream));
  CU(cudaMemcpyAsync(h->tmp64 + o, d_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  hvp<double>(h, h->u, h->tmp64, h->tmp64b, nullptr);
  CU(cudaMemcpyAsync(Kd_dev, h->tmp64b + o, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CU(cudaGetLastError());
  return SFEM_OK;
}

int sfem_matvec(sfem_handle* h, const double* d, double* Kd) {
  TRY(check_handle(h));
  TRY(set_device(h));
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  double* dbuf = h->k64.b;  // scratch
  CU(cudaMemcpyAsync(dbuf + o, d, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TRY(sfem_matvec_dev(h, dbuf + o, h->k64.x + o));
  CU(cudaMemcpyAsync(Kd, h->k64.x + o, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int sfem_dot(sfem_handle* h, const double* a, const double* b, double* out) {
  TRY(check_handle(h));
  TRY(set_device(h));
  const size_t n = 3 * (size_t)h->nf;
  CU(cudaMemcpyAsync(h->tmp64, a, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(h->tmp64b, b, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_dot((int64_t)n, h->tmp64, h->tmp64b, h->red(), h->dres, h->stream);
  CU(cudaMemcpyAsync(h->dres_h, h->dres, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  *out = h->dres_h[0];
  return SFEM_OK;
}

int sfem_jacobi_diagonal(sfem_handle* h, double* diag) {
  TRY(check_handle(h));
  TRY(set_device(h));
  TRY(jacobi<double>(h, h->k64.dinv, h->tmp64));
  CU(cudaMemcpyAsync(diag, h->tmp64 + 3 * h->nbc, 3 * (size_t)h->nf * sizeof(double), cudaMemcpyDeviceToHost,
                     h->stream));
  return sync(h);
}

int sfem_energy(sfem_handle* h, double* elastic, double* total) {
  TRY(check_handle(h));
  TRY(set_device(h));
  element_pass<double>(h, MODE_ENERGY, h->u, nullptr, h->fe, h->dres, nullptr, nullptr);
  const DynView dv = h->dyn();
  launch_potential(h->nbc, h->N, h->x0, h->u, h->mass, h->fext, h->grav, h->ff, h->red(), h->dres + 1, h->stream,
                   h->dt > 0 ? &dv : nullptr);
  CU(cudaMemcpyAsync(h->dres_h, h->dres, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  if (elastic) *elastic = h->dres_h[0];
  if (total) *total = h->dres_h[0] + h->dres_h[1];
  return SFEM_OK;
}

int sfem_count_inverted(sfem_handle* h, int64_t* count) {
  TRY(check_handle(h));
  TRY(set_device(h));
  int n = 0;
  TRY(residual(h, nullptr, &n));
  *count = n;
  return SFEM_OK;
}

int sfem_element_stress(sfem_handle* h, double* P) {
  TRY(check_handle(h));
  TRY(set_device(h));
  element_pass<double>(h, MODE_STRESS, h->u, nullptr, h->fe, nullptr, nullptr, nullptr);
  std::vector<double> tmp(12 * (size_t)h->E);
  CU(cudaMemcpyAsync(tmp.data(), h->fe, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  for (int64_t k = 0; k < h->E; k++) memcpy(P + 9 * (size_t)h->perm_h[k], &tmp[12 * (size_t)k], 9 * sizeof(double));
  return SFEM_OK;
}

int sfem_force_param_grads(sfem_handle* h, double* gmu, double* glambda, double* grho) {
  TRY(check_handle(h));
  TRY(set_device(h));
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  const int modes[3] = {MODE_PMU, MODE_PLAMBDA, MODE_NODALVOL};
  double* outs[3] = {gmu, glambda, grho};
  std::vector<double> nv(n);
  for (int m = 0; m < 3; m++) {
    element_pass<double>(h, modes[m], h->u, nullptr, h->fe, nullptr, nullptr, nullptr);
    launch_gather_diag<double>(h->nbc, h->N, h->csr(), h->fe, nullptr, h->tmp64, h->stream);
    CU(cudaMemcpyAsync(m < 2 ? outs[m] : nv.data(), h->tmp64 + o, n * sizeof(double), cudaMemcpyDeviceToHost,
                       h->stream));
    TRY(sync(h));
  }
  // d f / d rho = (nodal volume) * g: the nodal volume sits in every component slot 0 of the gather
  for (size_t i = 0; i < (size_t)h->nf; i++)
    for (int c = 0; c < 3; c++) grho[3 * i + c] = nv[3 * i] * h->grav[c];
  return SFEM_OK;
}

// stats of a batched solve: the largest instance iteration count, the largest instance relative
// residual, status 1 if any instance reached the iteration cap
static sfem_pcg_stats batched_stats(const sfem_handle* h, int its) {
  sfem_pcg_stats s{};
  s.iters = its;
  for (size_t q = 0; q < h->bt_iters_h.size(); q++) {
    const double rel = h->bt_bb_h[q] > 0 ? std::sqrt(h->bt_rr_h[q] / h->bt_bb_h[q]) : 0.0;
    s.rel_res = std::max(s.rel_res, rel);
    if (h->bt_status_h[q] == 3) s.status = 1;
  }
  return s;
}

int sfem_pcg(sfem_handle* h, const double* b, double* x, const sfem_pcg_opts* opts, sfem_pcg_stats* stats) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!b || !x || !opts) return fail(SFEM_ERR_INVALID, "null argument");
  if (opts->precond == SFEM_PC_LEARNED) return fail(SFEM_ERR_INVALID, "learned preconditioner: use sfem_newton_solve");
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  const bool pc = opts->precond == SFEM_PC_JACOBI;
  int st = 0;
  if (h->precision == SFEM_FP64) {
    KrylovWs<double>& w = h->k64;
    OperatorScope ops(h);
    TRY(ops.st);
    CU(cudaMemcpyAsync(w.b + o, b, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (pc) TRY(jacobi<double>(h, w.dinv, nullptr));
    int its = 0;
    const int bst = batched_pcg<double>(h, h->u, w.b, w, pc ? w.dinv : w.ones, opts->rel_tol, opts->max_iters, &its);
    if (bst < 0) return bst;
    if (bst == 0 && stats) *stats = batched_stats(h, its);
    if (bst != 0)
      st = pcg_device<double>(h, h->u, w.b, w.x, pc ? w.dinv : nullptr, opts->rel_tol, opts->max_iters,
                              opts->check_every, stats);
    if (st == SFEM_NEGATIVE_CURVATURE) return SFEM_ERR_BREAKDOWN;
    if (st < 0) return st;
    CU(cudaMemcpyAsync(x, w.x + o, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  } else {
    KrylovWs<float>& w = h->k32;
    OperatorScope ops(h);
    TRY(ops.st);
    CU(cudaMemcpyAsync(h->tmp64 + o, b, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_convert<double, float>((int64_t)n, h->tmp64 + o, w.b + o, h->stream);
    const float* u32 = disp<float>(h);
    if (pc) TRY(jacobi<float>(h, w.dinv, nullptr));
    int its = 0;
    const int bst = batched_pcg<float>(h, u32, w.b, w, pc ? w.dinv : w.ones, opts->rel_tol, opts->max_iters, &its);
    if (bst < 0) return bst;
    if (bst == 0 && stats) *stats = batched_stats(h, its);
    if (bst != 0)
      st = pcg_device<float>(h, u32, w.b, w.x, pc ? w.dinv : nullptr, opts->rel_tol, opts->max_iters,
                             opts->check_every, stats);
    if (st == SFEM_NEGATIVE_CURVATURE) return SFEM_ERR_BREAKDOWN;
    if (st < 0) return st;
    launch_convert<float, double>((int64_t)n, w.x + o, h->tmp64 + o, h->stream);
    CU(cudaMemcpyAsync(x, h->tmp64 + o, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  }
  TRY(sync(h));
  return st;
}

}  // extern "C"

// -----------------------------------------------------------------------------
// Newton
// -----------------------------------------------------------------------------
int sfem_gnn_inner_solve(sfem_handle* h, double eta, int max_cg, int* its);

namespace {

// one inner solve K dx = r64 at the current state, in the handle's precision;
// the step ends up in h->tmp64 (FP64, full length).
void batch_release(sfem_handle* h) {
  void* bufs[] = {h->bt_einst, h->bt_tile_node, h->bt_tile_cnt, h->bt_tile_inst, h->bt_inst_tile, h->bt_part,
                  h->bt_rz, h->bt_tol2bb, h->bt_rr, h->bt_done, h->bt_iters, h->bt_err, h->bt_bar};
  for (void* b : bufs)
    if (b) cudaFree(b);
  h->bt_einst = h->bt_tile_node = h->bt_tile_cnt = h->bt_tile_inst = h->bt_inst_tile = nullptr;
  h->bt_part = h->bt_rz = h->bt_tol2bb = h->bt_rr = nullptr;
  h->bt_done = h->bt_iters = h->bt_err = nullptr;
  h->bt_bar = nullptr;
  h->bt_ntiles = 0;
}

void coarse_release(sfem_handle* h) {
  void* bufs[] = {h->cs_aid,       h->cs_d,          h->cs_W,         h->cs_s,      h->cs_y,
                  h->cs_run_start, h->cs_blk_run,    h->cs_agg_run_ptr, h->cs_agg_run, h->cs_runpart};
  for (void* b : bufs)
    if (b) cudaFree(b);
  h->cs_aid = nullptr;
  h->cs_d = nullptr;
  h->cs_W = nullptr;
  h->cs_w_inv_scale = 1.f;
  h->cs_s = h->cs_y = nullptr;
  h->cs_run_start = h->cs_blk_run = h->cs_agg_run_ptr = h->cs_agg_run = nullptr;
  h->cs_runpart = nullptr;
  h->cs_n_runs = h->cs_n_blocks = h->cs_blk_off = 0;
  h->cs_on = false;
  h->cs_n_agg = h->cs_ld = 0;
}

// The instances' PCG solves of K x = rhs, each with its own recurrence and tolerance, in one
// persistent launch.  *its = the largest instance iteration count.  Returns 1 when the handle does
// not take this path (no instances, mode 0, or a material outside 0, 1, 3).
template <typename T>
int batched_pcg(sfem_handle* h, const T* u, const T* rhs, KrylovWs<T>& w, const T* dinv, double tol, int max_it,
                int* its) {
  const int mat = mat_id(h);
  if (h->n_inst == 0 || h->bt_mode == 0 || !(mat == 0 || mat == 1 || mat == 3)) return 1;
  const int K = h->n_inst;
  CU(cudaMemsetAsync(h->bt_bar, 0, 4 * sizeof(unsigned), h->stream));
  CU(cudaMemsetAsync(h->bt_err, 0, sizeof(int32_t), h->stream));
  BatchPcg b{};
  b.K = K;
  b.n_tiles = h->bt_ntiles;
  b.nbc = h->nbc;
  b.N = h->N;
  b.einst = h->bt_einst;
  b.tile_node = h->bt_tile_node;
  b.tile_cnt = h->bt_tile_cnt;
  b.tile_inst = h->bt_tile_inst;
  b.inst_tile = h->bt_inst_tile;
  b.part = h->bt_part;
  b.rz = h->bt_rz;
  b.tol2bb = h->bt_tol2bb;
  b.done = h->bt_done;
  b.iters = h->bt_iters;
  b.rr = h->bt_rr;
  b.bar = h->bt_bar;
  b.err = h->bt_err;
  b.tol = tol;
  b.max_it = max_it;
  b.wait_limit = h->bt_wait_limit;
  b.wait_test = h->bt_wait_test;
  ElemView<T> ev;
  if constexpr (std::is_same<T, float>::value)
    ev = h->ev32();
  else
    ev = h->ev64();
  const int lst = launch_batched_pcg<T>(mat, ev, h->csr(), b, u, rhs, w.x, w.r, w.p2, w.p, w.q, dinv,
                                        reinterpret_cast<T*>(h->fe), h->stream);
  if (lst == -2) return fail(SFEM_ERR_CUDA, "cooperative launch not available on this device");
  if (lst != 0) return fail(SFEM_ERR_CUDA, "batched PCG launch failed: %s", cudaGetErrorString(cudaGetLastError()));
  int32_t err = 0;
  h->bt_iters_h.assign(K, 0);
  h->bt_status_h.assign(K, 0);
  h->bt_rr_h.assign(K, 0.0);
  h->bt_bb_h.assign(K, 0.0);
  std::vector<double> t2((size_t)K);
  CU(cudaMemcpyAsync(&err, h->bt_err, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(h->bt_iters_h.data(), h->bt_iters, K * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(h->bt_status_h.data(), h->bt_done + 2 * K, K * sizeof(int32_t), cudaMemcpyDeviceToHost,
                     h->stream));
  CU(cudaMemcpyAsync(h->bt_rr_h.data(), h->bt_rr, K * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CU(cudaMemcpyAsync(t2.data(), h->bt_tol2bb, K * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  for (int q = 0; q < K; q++) h->bt_bb_h[q] = tol > 0 ? t2[q] / (tol * tol) : 0.0;
  if (err != 0)
    return fail(SFEM_ERR_TIMEOUT, "a device wait of the batched PCG gave up after %lld polls%s", h->bt_wait_limit,
                err == 2 ? " (wait self-test)" : "");
  int mx = 0;
  for (int q = 0; q < K; q++) {
    mx = std::max(mx, h->bt_iters_h[q]);
    if (h->bt_status_h[q] == 4) return fail(SFEM_ERR_NAN, "non-finite value in the Krylov recurrence of instance %d", q);
  }
  *its = mx;
  return 0;
}

int inner_solve(sfem_handle* h, double eta, int max_cg, int precond, int* its) {
  if (precond == SFEM_PC_LEARNED) return sfem_gnn_inner_solve(h, eta, max_cg, its);
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  const bool pc = precond == SFEM_PC_JACOBI;
  sfem_pcg_stats ps{};
  int st;
  const bool masked = h->n_inst > 0;
  if (masked) launch_segment_mask<double>(h->n_inst, h->inst_seg, h->inst_active, h->r64 + o, h->stream);
  if (h->precision == SFEM_FP64) {
    KrylovWs<double>& w = h->k64;
    OperatorScope ops(h);
    TRY(ops.st);
    if (pc) TRY(jacobi<double>(h, w.dinv, nullptr));
    if (masked) {
      // the unpreconditioned case masks a copy of the identity
      if (!pc) CU(cudaMemcpyAsync(w.dinv, w.ones, 3 * (size_t)h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
      launch_segment_mask<double>(h->n_inst, h->inst_seg, h->inst_active, w.dinv + o, h->stream);
    }
    int bst = masked ? batched_pcg<double>(h, h->u, h->r64, w, w.dinv, eta, max_cg, its) : 1;
    if (bst < 0) return bst;
    if (bst == 0) {
      CU(cudaMemcpyAsync(h->tmp64 + o, w.x + o, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
      CU(cudaGetLastError());
      return 0;
    }
    st = pcg_device<double>(h, h->u, h->r64, w.x, (pc || masked) ? w.dinv : nullptr, eta, max_cg, 0, &ps);
    if (st < 0) return st;
    CU(cudaMemcpyAsync(h->tmp64 + o, w.x + o, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  } else {
    KrylovWs<float>& w = h->k32;
    OperatorScope ops(h);
    TRY(ops.st);
    const float* u32 = disp<float>(h);
    launch_convert<double, float>((int64_t)n, h->r64 + o, w.b + o, h->stream);
    if (pc) TRY(jacobi<float>(h, w.dinv, nullptr));
    if (masked) {
      if (!pc) CU(cudaMemcpyAsync(w.dinv, w.ones, 3 * (size_t)h->N * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
      launch_segment_mask<float>(h->n_inst, h->inst_seg, h->inst_active, w.dinv + o, h->stream);
    }
    int bst = masked ? batched_pcg<float>(h, u32, w.b, w, w.dinv, eta, max_cg, its) : 1;
    if (bst < 0) return bst;
    if (bst == 0) {
      launch_convert<float, double>((int64_t)n, w.x + o, h->tmp64 + o, h->stream);
      CU(cudaGetLastError());
      return 0;
    }
    st = pcg_device<float>(h, u32, w.b, w.x, (pc || masked) ? w.dinv : nullptr, eta, max_cg, 0, &ps);
    if (st < 0) return st;
    launch_convert<float, double>((int64_t)n, w.x + o, h->tmp64 + o, h->stream);
  }
  *its = ps.iters;
  CU(cudaGetLastError());
  return 0;
}

// Independent instances: per-instance residual norms of r64, activity flags (an instance
// stays active while |r_k| > rel_tol |r_k(x_0)| and above abs_tol); returns true when all
// instances have converged.  The first call records |r_k(x_0)|.
int instances_update(sfem_handle* h, const sfem_newton_opts& op, bool first, bool* all_done) {
  const size_t o = 3 * (size_t)h->nbc;
  const int K = h->n_inst;
  launch_segment_norms(K, h->inst_seg, h->r64 + o, h->inst_norm, h->stream);
  std::vector<double> nk(K);
  CU(cudaMemcpyAsync(nk.data(), h->inst_norm, K * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  if (first) {
    h->inst_r0 = nk;
    h->inst_its.assign(K, 0);
  }
  std::vector<int32_t> act(K);
  bool done = true;
  for (int k = 0; k < K; k++) {
    h->inst_rel[k] = h->inst_r0[k] > 0 ? nk[k] / h->inst_r0[k] : 0.0;
    const bool conv = !(nk[k] > op.rel_tol * h->inst_r0[k]) || (op.abs_tol > 0 && nk[k] <= op.abs_tol);
    act[k] = conv ? 0 : 1;
    if (!conv) done = false;
  }
  CU(cudaMemcpyAsync(h->inst_active, act.data(), K * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  TRY(sync(h));
  *all_done = done;
  return 0;
}

// one line-search trial into the caller's trace buffer (Newton iteration, step length, |r|)
void trace_trial(sfem_handle* h, int iter, double step, double rnorm) {
  if (!h->ls_trace || !h->ls_trace_count || *h->ls_trace_count >= h->ls_trace_cap) return;
  double* t = h->ls_trace + 3 * (size_t)*h->ls_trace_count;
  t[0] = iter;
  t[1] = step;
  t[2] = rnorm;
  (*h->ls_trace_count)++;
}

// e_init (optional): the total energy at the starting state, computed with its residual
int newton_stage(sfem_handle* h, const sfem_newton_opts& op, double r_ref, double* rn_io, int* nit, int* cgit,
                 int* cuts, int max_newton, const double* e_init = nullptr) {
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  double rn = *rn_io, rprev = rn, eta = op.eta_max;
  const bool inst0 = h->n_inst > 0;
  bool have_e = e_init != nullptr && op.ls_condition == SFEM_LSC_ARMIJO && !inst0;  // e_acc: the energy here
  double e_acc = have_e ? *e_init : 0.0;
  const int max_bis = op.max_bisection > 0 ? op.max_bisection : 30;
  const bool inst = h->n_inst > 0;
  if (inst) h->inst_rel.assign(h->n_inst, 1.0);
  for (int k = 0; k < max_newton; k++) {
    if (inst) {
      bool all = false;
      TRY(instances_update(h, op, k == 0, &all));
      if (all) {
        *rn_io = rn;
        return SFEM_OK;
      }
    } else if (rn <= op.rel_tol * r_ref || (op.abs_tol > 0 && rn <= op.abs_tol)) {
      *rn_io = rn;
      return SFEM_OK;
    }
    // Eisenstat-Walker forcing term (choice 2, gamma 0.9, exponent 2) with safeguards
    if (k > 0) {
      double e2 = 0.9 * (rn / rprev) * (rn / rprev);
      double sg = 0.9 * eta * eta;
      if (sg > 0.1 && sg > e2) e2 = sg;
      eta = std::min(e2, op.eta_max);
    }
    eta = std::max(eta, 0.5 * op.rel_tol * r_ref / rn);
    eta = std::max(eta, op.eta_min);
    eta = std::min(eta, op.eta_max);
    int its = 0;
    using clk = std::chrono::steady_clock;
    clk::time_point t0, t1;
    if (op.verbose) {
      TRY(sync(h));
      t0 = clk::now();
    }
    TRY(inner_solve(h, eta, op.max_cg, op.precond, &its));
    if (op.verbose) {
      TRY(sync(h));
      t1 = clk::now();
    }
    *cgit += its;
    (*nit)++;
    // backtracking line search on the FP64 residual
    CU(cudaMemcpyAsync(h->ubase, h->u, 3 * (size_t)h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    double e_old = 0, slope = 0;
    if (op.ls_condition == SFEM_LSC_ARMIJO) {
      // the energy at this state was computed when the previous step accepted it (same kernel,
      // same state: the same value)
      if (have_e)
        e_old = e_acc;
      else
        TRY(sfem_energy(h, nullptr, &e_old));
      // slope = grad E . d = -r . d
      launch_dot((int64_t)n, h->r64 + o, h->tmp64 + o, h->red(), h->dres + 2, h->stream);
      CU(cudaMemcpyAsync(h->dres_h + 2, h->dres + 2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      TRY(sync(h));
      slope = -h->dres_h[2];
    }
    double rd_old = 0;
    if (op.ls_condition == SFEM_LSC_ENGINEERING) {
      launch_dot((int64_t)n, h->r64 + o, h->tmp64 + o, h->red(), h->dres + 2, h->stream);
      CU(cudaMemcpyAsync(h->dres_h + 2, h->dres + 2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
      TRY(sync(h));
      rd_old = -h->dres_h[2];  // Rold = -delta . rhs
    }
    double a = 1.0;
    bool ok = false;
    double rnew = rn, e_try = 0.0;
    if (op.ls_condition == SFEM_LSC_RESIDUAL) {
      // residual-norm backtracking: halve until |r| decreases sufficiently and no element inverts
      for (int ls = 0; ls <= max_bis; ls++) {
        launch_axpy_state<double>((int64_t)n, a, h->tmp64 + o, h->ubase + o, h->u + o, h->stream);
        int ninv = 0;
        TRY(residual(h, &rnew, &ninv));
        trace_trial(h, *nit - 1, a, rnew);
        if (ninv == 0 && std::isfinite(rnew) && rnew <= (1 - 1e-4 * a) * rn) {
          ok = true;
          break;
        }
        (*cuts)++;
        a *= 0.5;
      }
    } else {
      // NewtonSolverBackTrack's bisection (Include/NewtonSolver.h:242-293)
      double lo = 0.0, hi = 1.0;
      int bis = 0;
      for (;;) {
        launch_axpy_state<double>((int64_t)n, a, h->tmp64 + o, h->ubase + o, h->u + o, h->stream);
        int ninv = 0;
        double en[2] = {0.0, 0.0};  // elastic and total energy, with the residual (Armijo)
        TRY(residual(h, &rnew, &ninv, op.ls_condition == SFEM_LSC_ARMIJO ? en : nullptr));
        trace_trial(h, *nit - 1, a, rnew);
        bool cond = false;
        if (ninv == 0 && std::isfinite(rnew)) {
          if (op.ls_condition == SFEM_LSC_ARMIJO) {
            const double e_el = en[0], e_new = en[1];
            e_try = e_new;
            cond = e_new < e_old + 1e-4 * a * slope;  // Armijo, mAlpha = 1e-4
            // near convergence the energy decrease falls below FP64 resolution of the energy:
            // then a decrease of the residual norm decides
            const double res = 1e-12 * (std::fabs(e_old) + std::fabs(e_el));
            if (!cond && std::fabs(e_new - e_old) <= res && std::fabs(a * slope) <= res) cond = rnew < rn;
          } else {
            launch_dot((int64_t)n, h->r64 + o, h->tmp64 + o, h->red(), h->dres + 2, h->stream);
            CU(cudaMemcpyAsync(h->dres_h + 2, h->dres + 2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            TRY(sync(h));
            cond = -h->dres_h[2] < 0.5 * rd_old;  // Bonet-Wood as coded: Rnew < 0.5 Rold
          }
        }
        if (!cond) {
          hi = a;
          bis++;
          (*cuts)++;
        } else if (bis > 10 || a == 1.0) {
          ok = true;
          break;
        } else {
          lo = a;
          bis++;
        }
        a = 0.5 * (lo + hi);
        if (a < 1e-10) break;
      }
    }
    if (op.verbose) {
      TRY(sync(h));
      const double ms_cg = std::chrono::duration<double, std::milli>(t1 - t0).count();
      const double ms_ls = std::chrono::duration<double, std::milli>(clk::now() - t1).count();
      fprintf(stderr, "[sfem] newton %d: |r| %.6e -> %.6e  cg %d  eta %.2e  step %.3g  (%.2f ms solve, %.2f ms line search)\n",
              *nit, rn, rnew, its, eta, a, ms_cg, ms_ls);
    }
    if (!ok) {
      CU(cudaMemcpyAsync(h->u, h->ubase, 3 * (size_t)h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
      TRY(residual(h, &rn, nullptr));
      *rn_io = rn;
      return SFEM_LINESEARCH_FAILED;
    }
    rprev = rn;
    rn = rnew;
    have_e = op.ls_condition == SFEM_LSC_ARMIJO && !inst;
    e_acc = e_try;
    if (inst) {
      std::vector<int32_t> act(h->n_inst);
      CU(cudaMemcpyAsync(act.data(), h->inst_active, h->n_inst * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
      TRY(sync(h));
      for (int q = 0; q < h->n_inst; q++) h->inst_its[q] += act[q];
    }
  }
  *rn_io = rn;
  if (inst) {
    bool all = false;
    TRY(instances_update(h, op, false, &all));
    return all ? SFEM_OK : SFEM_NOT_CONVERGED;
  }
  return (rn <= op.rel_tol * r_ref || (op.abs_tol > 0 && rn <= op.abs_tol)) ? SFEM_OK : SFEM_NOT_CONVERGED;
}

}  // namespace

extern "C" {

int sfem_newton_solve(sfem_handle* h, const sfem_newton_opts* opts, sfem_newton_stats* stats) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (!opts) return fail(SFEM_ERR_INVALID, "opts is null");
  if (opts->precond == SFEM_PC_LEARNED && !h->gnn)
    return fail(SFEM_ERR_INVALID, "learned preconditioner not initialised (sfem_gnn_init)");
  sfem_newton_opts op = *opts;
  if (op.eta_max <= 0) op.eta_max = 0.5;
  if (op.eta_min <= 0) op.eta_min = h->precision == SFEM_FP32 ? 1e-5 : 1e-10;
  if (op.max_newton <= 0) op.max_newton = 50;
  if (op.max_cg <= 0) op.max_cg = 100000;
  if (h->precision == SFEM_FP32) TRY(alloc_ws(h, h->k32));
  CU(cudaEventRecord(h->ev0, h->stream));
  const double ff_final = h->ff;
  int nit = 0, cgit = 0, cuts = 0, st = SFEM_OK;
  double r0 = 0, rn = 0;
  const int steps = op.load_steps > 1 ? op.load_steps : 1;
  // |r(x_0)| of the full load defines the relative tolerance; for a one-step Armijo solve the same
  // element pass also gives the starting energy the first line search compares against
  const bool e_first = steps == 1 && op.ls_condition == SFEM_LSC_ARMIJO && h->n_inst == 0;
  double e0[2] = {0.0, 0.0};
  TRY(residual(h, &r0, nullptr, e_first ? e0 : nullptr));
  for (int s = 1; s <= steps; s++) {
    h->ff = ff_final * (double)s / steps;
    double r_ref = r0;
    sfem_newton_opts so = op;
    if (s < steps) {
      // intermediate load steps of the quasi-static ramp need only a rough equilibrium
      TRY(residual(h, &rn, nullptr));
      r_ref = rn;
      so.rel_tol = 1e-3;
      so.abs_tol = 0;
    } else if (steps > 1) {
      TRY(residual(h, &rn, nullptr));
    } else {
      rn = r0;
    }
    st = newton_stage(h, so, r_ref, &rn, &nit, &cgit, &cuts, op.max_newton - nit, e_first ? &e0[1] : nullptr);
    if (st < 0 || st == SFEM_LINESEARCH_FAILED) break;
  }
  h->ff = ff_final;
  CU(cudaEventRecord(h->ev1, h->stream));
  TRY(sync(h));
  float ms = 0;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  if (stats) {
    stats->newton_iters = nit;
    stats->cg_iters = cgit;
    stats->status = st;
    stats->line_search_cuts = cuts;
    stats->r0 = r0;
    stats->rel_res = r0 > 0 ? rn / r0 : 0;
    stats->seconds = ms * 1e-3;
  }
  if (st < 0) return st;
  if (!std::isfinite(rn)) return fail(SFEM_ERR_NAN, "residual is not finite");
  return st;
}

// NonlinearConjugateGradientMinimizer::Solve, Include/NonlinearCG.h:51-114 (constants eps = tol = 1e-2f).
int sfem_nonlinear_cg(sfem_handle* h, int32_t outer_iters, int32_t inner_iters, double abs_tol, int32_t* iters_done) {
  TRY(check_handle(h));
  TRY(set_device(h));
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  const double eps2 = (double)(1e-2f * 1e-2f), tol2 = (double)(1e-2f * 1e-2f);
  double* d = h->k64.p;  // search direction (full length, zero fixed block)
  double* df = h->k64.q;
  auto dot = [&](const double* a, const double* b, double* out) -> int {
    launch_dot((int64_t)n, a + o, b + o, h->red(), h->dres + 3, h->stream);
    CU(cudaMemcpyAsync(h->dres_h + 3, h->dres + 3, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    *out = h->dres_h[3];
    return 0;
  };
  double rn;
  TRY(residual(h, &rn, nullptr));
  CU(cudaMemsetAsync(d, 0, 3 * (size_t)h->N * sizeof(double), h->stream));
  CU(cudaMemcpyAsync(d + o, h->r64 + o, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  double delta = 0.0;
  TRY(dot(h->r64, h->r64, &delta));
  const double delta0 = delta;
  int iter = 0;
  if (delta != 0) {
    for (; iter < outer_iters; iter++) {
      double deltaD = 0.0;
      TRY(dot(d, d, &deltaD));
      for (int inner = 0; inner < inner_iters; inner++) {
        hvp<double>(h, h->u, d, df, nullptr);
        double rd = 0.0, ddf = 0.0;
        TRY(dot(h->r64, d, &rd));
        TRY(dot(d, df, &ddf));
        const double alpha = rd / ddf;
        launch_axpy_state<double>((int64_t)n, alpha, d + o, h->u + o, h->u + o, h->stream);
        TRY(residual(h, &rn, nullptr));
        if (alpha * alpha * deltaD < tol2) break;
      }
      double delta1 = 0.0;
      TRY(dot(h->r64, h->r64, &delta1));
      const double beta = delta1 / delta;
      delta = delta1;
      if (delta < abs_tol * abs_tol) { iter++; break; }
      if (delta <= eps2 * delta0) { iter++; break; }
      // d = r + beta d
      launch_axpy_state<double>((int64_t)n, beta, d + o, h->r64 + o, d + o, h->stream);
    }
  }
  if (iters_done) *iters_done = iter;
  TRY(sync(h));
  return std::isfinite(delta) ? SFEM_OK : fail(SFEM_ERR_NAN, "residual is not finite");
}

int sfem_adjoint_dev(sfem_handle* h, const double* dLdu_dev, double rel_tol, int32_t max_cg, double* dLdE_dev,
                     double* dLdf_dev) {
  TRY(check_handle(h));
  if (h->material == SFEM_MMT_COROTATIONAL || h->material > 3)
    return fail(SFEM_ERR_INVALID, "adjoint needs the consistent symmetric tangent of the linear, StVK or "
                                  "neo-Hookean material");
  if (h->has_scale && h->has_scale_la)
    return fail(SFEM_ERR_INVALID, "dL/dE assumes a uniform Poisson ratio (per-element Lame parameters are set)");
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  KrylovWs<double>& w = h->k64;
  CU(cudaMemcpyAsync(w.b + o, dLdu_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  TRY(jacobi<double>(h, w.dinv, nullptr));
  sfem_pcg_stats ps{};
  int st = pcg_device<double>(h, h->u, w.b, w.x, w.dinv, rel_tol, max_cg > 0 ? max_cg : 100000, 0, &ps);
  if (st == SFEM_NEGATIVE_CURVATURE) return SFEM_ERR_BREAKDOWN;
  if (st < 0) return st;
  // element internal forces at the current state
  element_pass<double>(h, MODE_FORCE, h->u, nullptr, h->fe, nullptr, nullptr, nullptr);
  if (!h->young_e) {
    std::vector<double> ye((size_t)h->E, h->young);
    TRY(dalloc(&h->young_e, (size_t)h->E));
    TRY(dalloc(&h->scale64, (size_t)h->E));
    TRY(dalloc(&h->scale32, (size_t)h->E));
    CU(cudaMemcpyAsync(h->young_e, ye.data(), ye.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    TRY(sync(h));
  } else if (!h->has_scale) {
    std::vector<double> ye((size_t)h->E, h->young);
    CU(cudaMemcpyAsync(h->young_e, ye.data(), ye.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    TRY(sync(h));
  }
  launch_adjoint_elem(h->tets, h->E, h->nbc, h->fe, w.x, h->young_e, h->perm, dLdE_dev, h->stream);
  // dL/df = ff * lambda
  launch_scale_copy((int64_t)n, h->ff, w.x + o, dLdf_dev, h->stream);
  CU(cudaGetLastError());
  return st;
}

int sfem_adjoint(sfem_handle* h, const double* dLdu, double rel_tol, int32_t max_cg, double* dLdE, double* dLdf) {
  TRY(check_handle(h));
  TRY(set_device(h));
  const size_t n = 3 * (size_t)h->nf;
  double *du = nullptr, *dE = nullptr, *dfp = nullptr;
  TRY(dalloc(&du, n));
  TRY(dalloc(&dE, (size_t)h->E));
  TRY(dalloc(&dfp, n));
  int st = 0;
  if (cudaMemcpyAsync(du, dLdu, n * sizeof(double), cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    st = fail(SFEM_ERR_CUDA, "copy failed");
  if (st == 0) st = sfem_adjoint_dev(h, du, rel_tol, max_cg, dE, dfp);
  if (st >= 0) {
    if (dLdE) cudaMemcpyAsync(dLdE, dE, (size_t)h->E * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (dLdf) cudaMemcpyAsync(dLdf, dfp, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    int s2 = sync(h);
    if (s2 < 0) st = s2;
  }
  cudaFree(du);
  cudaFree(dE);
  cudaFree(dfp);
  return st;
}

}  // extern "C"

// =============================================================================
// Learned preconditioner (extension; the reference has no learned components)
// =============================================================================
namespace {

struct GnnState {
  int64_t n = 0;  // free nodes
  int32_t *ptr = nullptr, *idx = nullptr;
  float* inv_deg = nullptr;
  float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16* Wb = nullptr;          // 3 packed BF16 weight sets (k_gnn_pack)
  __nv_bfloat16* h[gnn::NL + 1] = {};   // activations of S at x = D^-1/2 r
  __nv_bfloat16* hg[gnn::NL + 1] = {};  // activations of S at D^-1/2 dL/dM (training)
  float *x = nullptr, *xg = nullptr;    // the two inputs (training)
  float *G0 = nullptr, *G1 = nullptr, *G2 = nullptr;  // transposed-pass vectors (n x H, training)
  float* wpart = nullptr;
  float* spart = nullptr;
  unsigned* scount = nullptr;
  float* losses = nullptr;  // device, one per training step
  int64_t losses_cap = 0;
  float *z = nullptr, *rprev = nullptr;  // FCG vectors (3N)
  std::vector<float*> R, Ee;             // dataset: residual and correction (free block, 3n)
  std::vector<float> cinv;               // 1 / (e . r) per sample
  std::vector<float> rinv;               // 1 / (r . r) per sample
  float* tmp = nullptr;                  // 3N scratch
  int loss_mode = 0;                     // 0: energy norm of the error, 1: residual norm
  int batch = 1;                         // pairs per Adam step
  int infer_mode = 0;                    // 0: folded polynomial, 1: tensor-core layers
  gnn::PolyCoef pc{};                    // folded coefficients of the current weights
  bool pc_dirty = true;
  // polynomial-form FP16 node rows (gnn::Row16): the input sigma D^-1/2 r, y1, y2 (n each) and w
  // (4 x n); xstat: the rows' sum of d r^2 and sigma
  gnn::Row16 *px = nullptr, *py1 = nullptr, *py2 = nullptr, *pw = nullptr;
  float* xstat = nullptr;
  float* bpart = nullptr;  // block partials of the fused beta pass (4 per 256 nodes)
  int adam_t = 0;
  bool train_bufs = false;
  int16_t* d16 = nullptr;  // neighbour deltas (polynomial passes), when they fit
  uint16_t* pid = nullptr;  // neighbour patterns (polynomial passes), when the table is small
  int32_t* pptr = nullptr;
  int16_t* ptab = nullptr;
  int32_t npat = 0;
  gnn::Graph graph() const { return gnn::Graph{n, ptr, idx, inv_deg, d16, pid, pptr, ptab}; }
};

void gnn_free(GnnState* g) {
  void* bufs[] = {g->ptr, g->idx, g->inv_deg, g->params, g->grad, g->m, g->v, g->Wb, g->x, g->xg,
                  g->G0, g->G1, g->G2, g->wpart, g->spart, g->scount, g->losses, g->z, g->rprev, g->tmp,
                  g->px, g->py1, g->py2, g->pw, g->xstat, g->bpart, g->d16, g->pid, g->pptr, g->ptab};
  for (void* b : bufs)
    if (b) cudaFree(b);
  for (int l = 0; l <= gnn::NL; l++) {
    if (g->h[l]) cudaFree(g->h[l]);
    if (g->hg[l]) cudaFree(g->hg[l]);
  }
  for (float* b : g->R) cudaFree(b);
  for (float* b : g->Ee) cudaFree(b);
  delete g;
}

int gnn_need(const sfem_handle* h) {
  if (!h->gnn) return fail(SFEM_ERR_INVALID, "learned preconditioner not initialised (sfem_gnn_init)");
  if (h->precision != SFEM_FP32) return fail(SFEM_ERR_INVALID, "the learned preconditioner runs in FP32 handles");
  return 0;
}

int gnn_train_buffers(sfem_handle* h) {
  GnnState* g = h->gnn;
  if (g->train_bufs) return 0;
  const size_t nh = (size_t)g->n * gnn::H;
  for (int l = 0; l <= gnn::NL; l++) TRY(dalloc(&g->hg[l], nh));
  TRY(dalloc(&g->G0, nh));
  TRY(dalloc(&g->G1, nh));
  TRY(dalloc(&g->G2, nh));
  TRY(dalloc(&g->x, (size_t)g->n * gnn::FIN));
  TRY(dalloc(&g->xg, (size_t)g->n * gnn::FIN));
  const size_t nbl = (size_t)((g->n + gnn::TILE - 1) / gnn::TILE), nbe = (size_t)((g->n + 63) / 64);
  TRY(dalloc(&g->wpart, std::max(nbl * gnn::LPART, nbe * gnn::H * gnn::FIN)));
  g->train_bufs = true;
  return 0;
}

// current Jacobi diagonal (FP32) into k32.dinv
int gnn_refresh_diag(sfem_handle* h) {
  TRY(jacobi<float>(h, h->k32.dinv, nullptr));
  CU(cudaGetLastError());
  return 0;
}

float bf16_rne(float v) {  // the rounding of __float2bfloat16 for finite values
  uint32_t u;
  memcpy(&u, &v, 4);
  u += 0x7fffu + ((u >> 16) & 1u);
  u &= 0xffff0000u;
  float r;
  memcpy(&r, &u, 4);
  return r;
}

// Fold the current weights into the polynomial coefficients (FP64 on the host, from the same
// BF16-rounded layer weights the tensor-core kernels use):
//   prod_l (P_l + A Q_l) = sum_k A^k C_k,  P_l = I + Wa_l^T,  Q_l = Wb_l^T,
//   T_k = We^T C_k (3 x H),  G[k][j] = T_k T_j^T.
int gnn_poly_refresh(sfem_handle* h) {
  GnnState* g = h->gnn;
  if (!g->pc_dirty) return 0;
  constexpr int H = gnn::H, K = gnn::NL + 1;
  std::vector<float> prm(gnn::NPARAM);
  CU(cudaMemcpyAsync(prm.data(), g->params, gnn::NPARAM * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  std::vector<double> C((size_t)K * H * H, 0.0), N((size_t)K * H * H), P((size_t)H * H), Q((size_t)H * H);
  for (int a = 0; a < H; a++) C[(size_t)a * H + a] = 1.0;
  for (int l = 0; l < gnn::NL; l++) {
    const float* W = prm.data() + gnn::OFF_L + (size_t)l * gnn::L_STRIDE;  // [H][AIN]
    for (int a = 0; a < H; a++)
      for (int o = 0; o < H; o++) {
        P[(size_t)a * H + o] = (a == o ? 1.0 : 0.0) + bf16_rne(W[(size_t)o * gnn::AIN + a]);
        Q[(size_t)a * H + o] = bf16_rne(W[(size_t)o * gnn::AIN + H + a]);
      }
    std::fill(N.begin(), N.end(), 0.0);
    for (int k = 0; k <= l; k++) {
      const double* Ck = &C[(size_t)k * H * H];
      for (int a = 0; a < H; a++)
        for (int b = 0; b < H; b++) {
          const double cab = Ck[(size_t)a * H + b];
          if (cab == 0.0) continue;
          double* n0 = &N[(size_t)k * H * H + (size_t)a * H];
          double* n1 = &N[(size_t)(k + 1) * H * H + (size_t)a * H];
          for (int o = 0; o < H; o++) {
            n0[o] += cab * P[(size_t)b * H + o];
            n1[o] += cab * Q[(size_t)b * H + o];
          }
        }
    }
    C.swap(N);
  }
  std::vector<double> T((size_t)K * 3 * H, 0.0);
  for (int k = 0; k < K; k++)
    for (int f = 0; f < 3; f++)
      for (int b = 0; b < H; b++) {
        const double e = prm[gnn::OFF_WE + (size_t)b * gnn::FIN + f];
        for (int a = 0; a < H; a++) T[((size_t)k * 3 + f) * H + a] += e * C[(size_t)k * H * H + (size_t)b * H + a];
      }
  for (int k = 0; k < K; k++)
    for (int j = 0; j < K; j++)
      for (int f = 0; f < 3; f++)
        for (int q = 0; q < 3; q++) {
          double a = 0.0;
          for (int x = 0; x < H; x++) a += T[((size_t)k * 3 + f) * H + x] * T[((size_t)j * 3 + q) * H + x];
          g->pc.G[k][j][3 * f + q] = (float)a;
        }
  g->pc.c = (float)std::exp((double)prm[gnn::OFF_C]);
  g->pc_dirty = false;
  return 0;
}

// out = M(r) over the free block (r, out point at free-block starts); done may be null.
// With train, x = D^-1/2 r and the activations of S are kept for the weight gradient.
// Inference uses the folded polynomial (gnn_poly_refresh must have run) or the layers.
void gnn_apply_dev(sfem_handle* h, const float* r, float* out, const int* done, bool train) {
  GnnState* g = h->gnn;
  const size_t o = 3 * (size_t)h->nbc;
  const float* dinv = h->k32.dinv + o;
  if (train)
    gnn::launch_apply_train(g->graph(), r, dinv, g->params, g->Wb, g->h, g->x, g->G0, g->G1, g->G2, out, h->stream);
  else if (g->infer_mode == 0)
    gnn::launch_apply_poly(g->graph(), r, dinv, g->pc, g->px, g->py1, g->py2, g->pw, g->xstat, out, done, h->stream,
                           g->bpart, h->counter);
  else
    gnn::launch_apply(g->graph(), r, dinv, g->params, g->Wb, g->h, out, done, h->stream);
}

// loss of one sample and the parameter gradient into g->grad; loss into *loss_dev.
//   energy mode:   d = M(r) - e,      L = d.Kd / (e.r),   dL/dM = 2 K d / (e.r)
//   residual mode: d = K M(r) - r,    L = d.d / (r.r),    dL/dM = 2 K d / (r.r)
// With gy = D^-1/2 dL/dM and x = D^-1/2 r, the S-part of dL is d<S gy, S x>: the weight
// gradient of <S x, S gy> at input x plus that at input gy (S is linear), and
// dL/d(log c) = c gy.x.
int gnn_loss_grad_dev(sfem_handle* h, const float* r, const float* e, float cinv, float rinv, float* loss_dev,
                      int accumulate = 0) {
  GnnState* g = h->gnn;
  TRY(gnn_train_buffers(h));
  KrylovWs<float>& w = h->k32;
  const size_t o = 3 * (size_t)h->nbc, n3 = 3 * (size_t)g->n;
  const float* dinv = w.dinv + o;
  float* out = g->z + o;
  gnn_apply_dev(h, r, out, nullptr, true);
  float* Go = g->rprev + o;
  if (g->loss_mode == 0) {
    // d = M(r) - e into a full-length vector with a zero fixed block, q = K d
    gnn::launch_sub((int64_t)n3, out, e, w.b + o, h->stream);
    hvp<float>(h, w.u, w.b, w.q, nullptr);
    gnn::launch_loss((int64_t)n3, w.b + o, w.q + o, cinv, Go, g->spart, g->scount, loss_dev, h->stream);
  } else {
    CU(cudaMemcpyAsync(w.b + o, out, n3 * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
    hvp<float>(h, w.u, w.b, w.q, nullptr);                 // q = K M(r)
    gnn::launch_sub((int64_t)n3, w.q + o, r, w.b + o, h->stream);  // d = K M(r) - r
    hvp<float>(h, w.u, w.b, w.q, nullptr);                 // q = K d
    gnn::launch_loss((int64_t)n3, w.b + o, w.q + o, rinv, Go, g->spart, g->scount, g->spart + 4001, h->stream);
    gnn::launch_loss((int64_t)n3, w.b + o, w.b + o, rinv, g->tmp + o, g->spart, g->scount, loss_dev, h->stream);
  }
  const gnn::Graph gr = g->graph();
  gnn::launch_encode(gr, Go, dinv, g->params, g->hg[0], g->xg, nullptr, h->stream);
  gnn::launch_layers_fwd(gr, g->Wb, g->hg, nullptr, h->stream);
  gnn::launch_weight_grad(gr, g->hg[gnn::NL], g->h, g->x, g->Wb, g->G0, g->G1, g->G2, g->wpart, g->grad,
                          accumulate, h->stream);
  gnn::launch_weight_grad(gr, g->h[gnn::NL], g->hg, g->xg, g->Wb, g->G0, g->G1, g->G2, g->wpart, g->grad, 1,
                          h->stream);
  gnn::launch_cgrad((int64_t)n3, Go, r, dinv, g->params, g->spart, g->scount, g->grad, accumulate, h->stream);
  CU(cudaGetLastError());
  return 0;
}

// Flexible CG (Polak-Ribiere beta) with the learned preconditioner, FP32; b, x full length.
// Per iteration: the fused patch HVP builds p = z + beta p_old (or D^-1 r + beta p_old after a
// non-descent z) and K p, p.Kp, alpha; the fused update assembles the shared-node q and does
// x, r and r.r; the preconditioner's last pass forms z = M(r) and the next beta.
int fcg_device(sfem_handle* h, const float* b, float* x, double tol, int max_it, sfem_pcg_stats* st) {
  GnnState* g = h->gnn;
  KrylovWs<float>& w = h->k32;
  const int64_t o = 3 * h->nbc, n = 3 * h->nf;
  CgScalars s0;
  memset(&s0, 0, sizeof(s0));
  s0.tol2 = tol * tol;
  s0.max_it = max_it;
  *h->scal_h = s0;
  CU(cudaMemcpyAsync(h->scal, h->scal_h, sizeof(CgScalars), cudaMemcpyHostToDevice, h->stream));
  TRY(gnn_poly_refresh(h));
  NhCacheGuard<float> cache(h, w.u);
  launch_cg_init<float>(n, b + o, x + o, w.r + o, w.p + o, w.dinv + o, h->red(), h->scal, h->stream);
  const int* done = &h->scal->done;
  float* part = reinterpret_cast<float*>(h->partials);
  const float* dinv = w.dinv + o;
  // the polynomial's input rows D^-1/2 r, formed by the update kernel from the second pass on
  gnn::Row16* xs = g->infer_mode == 0 ? g->px : nullptr;
  const CoarseView cvw = h->cv();
  auto precondition = [&](bool with_beta, bool runs_done) {
    if (h->cs_on && g->infer_mode == 0) {
      // two-level: y = W B^T r (the update may have formed the restriction's run sums) on the coarse
      // chain's own stream, beside the polynomial's first five passes; the last pass waits for it,
      // adds B y to M(r) and forms beta, z.r
      cudaEventRecord(h->cs_fork, h->stream);  // errors surface at the loop's next check
      cudaStreamWaitEvent(h->cs_stream, h->cs_fork, 0);
      if (runs_done)
        launch_coarse_sum_gemv(cvw, h->cs_stream);
      else
        launch_coarse_restrict_gemv(cvw, w.r + o, h->cs_stream);
      cudaEventRecord(h->cs_join, h->cs_stream);
      gnn::launch_apply_poly(g->graph(), w.r + o, dinv, g->pc, g->px, g->py1, g->py2, g->pw, g->xstat, g->z + o,
                             done, h->stream, g->bpart, h->counter, with_beta ? g->rprev + o : nullptr,
                             with_beta ? h->scal : nullptr, with_beta, CoarseAdd{h->cs_aid, h->cs_d, h->cs_y, h->cs_nm},
                             h->cs_join);
      return;
    }
    if (h->cs_on) {
      // two-level through the layer kernels: z = M(r) + P Kc^-1 P^T r, then beta and z.r from the complete z
      gnn::launch_apply(g->graph(), w.r + o, dinv, g->params, g->Wb, g->h, g->z + o, done, h->stream);
      launch_coarse_apply(h->cv(), w.r + o, g->z + o, h->stream);
      if (with_beta)
        gnn::launch_fcg_beta(n, w.r + o, g->rprev + o, g->z + o, dinv, part, h->counter, h->scal, h->stream);
      return;
    }
    if (g->infer_mode == 0) {
      gnn::launch_apply_poly(g->graph(), w.r + o, dinv, g->pc, g->px, g->py1, g->py2, g->pw, g->xstat, g->z + o,
                             done, h->stream, g->bpart, h->counter, with_beta ? g->rprev + o : nullptr,
                             with_beta ? h->scal : nullptr, with_beta);
    } else {
      gnn::launch_apply(g->graph(), w.r + o, dinv, g->params, g->Wb, g->h, g->z + o, done, h->stream);
      if (with_beta)
        gnn::launch_fcg_beta(n, w.r + o, g->rprev + o, g->z + o, dinv, part, h->counter, h->scal, h->stream);
    }
  };
  precondition(false, false);
  gnn::launch_fcg_init(n, w.r + o, g->z + o, w.p + o, part, h->counter, h->scal, h->stream);  // p_old = 0
  float* pbuf[2] = {w.p, w.p2};
  // iterations between the host's looks at the stop flag: 16, or fewer once the residual's decay
  // over the last look predicts convergence sooner (the launches queued past convergence return at
  // once, but each still costs a launch)
  const int check_every = 16;
  int chunk = check_every, it = 0, it_prev = -1;
  double rr_prev = 0.0;
  bool pending = false;
  if (h->profiling) {
    h->prof_precision = SFEM_FP32;
    h->prof_op = h->sell_on ? 1 : 0;
  }
  for (;;) {
    CU(cudaMemcpyAsync(h->scal_h, h->scal, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    if (h->scal_h->done || it >= max_it) break;
    {
      const double rr = h->scal_h->rr, goal = h->scal_h->tol2;
      chunk = check_every;
      if (it_prev >= 0 && rr > 0.0 && goal > 0.0 && rr_prev > rr && h->scal_h->it > it_prev) {
        const double rate = std::log(rr_prev / rr) / (double)(h->scal_h->it - it_prev);
        const double need = std::log(rr / goal) / rate;
        if (need < check_every - 2) chunk = std::max(2, (int)std::ceil(need * 1.1) + 1);
      }
      it_prev = h->scal_h->it;
      rr_prev = rr;
    }
    if (pending) {
      float a = 0, bms = 0;
      cudaEventElapsedTime(&a, h->pev[0], h->pev[1]);
      cudaEventElapsedTime(&bms, h->pev[1], h->pev[2]);
      h->prof_elem_ms += a;
      h->prof_gather_ms += bms;
      h->prof_samples++;
      pending = false;
    }
    for (int k = 0; k < chunk && it < max_it; k++, it++) {
      const bool sample = h->profiling && k == 0;
      float* pold = pbuf[it % 2];
      float* pnew = pbuf[(it + 1) % 2];
      if (sample) CU(cudaEventRecord(h->pev[0], h->stream));
      krylov_hvp<float>(h, w.u, pold, w.q, sample ? h->pev[1] : nullptr, w.r, w.dinv, pnew, g->z);
      if (sample) {
        CU(cudaEventRecord(h->pev[2], h->stream));
        pending = true;
      }
      if (h->profiling) h->prof_launches++;
      const bool runs = launch_fcg_update_patch<float>(
          h->nbc, h->N, krylov_bslot<float>(h), reinterpret_cast<const float*>(h->partial), x, w.r, g->rprev, pnew, w.q,
          h->red(), h->scal, h->stream, xs ? w.dinv : nullptr, xs, g->xstat,
          h->cs_on && g->infer_mode == 0 ? &cvw : nullptr);
      precondition(true, runs);
    }
  }
  if (pending) {
    float a = 0, bms = 0;
    cudaEventElapsedTime(&a, h->pev[0], h->pev[1]);
    cudaEventElapsedTime(&bms, h->pev[1], h->pev[2]);
    h->prof_elem_ms += a;
    h->prof_gather_ms += bms;
    h->prof_samples++;
  }
  const CgScalars& s = *h->scal_h;
  if (st) {
    st->iters = s.it;
    st->status = s.status;
    st->rel_res = s.bb > 0 ? std::sqrt(s.rr / s.bb) : 0.0;
  }
  if (s.status == -3) return fail(SFEM_ERR_NAN, "non-finite value in the flexible Krylov recurrence");
  if (s.status == 2) {
    // negative curvature at the first iteration: return the first direction (z itself)
    if (s.it == 0) CU(cudaMemcpyAsync(x + o, pbuf[1] + o, n * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
    return SFEM_NEGATIVE_CURVATURE;
  }
  return s.status == 1 ? SFEM_NOT_CONVERGED : SFEM_OK;
}

}  // namespace

// learned inner solve of the Newton driver (declared before inner_solve's use below)
int sfem_gnn_inner_solve(sfem_handle* h, double eta, int max_cg, int* its) {
  TRY(gnn_need(h));
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  KrylovWs<float>& w = h->k32;
  OperatorScope ops(h);
  TRY(ops.st);
  launch_convert<double, float>(3 * h->N, h->u, w.u, h->stream);
  launch_convert<double, float>((int64_t)n, h->r64 + o, w.b + o, h->stream);
  TRY(gnn_refresh_diag(h));
  sfem_pcg_stats ps{};
  int st = fcg_device(h, w.b, w.x, eta, max_cg, &ps);
  if (st < 0) return st;
  launch_convert<float, double>((int64_t)n, w.x + o, h->tmp64 + o, h->stream);
  *its = ps.iters;
  CU(cudaGetLastError());
  return 0;
}

extern "C" {

int sfem_gnn_num_params(int32_t* n) {
  if (!n) return fail(SFEM_ERR_INVALID, "null");
  *n = gnn::NPARAM;
  return SFEM_OK;
}

int sfem_gnn_init(sfem_handle* h, uint64_t seed) {
  TRY(check_handle(h));
  TRY(set_device(h));
  if (h->precision != SFEM_FP32) return fail(SFEM_ERR_INVALID, "the learned preconditioner runs in FP32 handles");
  if (h->gnn) {
    gnn_free(h->gnn);
    h->gnn = nullptr;
  }
  GnnState* g = new GnnState();
  h->gnn = g;
  const int64_t nbc = h->nbc, n = h->nf;
  g->n = n;
  // free-node graph from the element edges
  std::vector<int4> tt((size_t)h->E);
  CU(cudaMemcpyAsync(tt.data(), h->tets, tt.size() * sizeof(int4), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  std::vector<uint64_t> edges;
  edges.reserve(tt.size() * 12);
  for (const int4& t4 : tt) {
    const int32_t v[4] = {t4.x, t4.y, t4.z, t4.w};
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++)
        if (a != b && v[a] >= nbc && v[b] >= nbc)
          edges.push_back(((uint64_t)(v[a] - nbc) << 32) | (uint32_t)(v[b] - nbc));
  }
  std::sort(edges.begin(), edges.end());
  edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
  std::vector<int32_t> ptr((size_t)n + 1, 0), idx(edges.size());
  for (size_t k = 0; k < edges.size(); k++) {
    ptr[(edges[k] >> 32) + 1]++;
    idx[k] = (int32_t)(edges[k] & 0xffffffffu);
  }
  for (int64_t i = 0; i < n; i++) ptr[i + 1] += ptr[i];
  std::vector<float> invdeg((size_t)n);
  for (int64_t i = 0; i < n; i++) invdeg[i] = 1.f / (float)std::max(1, ptr[i + 1] - ptr[i]);
  // 16-bit neighbour deltas halve the index traffic of the polynomial passes when they fit
  std::vector<int16_t> d16(idx.size());
  bool fits16 = true;
  for (int64_t i = 0; i < n && fits16; i++)
    for (int32_t k = ptr[i]; k < ptr[i + 1]; k++) {
      const int64_t dlt = (int64_t)idx[k] - i;
      if (dlt < -32768 || dlt > 32767) {
        fits16 = false;
        break;
      }
      d16[k] = (int16_t)dlt;
    }
  // Nodes with equal delta lists (the interior of a structured lattice, each face, edge and
  // corner class) share one entry of a pattern table; a polynomial pass then reads a 2-byte id
  // per node instead of the node's list.  Kept when the table is at most a quarter of the
  // deltas and 32768 entries, i.e. when most nodes repeat a pattern.
  std::vector<uint16_t> pid;
  std::vector<int32_t> pptr(1, 0);
  std::vector<int16_t> ptab;
  if (fits16 && n > 0) {
    const size_t cap = std::min<size_t>(32768, d16.size() / 4);
    std::map<std::vector<int16_t>, uint16_t> seen;
    pid.resize((size_t)n);
    std::vector<int16_t> key;
    for (int64_t i = 0; i < n; i++) {
      key.assign(d16.begin() + ptr[i], d16.begin() + ptr[i + 1]);
      auto it = seen.find(key);
      if (it == seen.end()) {
        if (seen.size() >= 65535 || ptab.size() + key.size() > cap) {
          pid.clear();
          break;
        }
        it = seen.emplace(key, (uint16_t)seen.size()).first;
        ptab.insert(ptab.end(), key.begin(), key.end());
        pptr.push_back((int32_t)ptab.size());
      }
      pid[(size_t)i] = it->second;
    }
  }
  // seeded normal weights; log c = 0
  std::vector<float> prm(gnn::NPARAM, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (int i = 0; i < gnn::H * gnn::FIN; i++) prm[gnn::OFF_WE + i] = nd(rng) * 0.3f;
  for (int l = 0; l < gnn::NL; l++)
    for (int i = 0; i < gnn::H * gnn::AIN; i++)
      prm[gnn::OFF_L + l * gnn::L_STRIDE + i] = nd(rng) * (0.5f / std::sqrt((float)gnn::AIN));
  const size_t nh = (size_t)n * gnn::H;
  TRY(dalloc(&g->ptr, ptr.size()));
  TRY(dalloc(&g->idx, std::max<size_t>(idx.size(), 1)));
  TRY(dalloc(&g->inv_deg, (size_t)n));
  TRY(dalloc(&g->params, gnn::NPARAM));
  TRY(dalloc(&g->grad, gnn::NPARAM));
  TRY(dalloc(&g->m, gnn::NPARAM));
  TRY(dalloc(&g->v, gnn::NPARAM));
  TRY(dalloc(&g->Wb, (size_t)3 * gnn::NL * gnn::H * gnn::AIN));
  for (int l = 0; l <= gnn::NL; l++) TRY(dalloc(&g->h[l], nh));
  TRY(dalloc(&g->px, (size_t)n));
  TRY(dalloc(&g->py1, (size_t)n));
  TRY(dalloc(&g->py2, (size_t)n));
  TRY(dalloc(&g->pw, 4 * (size_t)n));
  TRY(dalloc(&g->xstat, 2));
  {
    const float xs0[2] = {0.f, 1.f};
    CU(cudaMemcpyAsync(g->xstat, xs0, sizeof(xs0), cudaMemcpyHostToDevice, h->stream));
    TRY(sync(h));
  }
  TRY(dalloc(&g->bpart, 4 * (size_t)((n + 255) / 256) + 64));
  TRY(dalloc(&g->spart, 4096));
  TRY(dalloc(&g->scount, 1));
  TRY(dalloc(&g->z, 3 * (size_t)h->N));
  TRY(dalloc(&g->rprev, 3 * (size_t)h->N));
  TRY(dalloc(&g->tmp, 3 * (size_t)h->N));
  CU(cudaMemcpyAsync(g->ptr, ptr.data(), ptr.size() * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  if (!idx.empty())
    CU(cudaMemcpyAsync(g->idx, idx.data(), idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemcpyAsync(g->inv_deg, invdeg.data(), invdeg.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  if (fits16 && !d16.empty()) {
    TRY(dalloc(&g->d16, d16.size()));
    CU(cudaMemcpyAsync(g->d16, d16.data(), d16.size() * sizeof(int16_t), cudaMemcpyHostToDevice, h->stream));
  }
  if (!pid.empty() && !ptab.empty()) {
    g->npat = (int32_t)pptr.size() - 1;
    TRY(dalloc(&g->pid, pid.size()));
    TRY(dalloc(&g->pptr, pptr.size()));
    TRY(dalloc(&g->ptab, ptab.size()));
    CU(cudaMemcpyAsync(g->pid, pid.data(), pid.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(g->pptr, pptr.data(), pptr.size() * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CU(cudaMemcpyAsync(g->ptab, ptab.data(), ptab.size() * sizeof(int16_t), cudaMemcpyHostToDevice, h->stream));
  }
  CU(cudaMemcpyAsync(g->params, prm.data(), prm.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  CU(cudaMemsetAsync(g->m, 0, gnn::NPARAM * sizeof(float), h->stream));
  CU(cudaMemsetAsync(g->v, 0, gnn::NPARAM * sizeof(float), h->stream));
  CU(cudaMemsetAsync(g->scount, 0, sizeof(unsigned), h->stream));
  CU(cudaMemsetAsync(g->z, 0, 3 * (size_t)h->N * sizeof(float), h->stream));
  CU(cudaMemsetAsync(g->rprev, 0, 3 * (size_t)h->N * sizeof(float), h->stream));
  gnn::launch_pack(g->params, g->Wb, h->stream);
  return sync(h);
}

int sfem_gnn_set_loss(sfem_handle* h, int32_t mode) {
  TRY(check_handle(h));
  TRY(gnn_need(h));
  if (mode != 0 && mode != 1) return fail(SFEM_ERR_INVALID, "loss mode is 0 (energy) or 1 (residual)");
  h->gnn->loss_mode = mode;
  return SFEM_OK;
}

int sfem_gnn_set_inference(sfem_handle* h, int32_t mode) {
  TRY(check_handle(h));
  TRY(gnn_need(h));
  if (mode != 0 && mode != 1) return fail(SFEM_ERR_INVALID, "inference mode is 0 (folded polynomial) or 1 (layers)");
  h->gnn->infer_mode = mode;
  return SFEM_OK;
}

int sfem_gnn_graph_form(sfem_handle* h, int32_t* form, int32_t* patterns) {
  TRY(check_handle(h));
  TRY(gnn_need(h));
  const GnnState* g = h->gnn;
  if (form) *form = g->pid ? 2 : g->d16 ? 1 : 0;
  if (patterns) *patterns = g->npat;
  return SFEM_OK;
}

int sfem_gnn_set_batch(sfem_handle* h, int32_t batch) {
  TRY(check_handle(h));
  TRY(gnn_need(h));
  if (batch < 1 || batch > 4096) return fail(SFEM_ERR_INVALID, "batch must be in [1, 4096]");
  h->gnn->batch = batch;
  return SFEM_OK;
}

int sfem_gnn_get_params(sfem_handle* h, float* params) {
  TRY(check_handle(h));
  TRY(gnn_need(h));
  CU(cudaMemcpyAsync(params, h->gnn->params, gnn::NPARAM * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

int sfem_gnn_set_params(sfem_handle* h, const float* params) {
  TRY(check_handle(h));
  TRY(gnn_need(h));
  CU(cudaMemcpyAsync(h->gnn->params, params, gnn::NPARAM * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  gnn::launch_pack(h->gnn->params, h->gnn->Wb, h->stream);
  h->gnn->pc_dirty = true;
  h->gnn->adam_t = 0;
  CU(cudaMemsetAsync(h->gnn->m, 0, gnn::NPARAM * sizeof(float), h->stream));
  CU(cudaMemsetAsync(h->gnn->v, 0, gnn::NPARAM * sizeof(float), h->stream));
  return sync(h);
}

// M(r) at the current state (Jacobi diagonal of the current tangent); free-DOF vectors
int sfem_gnn_apply(sfem_handle* h, const double* r_free, double* out_free) {
  TRY(check_handle(h));
  TRY(set_device(h));
  TRY(gnn_need(h));
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  KrylovWs<float>& w = h->k32;
  launch_convert<double, float>(3 * h->N, h->u, w.u, h->stream);
  TRY(gnn_refresh_diag(h));
  CU(cudaMemcpyAsync(h->tmp64 + o, r_free, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_convert<double, float>((int64_t)n, h->tmp64 + o, w.r + o, h->stream);
  TRY(gnn_poly_refresh(h));
  gnn_apply_dev(h, w.r + o, h->gnn->z + o, nullptr, false);
  launch_convert<float, double>((int64_t)n, h->gnn->z + o, h->tmp64b + o, h->stream);
  CU(cudaMemcpyAsync(out_free, h->tmp64b + o, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

// one sample's energy-norm loss ||M(r) - e||_K^2 / (e.r) and its parameter gradient
int sfem_gnn_loss_grad(sfem_handle* h, const double* r_free, const double* e_free, double* loss, float* grad) {
  TRY(check_handle(h));
  TRY(set_device(h));
  TRY(gnn_need(h));
  GnnState* g = h->gnn;
  TRY(gnn_train_buffers(h));
  const size_t o = 3 * (size_t)h->nbc, n = 3 * (size_t)h->nf;
  KrylovWs<float>& w = h->k32;
  launch_convert<double, float>(3 * h->N, h->u, w.u, h->stream);
  TRY(gnn_refresh_diag(h));
  std::vector<double> er(n);
  std::vector<double> rh(r_free, r_free + n), eh(e_free, e_free + n);
  double c = 0, rr = 0;
  for (size_t i = 0; i < n; i++) {
    c += eh[i] * rh[i];
    rr += rh[i] * rh[i];
  }
  float *rd = nullptr, *ed = nullptr, *ld = nullptr;
  TRY(dalloc(&rd, n));
  TRY(dalloc(&ed, n));
  TRY(dalloc(&ld, 1));
  CU(cudaMemcpyAsync(h->tmp64 + o, r_free, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_convert<double, float>((int64_t)n, h->tmp64 + o, rd, h->stream);
  CU(cudaMemcpyAsync(h->tmp64b + o, e_free, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_convert<double, float>((int64_t)n, h->tmp64b + o, ed, h->stream);
  int st = gnn_loss_grad_dev(h, rd, ed, (float)(1.0 / c), (float)(1.0 / rr), ld);
  float lf = 0;
  if (st == 0) {
    cudaMemcpyAsync(&lf, ld, sizeof(float), cudaMemcpyDeviceToHost, h->stream);
    if (grad) cudaMemcpyAsync(grad, g->grad, gnn::NPARAM * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
    st = sync(h);
  }
  cudaFree(rd);
  cudaFree(ed);
  cudaFree(ld);
  if (loss) *loss = lf;
  return st;
}

// Training pairs from a plain Jacobi-PCG solve (FP32) of K x = b at the current state:
// every `every` iterations the residual r_j and the iterate x_j are kept, and after the
// solve e_j = x_final - x_j is the correction that solves K e_j = r_j.  b_free == NULL
// uses the current nonlinear residual.  Appends up to max_snaps samples.
int sfem_gnn_collect(sfem_handle* h, const double* b_free, int32_t every, int32_t max_snaps, double rel_tol,
                     int32_t* n_added) {
  TRY(check_handle(h));
  TRY(set_device(h));
  TRY(gnn_need(h));
  GnnState* g = h->gnn;
  KrylovWs<float>& w = h->k32;
  const int64_t o = 3 * h->nbc, n = 3 * h->nf;
  if (every <= 0 || max_snaps <= 0) return fail(SFEM_ERR_INVALID, "every and max_snaps must be positive");
  launch_convert<double, float>(3 * h->N, h->u, w.u, h->stream);
  if (b_free) {
    CU(cudaMemcpyAsync(h->tmp64 + o, b_free, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_convert<double, float>(n, h->tmp64 + o, w.b + o, h->stream);
  } else {
    double rn;
    TRY(residual(h, &rn, nullptr));
    launch_convert<double, float>(n, h->r64 + o, w.b + o, h->stream);
  }
  TRY(jacobi<float>(h, w.dinv, nullptr));
  // snapshot buffers: r_j then x_j
  std::vector<float*> rs, xs;
  CgScalars s0;
  memset(&s0, 0, sizeof(s0));
  s0.tol2 = rel_tol * rel_tol;
  s0.max_it = 50000;  // the solve that labels the pairs; FP32 stalls below ~1e-6 relative
  *h->scal_h = s0;
  CU(cudaMemcpyAsync(h->scal, h->scal_h, sizeof(CgScalars), cudaMemcpyHostToDevice, h->stream));
  launch_cg_init<float>(n, w.b + o, w.x + o, w.r + o, w.p + o, w.dinv + o, h->red(), h->scal, h->stream);
  float* pbuf[2] = {w.p, w.p2};
  int it = 0;
  for (;;) {
    CU(cudaMemcpyAsync(h->scal_h, h->scal, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    if (h->scal_h->done) break;
    if ((int)rs.size() < max_snaps) {
      float *rj = nullptr, *xj = nullptr;
      TRY(dalloc(&rj, (size_t)n));
      TRY(dalloc(&xj, (size_t)n));
      CU(cudaMemcpyAsync(rj, w.r + o, n * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
      CU(cudaMemcpyAsync(xj, w.x + o, n * sizeof(float), cudaMemcpyDeviceToDevice, h->stream));
      rs.push_back(rj);
      xs.push_back(xj);
    }
    for (int k = 0; k < every; k++, it++) {
      float* pold = pbuf[it % 2];
      float* pnew = pbuf[(it + 1) % 2];
      hvp<float>(h, w.u, pold, w.q, h->scal, nullptr, w.r, w.dinv, pnew);
      launch_cg_update_patch<float>(h->nbc, h->N, h->bslot, reinterpret_cast<const float*>(h->partial), w.x,
                                    w.r, pnew, w.q, w.dinv, h->red(), h->scal, h->stream);
    }
  }
  // e_j = x_final - x_j, c_j = e_j . r_j
  int added = 0;
  for (size_t j = 0; j < rs.size(); j++) {
    gnn::launch_sub(n, w.x + o, xs[j], xs[j], h->stream);
    float cf = 0, rf = 0;
    gnn::launch_loss(n, xs[j], rs[j], 1.f, g->rprev + o, g->spart, g->scount, g->spart + 4000, h->stream);
    gnn::launch_loss(n, rs[j], rs[j], 1.f, g->rprev + o, g->spart, g->scount, g->spart + 4002, h->stream);
    CU(cudaMemcpyAsync(&cf, g->spart + 4000, sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CU(cudaMemcpyAsync(&rf, g->spart + 4002, sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    if (cf > 0.f && std::isfinite(cf) && rf > 0.f && std::isfinite(rf)) {
      if (h->cs_on) {
        // two-level: the network supplies M(r) beside the coarse correction C r, so it learns
        // e_j - C r_j (the loss keeps e_j . r_j as its scale)
        CU(cudaMemsetAsync(w.q + o, 0, n * sizeof(float), h->stream));
        launch_coarse_apply(h->cv(), rs[j], w.q + o, h->stream);
        gnn::launch_sub(n, xs[j], w.q + o, xs[j], h->stream);
      }
      g->R.push_back(rs[j]);
      g->Ee.push_back(xs[j]);
      g->cinv.push_back(1.f / cf);
      g->rinv.push_back(1.f / rf);
      added++;
    } else {
      cudaFree(rs[j]);
      cudaFree(xs[j]);
    }
  }
  if (n_added) *n_added = added;
  return SFEM_OK;
}

int sfem_gnn_dataset_size(sfem_handle* h, int32_t* n) {
  TRY(check_handle(h));
  TRY(gnn_need(h));
  *n = (int32_t)h->gnn->R.size();
  return SFEM_OK;
}

int sfem_gnn_clear_dataset(sfem_handle* h) {
  TRY(check_handle(h));
  TRY(gnn_need(h));
  for (float* b : h->gnn->R) cudaFree(b);
  for (float* b : h->gnn->Ee) cudaFree(b);
  h->gnn->R.clear();
  h->gnn->Ee.clear();
  h->gnn->cinv.clear();
  h->gnn->rinv.clear();
  return SFEM_OK;
}

// Adam training over the collected pairs (one sample per step, drawn with a seeded
// generator); losses (optional, host) receives every step's loss.
int sfem_gnn_train(sfem_handle* h, int32_t steps, float lr, uint64_t seed, float* losses) {
  TRY(check_handle(h));
  TRY(set_device(h));
  TRY(gnn_need(h));
  GnnState* g = h->gnn;
  if (g->R.empty()) return fail(SFEM_ERR_INVALID, "no training pairs (sfem_gnn_collect)");
  TRY(gnn_train_buffers(h));
  if (g->losses_cap < steps) {
    if (g->losses) cudaFree(g->losses);
    TRY(dalloc(&g->losses, (size_t)steps));
    g->losses_cap = steps;
  }
  KrylovWs<float>& w = h->k32;
  launch_convert<double, float>(3 * h->N, h->u, w.u, h->stream);
  TRY(gnn_refresh_diag(h));
  std::mt19937_64 rng(seed);
  for (int t = 0; t < steps; t++) {
    // gradient summed over `batch` seeded random pairs; losses[t] is the first pair's loss
    for (int b = 0; b < g->batch; b++) {
      const size_t j = (size_t)(rng() % g->R.size());
      TRY(gnn_loss_grad_dev(h, g->R[j], g->Ee[j], g->cinv[j], g->rinv[j], b == 0 ? g->losses + t : g->spart + 4003,
                            b > 0));
    }
    g->adam_t++;
    gnn::launch_adam(g->grad, g->params, g->m, g->v, lr, g->adam_t, 1.f / (float)g->batch, g->Wb, h->stream);
    g->pc_dirty = true;
    if ((t & 63) == 63) TRY(sync(h));
  }
  if (losses) CU(cudaMemcpyAsync(losses, g->losses, (size_t)steps * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  return sync(h);
}

}  // extern "C"
