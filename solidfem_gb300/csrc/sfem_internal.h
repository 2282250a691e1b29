// Internal declarations shared by the host driver (sfem_host.cpp) and the
// CUDA kernels (sfem_kernels.cu).  Not part of the public ABI.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sfem_gnn.h"

namespace sfem {

enum Mode {
  MODE_FORCE = 0,    // element internal forces (12 per element)
  MODE_HVP = 1,      // element force differential of a direction p
  MODE_DIAG = 2,     // diagonal of the element tangent (12 per element)
  MODE_ENERGY = 3,   // sum of V * Psi(F)
  MODE_STRESS = 4,   // PK1 stress (9 per element, 12-stride)
  MODE_PMU = 5,      // forces of the mu-part of the neo-Hookean stress
  MODE_PLAMBDA = 6,  // forces of the lambda-part
  MODE_NODALVOL = 7,      // V/4 per element corner
  MODE_FORCE_ENERGY = 8   // MODE_FORCE and the MODE_ENERGY sum in one pass
};

// Element arrays on the device, structure-of-arrays.
//   tets:  E int4 of reshuffled node indices
//   X:     9 x E, X[k * E + e] = (Dm^-1)_{k/3, k%3} of element e
//   vol:   E signed rest volumes
//   scale: E per-element stiffness scales (E_e / E) or nullptr; scale_la the lambda
//          scales when they differ (per-element Poisson ratio)
template <typename T>
struct ElemView {
  const int4* tets;
  const T* X;
  const T* vol;
  const T* scale;     // per-element mu scale (E_e / E), or nullptr
  const T* scale_la;  // per-element lambda scale, or nullptr (then scale)
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
  int32_t jac;     // flexible CG: the next direction uses D^-1 r instead of the preconditioner output
};

// Element patches for the fused Hessian-vector product.  Elements are stored in
// patch order (Morton order of centroids, cut into patches of at most
// kPatchElems elements touching at most kPatchNodes distinct nodes).  Per patch:
//   elem_off[c] .. elem_off[c+1]   its elements
//   node_off[c] .. node_off[c+1]   its node slots; pnode[slot] = global node id,
//                                  or ~id if the node belongs to several patches
//   lptr[node_off[c] + c + j]      local CSR: entries lent[4 elem_off[c] + t] = shared-memory
//                                  offset kFeStride * local element + 3 * corner, element order
//   lidx[e]                        local node ids of element e's four corners
// Shared free nodes are summed by a second pass over bnode/bptr/bslot.
template <typename T>
struct PatchView {
  const int64_t* elem_off;
  const int64_t* node_off;
  const int32_t* pnode;
  const int32_t* pdest;  // shared free node slot -> its position in the boundary partial array, else -1
  const uint16_t* lptr;
  const uint16_t* lent;
  const ushort4* lidx;
  const T* X;
  const T* vol;
  const T* scale;
  const T* scale_la;
  int64_t E;
  int64_t n_patches;
  int64_t nbc;
  T mu, lambda;
  const T* pm;   // implicit dynamics: per slot m_g / (h^2 * patches sharing g), else nullptr
  const T* nhc;  // neo-Hookean tangent cache (k_nh_cache, 12 E values) valid for this solve, or nullptr
  int max_nodes;  // the largest node count of a patch (sizes the shared-memory node arrays)
  const T* rec;   // per element 12 values: X (9), vol, the local corners' 8 bytes, padding (16-byte rows)
  const uint16_t* lent12;  // the local CSR entries as offsets 12 * local element + 3 * corner (FP32 neo-Hookean
                           // product, results over the 12-value records), or nullptr
};

// Implicit-dynamics terms of the residual (FemPhysicsMatrixFree::ComputeGradients :546-557):
// r += (m/h) v - (m/h^2) (x - x_start); vel == nullptr for static solves
struct DynView {
  const double* vel;      // 3N, reshuffled
  const double* u_start;  // displacement at the start of the step, 3N
  double inv_h, inv_h2;
};

struct PatchBoundary {
  int64_t n;             // shared free nodes
  const int32_t* node;   // n
  const int32_t* ptr;    // n + 1: node i's partials are partial[3 ptr[i] .. 3 ptr[i+1]) in patch order
};

struct Reduce {
  double* partials;   // >= kMaxBlocks * 4 doubles
  unsigned* counter;  // zero-initialised
};

unsigned long long launch_count();
void count_launch();  // every kernel launcher of the library calls this once per launch
// records the thread's last error message (sfem_last_error) and returns code
int set_error(int code, const char* msg);

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 2048;

// ---- element passes ----
template <typename T, int MAT>
void launch_element(int mode, const ElemView<T>& ev, const T* u, const T* p, T* fe, Reduce red,
                    double* result, int* n_inverted, const CgScalars* s, cudaStream_t st);

// FP32 neo-Hookean patch product with the records staged by a bulk asynchronous copy (sfem_patch_nh32.cu)
size_t patch_hvp_nh32_smem(int max_nodes);
void launch_patch_hvp_nh32(const PatchView<float>& pv, const float* u, const float* p, float* q, float* partial,
                           Reduce red, CgScalars* s, cudaStream_t st, const float* r, const float* dinv, float* p_new,
                           const float* z);

constexpr int kPatchElems = 768;
constexpr int kPatchNodes = 512;
constexpr int kFeStride = 13;  // odd row stride of the element results in shared memory

// ---- fused patch Hessian-vector product: q = K p (negated force differential) ----
// writes q for nodes owned by one patch and partials for shared nodes; the
// boundary pass completes q and the p.q reduction (alpha, as the HVP gather).
// With r, dinv and p_new given (Krylov iterations), the kernel first forms the search
// direction p_new = dinv * r + beta * p (beta from s; p is the previous direction) for the
// nodes it stages, writes it for every free node it touches and multiplies that; otherwise
// it multiplies p.
template <typename T, int MAT>
void launch_patch_hvp(const PatchView<T>& pv, PatchBoundary pb, const T* u, const T* p, T* q, T* partial,
                      Reduce red, CgScalars* s, cudaStream_t st, cudaEvent_t mid = nullptr, const T* r = nullptr,
                      const T* dinv = nullptr, T* p_new = nullptr, const T* z = nullptr);

// fused Krylov update for the patch product (assembles q at shared nodes: bslot[g] = (first
// partial slot, count), count 0 for nodes of one patch); with xs, also the preconditioner's
// input rows sigma D^-1/2 r of the free nodes (FP16, gnn::Row16), sigma from the sum of d r^2 that
// the previous update left in xstat[0]; the update leaves sigma in xstat[1] and its own sum in
// xstat[0].  With cv (the two-level preconditioner) and q complete (bslot null), the same pass also
// forms the coarse restriction's run sums (k_coarse_runs' output) and the call returns true.
struct CoarseView;
template <typename T>
bool launch_fcg_update_patch(int64_t nbc, int64_t N, const int2* bslot, const T* partial, T* x, T* r, T* rprev,
                             const T* p, const T* q, Reduce red, CgScalars* s, cudaStream_t st,
                             const T* dinv = nullptr, gnn::Row16* xs = nullptr, float* xstat = nullptr,
                             const CoarseView* cv = nullptr);
template <typename T>
void launch_cg_update_patch(int64_t nbc, int64_t N, const int2* bslot, const T* partial, T* x, T* r, const T* p,
                            const T* q, const T* dinv, Reduce red, CgScalars* s, cudaStream_t st);

// ---- node gathers (FP64 residual / T HVP / T diagonal) ----
// follower pressure (FemPhysicsMatrixFree::ComputePressureForces): per triangle the force
// ff * (area / 3) * pressure * unit normal at the current positions, summed per node
struct PressureView {
  int64_t n_tris;
  const int32_t* tri;   // 3 per triangle, reshuffled node indices
  const int32_t* tptr;  // node -> triangle CSR (N + 1)
  const int32_t* tent;
  double* ptf;          // 3 per triangle (scratch)
  double pressure;
};
void launch_pressure_tris(PressureView pv, const double* x0, const double* u, double ff, cudaStream_t st);
void launch_gather_force(int64_t nbc, int64_t N, NodeCsr csr, const double* fe, const double* mass,
                         const double* fext, const double* grav, double ff, double* r, Reduce red,
                         double* rr_out, cudaStream_t st, const PressureView* pv = nullptr,
                         const DynView* dv = nullptr, const double* u = nullptr, bool fe_df = false);
// The element geometry as two-term FP32 values: the FP32 copies of X and V and their low parts.
struct DfGeom {
  const float* Xhi;    // 9 x E
  const float* Xlo;    // 9 x E, RN(X - Xhi)
  const float* volhi;  // E
  const float* vollo;  // E
};
// neo-Hookean element forces (+ energy sum) to FP64 accuracy in two-term FP32 arithmetic; fe holds
// 12 (hi, lo) pairs per element
void launch_element_nh_df(bool energy, const ElemView<double>& ev, const DfGeom& dg, const double* u, float2* fe,
                          Reduce red, double* result, int* n_inverted, cudaStream_t st);
void launch_split_geom(int64_t n, const double* x, const float* hi, float* lo, cudaStream_t st);
template <typename T>
void launch_gather_hvp(int64_t nbc, int64_t N, NodeCsr csr, const T* fe, const T* p, T* q, Reduce red,
                       CgScalars* s, cudaStream_t st);
template <typename T>
void launch_gather_diag(int64_t nbc, int64_t N, NodeCsr csr, const T* fe, T* dinv, T* diag,
                        cudaStream_t st, const double* mass = nullptr, double inv_h2 = 0.0);
// per-element forces of the FP64 force pass in element-major 12-vectors are
// reused by the adjoint: g_e = sum_a lam_a . f_a / E_e
void launch_adjoint_elem(const int4* tets, int64_t E, int64_t nbc, const double* fe, const double* lam,
                         const double* young_e, const int32_t* perm, double* dLdE, cudaStream_t st);
// out[k] = in[perm[k]] (element arrays into patch order)
void launch_permute(int64_t E, const int32_t* perm, const double* in, double* out, cudaStream_t st);

// ---- Krylov vector kernels (T = float or double) ----
template <typename T>
void launch_cg_init(int64_t n, const T* b, T* x, T* r, T* p, const T* dinv, Reduce red, CgScalars* s,
                    cudaStream_t st);
template <typename T>
void launch_cg_update(int64_t n, T* x, T* r, const T* p, const T* q, const T* dinv, Reduce red,
                      CgScalars* s, cudaStream_t st);
template <typename T>
void launch_cg_direction(int64_t n, const T* r, const T* dinv, T* p, const CgScalars* s, cudaStream_t st);

// per-segment 2-norms of a free-DOF vector: one block per segment, fixed order
void launch_segment_norms(int k, const int64_t* seg, const double* v, double* out, cudaStream_t st);
// zero v on the DOFs of inactive segments (active[k] == 0)
template <typename T>
void launch_segment_mask(int k, const int64_t* seg, const int32_t* active, T* v, cudaStream_t st);

// ---- misc vector kernels ----
void launch_dot(int64_t n, const double* a, const double* b, Reduce red, double* out, cudaStream_t st);
void launch_potential(int64_t nbc, int64_t N, const double* x0, const double* u, const double* mass,
                      const double* fext, const double* grav, double ff, Reduce red, double* out,
                      cudaStream_t st, const DynView* dv = nullptr);
// neo-Hookean tangent factors per element (F^-T, mu_e, lambda_e, mu_e - lambda_e log J; 12 E values)
template <typename T>
void launch_nh_cache(const ElemView<T>& ev, const T* u, T* cache, cudaStream_t st);
// assembled tangent: element stiffness (144 doubles per element), block-CSR assembly over free
// nodes (slot: 16 per element, -1 for a fixed corner; dslot: diagonal block of each free node),
// block-CSR product
template <typename T, int MAT>
void launch_element_stiffness(const ElemView<T>& ev, const T* u, T* Ke, cudaStream_t st);
void launch_assemble_bsr(int64_t nbc, int64_t N, NodeCsr csr, const double* Ke, const int32_t* slot,
                         const int32_t* dslot, const double* mass, double inv_h2, double* vals, cudaStream_t st);
void launch_bsr_spmv(int64_t nrows, const int32_t* rowptr, const int32_t* col, const double* vals, const double* x,
                     double* y, cudaStream_t st);
// the same tangent in sliced ELL for the Krylov loops (32 rows per slice; block-slot t of row r is
// base[r / 32] + 32 k + r % 32, values at 9 (t - t % 32) + 32 q + t % 32, q = 3 i + c)
// element stiffness as 3 x 3 blocks of 12 slots: the ten blocks a <= b of a symmetric tangent, all
// sixteen of a corotational one (returns the block count, 10 or 16); neo-Hookean in closed form
template <typename T, int MAT>
int launch_element_stiffness_sym(const ElemView<T>& ev, const T* u, T* Ke, cudaStream_t st);
// assembly: block-slot t sums its contributions code[cptr[t] .. cptr[t+1]) (code = 16 e + 4 a + b:
// block (a, b) of element e, from Ke in the ten-block layout); with mass, (m / h^2) I on each
// diagonal block
template <typename T>
void launch_assemble_sell(int64_t nslots, const int64_t* cptr, const uint32_t* code, const T* Ke, int nb,
                          int64_t nbc, int64_t nf, const int32_t* dslot, const double* mass, double inv_h2, T* vals,
                          cudaStream_t st);
// dinv = 1 / diag over the free rows from the assembled operator's diagonal blocks
template <typename T>
void launch_sell_diag_inv(int64_t nbc, int64_t nf, const int32_t* dslot, const T* vals, T* dinv, cudaStream_t st);
// the FP32 neo-Hookean tangent the same way through 24 factors per element (Kf: 24 E floats)
// instead of its blocks: h_a = F^-T g_a, vol mu (g_a . g_b), vol (mu - lambda log J), vol lambda
constexpr int kNhFactorsHost = 24;
void launch_assemble_sell_nh32(const ElemView<float>& ev, const float* u, float* Kf, int64_t nslots, const int64_t* cptr,
                               const uint32_t* code, int64_t nbc, int64_t nf, const int32_t* dslot, const double* mass,
                               double inv_h2, float* vals, cudaStream_t st);
// q = K p over the free rows (+ p.q, alpha with s); with p_new the direction is formed on the fly,
// p = (z or D^-1 r) + beta p_old, as the patch product does
// (columns: col, free-node indices, or col16, differences to the row when every one fits 16 bits)
template <typename T>
void launch_sell_hvp(int64_t nbc, int64_t nf, const int64_t* base, const int32_t* col, const int16_t* col16,
                     const T* vals, const T* p, T* q, Reduce red, CgScalars* s, cudaStream_t st,
                     const T* r = nullptr, const T* dinv = nullptr, T* p_new = nullptr, const T* z = nullptr);
// the same product from a symmetric tangent stored as its diagonal and upper blocks (base/col/col16, as
// above), each row's lower blocks read transposed from their mirror rows: lower entry (row r, position k)
// at lbase[r / 32] + 32 k + r % 32 names the column j (lcol, or lcol16 = j - r) and the block-slot of
// block (j, r) in row j (lslot; -1: padding)
template <typename T>
void launch_ssell_hvp(int64_t nbc, int64_t nf, const int64_t* base, const int32_t* col, const int16_t* col16,
                      const int64_t* lbase, const int32_t* lcol, const int16_t* lcol16, const int32_t* lslot,
                      const T* vals, const T* p, T* q, Reduce red, CgScalars* s, cudaStream_t st,
                      const T* r = nullptr, const T* dinv = nullptr, T* p_new = nullptr, const T* z = nullptr);
// ---- coarse-space correction of the two-level preconditioner (sfem_coarse_kernels.cu) ----
// z += B W B^T r over the free block: per free node its aggregate aid[i] and offset d_i from the
// aggregate's centroid (x, y, z, 0); W the 6 n_agg square matrix R Kc^-1 R^T in FP16, scaled by a
// power of two (w_inv_scale undoes it; rows of ld halves, ld a multiple of 8); s and y two ld-long
// FP32 scratch vectors.  The restriction reads the free nodes in order, in n_blocks
// blocks that match the flexible-CG update's CTAs (256 groups of four nodes, the groups starting at
// the first node index that is a multiple of four): block b > 0 starts at free node blk_off + 1024 b,
// block 0 at 0 and the last block ends at nf (so the first also takes the blk_off <= 3 nodes before the
// first group and the last the <= 3 after the last group; at most kCoarseSpan nodes each).  Block b's
// nodes split into runs (consecutive nodes of one aggregate, at most kCoarseRun each), runs
// blk_run[b] .. blk_run[b+1] - 1, run k the nodes run_start[k] .. run_start[k+1] - 1.  A run's six sums
// go to runpart (six arrays of n_runs floats); aggregate a's runs are agg_run[agg_run_ptr[a] ..
// agg_run_ptr[a+1] - 1], in increasing order.
constexpr int kCoarseBlock = 1024;
constexpr int kCoarseSpan = 1032;
constexpr int kCoarseRun = 32;
// first free node of restriction block b (n_blocks blocks; b == n_blocks gives nf)
__host__ __device__ inline int64_t coarse_block_start(int64_t b, int64_t n_blocks, int blk_off, int64_t nf) {
  return b == 0 ? 0 : (b >= n_blocks ? nf : blk_off + (int64_t)kCoarseBlock * b);
}
struct CoarseView {
  int n_agg;
  int nm;  // modes per aggregate: 6 (rigid: y_a = (u, w), z_i += u + w x d_i, s_a = (sum r_i, sum d_i x r_i))
           // or 3 F = 12 / 30 (polynomial, F features f(d) = 1, d (, its quadratic terms): z_i[k] +=
           // sum_m y_a[F k + m] f_m(d_i), s_a[F k + m] = sum r_i[k] f_m(d_i))
  int ld;
  int64_t nf;
  const int32_t* aid;
  const float4* d;
  const __half* W;
  float w_inv_scale;
  float* s;
  float* y;
  int n_runs;
  int n_blocks;
  int blk_off;
  const int32_t* run_start;
  const int32_t* blk_run;
  const int32_t* agg_run_ptr;
  const int32_t* agg_run;
  float* runpart;
};
// the correction's prolongation, z_i += u_a + w_a x d_i with (u_a, w_a) = y_a, as a term of another
// kernel's node loop (aid == nullptr: none)
struct CoarseAdd {
  const int32_t* aid;
  const float4* d;
  const float* y;
  int nm;
};
// z += B W B^T r (restriction, coarse product, prolongation)
void launch_coarse_apply(const CoarseView& cv, const float* r, float* z, cudaStream_t st);
// y = W B^T r only (the prolongation then runs inside the preconditioner's last pass)
void launch_coarse_restrict_gemv(const CoarseView& cv, const float* r, cudaStream_t st);
// the same after the run sums are in place (the flexible-CG update formed them)
void launch_coarse_sum_gemv(const CoarseView& cv, cudaStream_t st);

// ---- batched independent bodies: one persistent kernel per Krylov solve ----
// Each instance (body) runs its own preconditioned CG recurrence (its own alpha, beta, r.z and
// convergence test: SolveConjugateGradientMF, Math/IterativeSolvers.h:115-195, per body) inside one
// cooperative launch; phases (element products, node gather + p.q, updates, directions) are separated
// by grid barriers whose waits give up after wait_limit polls and set *err.  Free nodes are grouped
// in tiles of at most 32 (one warp each) that never straddle two instances, so every per-instance sum
// is a fixed-order sum of tile partials (deterministic).
struct BatchPcg {
  int K;                    // instances
  int n_tiles;
  int64_t nbc, N;
  const int32_t* einst;     // E: instance of each element (element order of the handle)
  const int32_t* tile_node; // n_tiles: first free node (0-based among the free nodes)
  const int32_t* tile_cnt;  // n_tiles: nodes in the tile (1..32)
  const int32_t* tile_inst; // n_tiles: the tile's instance
  const int32_t* inst_tile; // K + 1: the tiles of instance k are inst_tile[k] .. inst_tile[k + 1] - 1
  double* part;             // 3 n_tiles: per-tile p.q, r.z, r.r
  double* rz;               // 2 K: r.z of the current / next iteration (by parity)
  double* tol2bb;           // K: tol^2 |b_k|^2
  int32_t* done;            // 2 K: 0 running, 1 converged, 2 non-positive curvature, 3 iteration cap, 4 non-finite
  int32_t* iters;           // K
  double* rr;               // K: final |r_k|^2
  unsigned* bar;            // 2: barrier arrival count and generation
  int32_t* err;             // 1: a wait gave up (0 ok)
  double tol;
  int max_it;
  long long wait_limit;     // polls of one barrier wait before it gives up
  int wait_test;            // 1: block 0 first waits for a flag that nothing sets (exercises the limit)
};
template <typename T>
int launch_batched_pcg(int mat, const ElemView<T>& ev, NodeCsr csr, const BatchPcg& b, const T* u, const T* rhs, T* x,
                       T* r, T* z, T* p, T* q, const T* dinv, T* fe, cudaStream_t st);
// implicit dynamics: per patch-node slot mass share m_g / (h^2 k_g) (k_g patches touch g)
template <typename T>
void launch_patch_mass(int64_t n_slots, int64_t nbc, const int32_t* pnode, const int32_t* bidx, PatchBoundary pb,
                       const double* mass, double inv_h2, T* pm, cudaStream_t st);
// explicit substep (FemPhysicsMatrixFree::SubStep :371-387): v += (h/m) f + h g, u += h v
void launch_explicit_substep(int64_t nbc, int64_t N, const double* f, const double* mass, const double* grav,
                             double hs, double* vel, double* u, cudaStream_t st);
// implicit step end (FemPhysicsMatrixFree::Solve :589-597): v = (u - u_start) / h
void launch_velocity_update(int64_t nbc, int64_t N, const double* u, const double* u_start, double inv_h,
                            double* vel, cudaStream_t st);
// node vectors between the caller's order and the reshuffled order (map: original -> reshuffled)
// in: dst[3 map[i] + c] = src[3 i + c] - sub[...] (sub optional; zero where map[i] < nzero)
void launch_nodes_in(int64_t N, const int32_t* map, const double* src, const double* sub, int64_t nzero, double* dst,
                     cudaStream_t st);
// out: dst[3 i + c] = a[3 map[i] + c] + b[...] (b optional)
void launch_nodes_out(int64_t N, const int32_t* map, const double* a, const double* b, double* dst, cudaStream_t st);
template <typename Tin, typename Tout>
void launch_convert(int64_t n, const Tin* a, Tout* b, cudaStream_t st);
// x = x + a * d   (FP64 state += precision-T direction)
template <typename T>
void launch_axpy_state(int64_t n, double a, const T* d, const double* base, double* x, cudaStream_t st);
void launch_scale_copy(int64_t n, double a, const double* x, double* y, cudaStream_t st);

}  // namespace sfem

// ---- learned preconditioner launchers (sfem_gnn.cu) ----
#include <cuda_bf16.h>

#include "sfem_gnn.h"
namespace sfem {
namespace gnn {
// M(r) over the free block: NL layers of S then NL transposed layers (encoder and output
// fused into the first and last); Wb holds the 3 packed BF16 weight sets (k_gnn_pack)
void launch_apply(const Graph& g, const float* r, const float* dinv, const float* params, const __nv_bfloat16* Wb,
                  __nv_bfloat16* const* h, float* out, const int* done, cudaStream_t st);
// the same M(r) through the folded polynomial: six gather passes over FP16 node rows (Row16)
// scaled by sigma (xstat); x4, y1, y2: n rows, w: 4 x n rows.  x4 = sigma D^-1/2 r is formed first
// (with sigma from sum d r^2) unless x_ready (the flexible-CG update wrote it and xstat).
// partials / counter: scratch of the fixed-order sums.  With s (flexible CG), the last pass also
// forms the Polak-Ribiere beta from r, rprev (like k_fcg_beta).
void launch_apply_poly(const Graph& g, const float* r, const float* dinv, const PolyCoef& pc, Row16* x4, Row16* y1,
                       Row16* y2, Row16* w, float* xstat, float* out, const int* done, cudaStream_t st,
                       float* partials, unsigned* counter, const float* rprev = nullptr, CgScalars* s = nullptr,
                       bool x_ready = false, CoarseAdd ca = CoarseAdd{nullptr, nullptr, nullptr, 6},
                       cudaEvent_t before_last = nullptr);
// x4 rows = sigma D^-1/2 r (r, dinv: 3n), sigma and sum d r^2 into xstat
void launch_scale_sqrt4(int64_t n, const float* r, const float* dinv, float* xstat, float* partials, unsigned* counter,
                        Row16* x4, cudaStream_t st);
// the same M(r) keeping the activations h0..h3 of S and x = D^-1/2 r (training)
void launch_apply_train(const Graph& g, const float* r, const float* dinv, const float* params,
                        const __nv_bfloat16* Wb, __nv_bfloat16* const* h, float* x, float* G0, float* G1, float* G2,
                        float* out, cudaStream_t st);
int launch_count_apply();
// h0 = We (v D^-1/2) (x = v D^-1/2 kept in xout when given), then the NL layers of S
void launch_encode(const Graph& g, const float* v, const float* dinv, const float* params, __nv_bfloat16* h0,
                   float* xout, const int* done, cudaStream_t st);
void launch_layers_fwd(const Graph& g, const __nv_bfloat16* Wb, __nv_bfloat16* const* h, const int* done,
                       cudaStream_t st);
// weight gradient of <cot, S x> for the activations h of S at input x, into (or added to) grad
void launch_weight_grad(const Graph& g, const __nv_bfloat16* cot, __nv_bfloat16* const* h, const float* x,
                        const __nv_bfloat16* Wb, float* G0, float* G1, float* G2, float* partial, float* grad,
                        int accumulate, cudaStream_t st);
// grad[OFF_C] (+)= dL/d(log c)
void launch_cgrad(int64_t n3, const float* Go, const float* r, const float* dinv, const float* params, float* partials,
                  unsigned* counter, float* grad, int accumulate, cudaStream_t st);
void launch_loss(int64_t n3, const float* d, const float* q, float inv_c, float* Go, float* partials,
                 unsigned* counter, float* loss, cudaStream_t st);
void launch_adam(const float* grad, float* prm, float* m, float* v, float lr, int t, float clip_scale,
                 __nv_bfloat16* Wb, cudaStream_t st);
void launch_pack(const float* prm, __nv_bfloat16* Wb, cudaStream_t st);
void launch_sub(int64_t n, const float* a, const float* b, float* d, cudaStream_t st);
// flexible CG (Polak-Ribiere) vector kernels; partials need >= 4096 floats
void launch_fcg_init(int64_t n, const float* r, const float* z, float* p, float* partials, unsigned* counter,
                     CgScalars* s, cudaStream_t st);
void launch_fcg_beta(int64_t n, const float* r, const float* rprev, const float* z, const float* dinv,
                     float* partials, unsigned* counter, CgScalars* s, cudaStream_t st);
}  // namespace gnn
}  // namespace sfem
