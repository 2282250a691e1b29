/*
 * sfem.h -- C ABI of the GB300-native matrix-free nonlinear elasticity solver.
 *
 * Drop-in boundary for SolidFEM's FemPhysicsMatrixFree / NewtonSolver /
 * NonlinearCG / ElasticEnergy path.  The reference exposes that path as a C++
 * class, not as an FFI; every entry point below names the reference member it
 * replaces (file:line within the SolidFEM project).
 *
 * Conventions
 *  - Plain pointers and sizes; no library types cross the boundary.
 *  - Node arrays passed in "original order" are N x 3 doubles, row-major.
 *  - "Free-DOF vectors" are 3*N_f doubles in the reference's reshuffled order:
 *    fixed nodes first, then free nodes in their original relative order
 *    (FemPhysicsMatrixFree::ReshuffleFixedNodes, Source/FemPhysicsMatrixFree.cpp:229-263);
 *    entry i of a free-DOF vector is reshuffled node i + N_bc.
 *  - Host-pointer entry points copy in and out on the handle's stream and
 *    return after the result is on the host.  *_dev entry points take device
 *    pointers and are stream-ordered (asynchronous) on the handle's stream.
 *  - Every call returns an int status: 0 = OK, > 0 = ran but did not
 *    converge (see SFEM_*), < 0 = error.  sfem_last_error() gives the message.
 *  - One handle per host thread; a handle is not thread-safe.
 */
#ifndef SFEM_H
#define SFEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SFEM_OK 0
#define SFEM_NOT_CONVERGED 1      /* iteration cap reached */
#define SFEM_LINESEARCH_FAILED 2  /* backtracking gave up (reference: NewtonSolver.h:282-292) */
#define SFEM_ERR_INVALID (-1)
#define SFEM_ERR_CUDA (-2)
#define SFEM_ERR_NAN (-3)               /* reference: NewtonSolver.h:313-319 */
#define SFEM_ERR_INVERTED (-4)          /* reference: FemPhysicsBase::CheckForInversion */
#define SFEM_ERR_OOM (-5)
#define SFEM_ERR_BREAKDOWN (-6)         /* CG curvature p.Ap <= 0 */
#define SFEM_ERR_NO_DEVICE (-7)
#define SFEM_ERR_TIMEOUT (-8)           /* a bounded device-side wait gave up */

/* ---- material models: values of MaterialModelType, Include/FemDataStructures.h:90-105 ---- */
#define SFEM_MMT_LINEAR 0
#define SFEM_MMT_STVK 1
#define SFEM_MMT_COROTATIONAL 2
#define SFEM_MMT_NEO_HOOKEAN 3
/* the other MaterialModelType values (FemDataStructures.h:93-107), FP64 handles; their tangent is
 * the reference's ElasticEnergy::ComputeLocalForceDifferential (ElasticEnergy.cpp:412-479) */
#define SFEM_MMT_NEO_HOOKEAN_OGDEN 4
#define SFEM_MMT_DISTORTIONAL_LINEAR 5
#define SFEM_MMT_DISTORTIONAL_MOONEY 6
#define SFEM_MMT_DISTORTIONAL_NH2 7
#define SFEM_MMT_DISTORTIONAL_NH3 8
#define SFEM_MMT_DISTORTIONAL_BW 9
#define SFEM_MMT_DISTORTIONAL_OGDEN 10
#define SFEM_MMT_DISTORTIONAL_NH6 11
#define SFEM_MMT_DISTORTIONAL_NH7 12

/* ---- precision of the element kernels and the inner Krylov solve ---- */
#define SFEM_FP64 0
#define SFEM_FP32 1 /* FP32 element kernels + CG; FP64-accurate Newton residual, FP64 convergence test */

/* ---- tangent used by the Hessian-vector product ---- */
#define SFEM_TANGENT_REFERENCE 0 /* the reference's force differential (FemPhysicsMatrixFree.cpp:436-470) */
#define SFEM_TANGENT_EXACT 1     /* exact derivative of the force; differs only for corotational,
                                    whose reference differential assumes a true polar R */

/* ---- preconditioners ---- */
#define SFEM_PC_NONE 0   /* reference SolveConjugateGradientMF with usePrecond=false */
#define SFEM_PC_JACOBI 1 /* per-DOF diagonal of the element tangents */
#define SFEM_PC_LEARNED 2 /* graph-network preconditioner in flexible PCG (sfem_gnn_*) */

/* ---- line-search conditions: values of LSCondition, Include/NewtonSolver.h:54-58, plus one ---- */
#define SFEM_LSC_ARMIJO 0        /* energy decrease (reference: mOptimizer merit) */
#define SFEM_LSC_ENGINEERING 1   /* Bonet-Wood condition as coded in NewtonSolver.h:257-261 */
#define SFEM_LSC_RESIDUAL 2      /* |r(x + a d)| <= (1 - 1e-4 a) |r(x)| */

typedef struct sfem_handle sfem_handle;

/* Replaces FemConfig (Include/FemDataStructures.h:131-156) for this path. */
typedef struct {
  double young;       /* mYoungsModulus */
  double poisson;     /* mPoissonRatio */
  double density;     /* mDensity */
  double gravity[3];  /* mGravity as a vector (reference: scalar + mZUpAxis, FemPhysicsBase.cpp:30-33) */
  int32_t material;   /* SFEM_MMT_* (mMaterial) */
  int32_t precision;  /* SFEM_FP64 / SFEM_FP32 */
  int32_t device;     /* CUDA device ordinal */
  int32_t tangent;    /* SFEM_TANGENT_* */
} sfem_config;

typedef struct {
  double rel_tol;     /* stop when |r| <= rel_tol |b| (reference eps on r.z, IterativeSolvers.h:184) */
  int32_t max_iters;  /* mInnerIterations */
  int32_t precond;    /* SFEM_PC_* */
  int32_t check_every;/* host convergence poll interval (iterations); 0 = default */
  int32_t reserved;
} sfem_pcg_opts;

typedef struct {
  int32_t iters;
  int32_t status;
  double rel_res;     /* final |r| / |b| of the Krylov recurrence */
} sfem_pcg_stats;

/* Replaces NewtonSolverBackTrack's fields (Include/NewtonSolver.h:77-93) and
 * FemPhysicsMatrixFree::SolveNewtonCG's loop (Source/FemPhysicsMatrixFree.cpp:604-628). */
typedef struct {
  double rel_tol;        /* converge when |r(x)| <= rel_tol |r(x_0)| (FP64 residual) */
  double abs_tol;        /* ... or |r(x)| <= abs_tol (mResidualThreshold); 0 disables */
  int32_t max_newton;    /* mNumIterations */
  int32_t max_cg;        /* per inner solve (mInnerIterations) */
  double eta_max;        /* inexact-Newton forcing term cap (0 -> 0.5) */
  double eta_min;        /* forcing term floor (0 -> 1e-10 FP64, 1e-5 FP32) */
  int32_t precond;       /* SFEM_PC_* */
  int32_t ls_condition;  /* SFEM_LSC_* */
  int32_t max_bisection; /* backtracking halvings (mMaxBisection; 0 -> 30) */
  int32_t verbose;
  int32_t load_steps;    /* >1: quasi-static force-fraction ramp (ST_QUASI_STATIC, FemPhysicsMatrixFree.cpp:333-340) */
  int32_t reserved;
} sfem_newton_opts;

typedef struct {
  int32_t newton_iters;
  int32_t cg_iters;       /* total inner iterations */
  int32_t status;
  int32_t line_search_cuts;
  double r0;              /* |r(x_0)| */
  double rel_res;         /* |r(x)| / |r(x_0)| at return */
  double seconds;         /* device time of the solve (CUDA events) */
} sfem_newton_stats;

/* ---- lifetime ---- */

/* FemPhysicsMatrixFree::FemPhysicsMatrixFree (Source/FemPhysicsMatrixFree.cpp:71-213) with
 * the orientation fix of FemBody::Prepare (Source/FemBody.cpp:127-156) and the fixed-node
 * flags of PyNonlinearFEM's constructor (PySolidFEM/PyNonlinearFEM.cpp:48-55).
 * nodes: N x 3; tets: E x 4 (0-based); fixed: node indices. */
int sfem_create(const double* nodes, int64_t n_nodes, const int32_t* tets, int64_t n_tets,
                const int32_t* fixed, int64_t n_fixed, const sfem_config* cfg, sfem_handle** out);
int sfem_destroy(sfem_handle* h);
/* Last error message of this thread (never NULL). */
const char* sfem_last_error(void);

/* ---- queries ---- */
/* GetNumNodes / GetNumFreeNodes / GetNumElements (Include/FemPhysicsMatrixFree.h:74-77) */
int sfem_sizes(const sfem_handle* h, int64_t* n_nodes, int64_t* n_free, int64_t* n_tets);
/* mReshuffleMap (Include/FemPhysicsBase.h:173): original -> reshuffled node index */
int sfem_reshuffle_map(const sfem_handle* h, int32_t* map);
/* the CUDA stream the handle's work is ordered on (cudaStream_t) */
int sfem_get_stream(const sfem_handle* h, void** stream);
int sfem_set_stream(sfem_handle* h, void* stream);

/* ---- state ---- */
/* GetDeformedPosition / SetDeformedPosition for all nodes, original order
 * (Include/FemPhysicsMatrixFree.h:69-71; PyNonlinearFEM::GetNodes, PyNonlinearFEM.cpp:145-159). */
int sfem_get_positions(sfem_handle* h, double* pos);
int sfem_set_positions(sfem_handle* h, const double* pos);
/* Free-node positions in reshuffled order (UpdatePosAndComputeGradients' input,
 * Source/FemPhysicsMatrixFree.cpp:562-568). */
int sfem_get_free_positions(sfem_handle* h, double* pos_free);
int sfem_set_free_positions(sfem_handle* h, const double* pos_free);
/* SetLameParams (Include/FemPhysicsBase.h:106-114). */
int sfem_set_lame_params(sfem_handle* h, double mu, double lambda);
/* mForceFraction (Include/FemPhysicsBase.h:176). */
int sfem_set_force_fraction(sfem_handle* h, double f);
/* Extension (no reference counterpart: material parameters are scalars,
 * Include/FemPhysicsBase.h:152-155): per-element Young's modulus, original element
 * order; NULL restores the uniform modulus. */
int sfem_set_element_youngs(sfem_handle* h, const double* young_e);
/* FemPhysicsMatrixFree::SetBoundaryConditionsSurface (Source/FemPhysicsMatrixFree.cpp:1051-1060):
 * follower pressure on triangles (n_tris x 3 original node indices), applied as in
 * ComputePressureForces (:967-1049): ff * (area/3) * pressure * unit normal per triangle node
 * at the current positions.  Its stiffness is not part of the Hessian-vector product (as in the
 * reference's MatrixVectorMultiply).  NULL / 0 removes the surface. */
int sfem_set_pressure_surface(sfem_handle* h, const int32_t* tris, int64_t n_tris, double pressure);
/* Extension: per-element Lame parameters (caller's element order), e.g. bodies with their own
 * Young's modulus and Poisson ratio in one mesh; NULL restores the uniform parameters. */
int sfem_set_element_lame(sfem_handle* h, const double* mu_e, const double* lambda_e);
/* Extension: the mesh is a union of k independent bodies; body q owns the caller's nodes
 * [node_offsets[q], node_offsets[q+1]) (node_offsets[0] = 0, node_offsets[k] = N).  Every kernel
 * launch still covers all bodies; sfem_newton_solve converges each body against its own initial
 * residual and masks converged bodies (zero right-hand side and Jacobi inverse) while the others
 * continue.  k = 0 removes the instances. */
int sfem_set_instances(sfem_handle* h, int32_t k, const int64_t* node_offsets);
/* per-body |r_q| / |r_q(x_0)| and Newton iterations of the last sfem_newton_solve */
int sfem_instance_stats(const sfem_handle* h, double* rel_res, int32_t* newton_iters);
/* Krylov solves of a handle with instances (materials 0, 1, 3): mode 1 (default) runs every
 * instance's own PCG recurrence -- its own alpha, beta, r.z and stop test rr <= tol^2 bb, as
 * SolveConjugateGradientMF (Math/IterativeSolvers.h:115-195) runs per body -- in one persistent
 * cooperative kernel per solve (element products, node gather, updates and directions between grid
 * barriers whose waits are bounded); mode 0 runs one recurrence over all instances (converged
 * instances masked between Newton steps). */
int sfem_set_batched_pcg(sfem_handle* h, int32_t mode);
/* Per instance, of the last batched PCG solve: iterations, status (1 converged, 2 non-positive
 * curvature, 3 iteration cap) and |r| / |b|. */
int sfem_instance_pcg_stats(const sfem_handle* h, int32_t* iters, int32_t* status, double* rel_res);
/* Bound of the device-side waits (grid barriers) of the persistent kernels: `limit` polls of at
 * least 64 ns each (default 2e7), after which the kernel stops and the call returns
 * SFEM_ERR_TIMEOUT; test != 0 makes the next launches first wait for a flag that nothing sets, so
 * that the limit is reached (a self-test of the error path that faults nothing). */
int sfem_set_device_wait(sfem_handle* h, int64_t limit, int32_t test);
/* Extension (FemPhysicsBase::SetExternalForces is an ASSERT stub, Include/FemPhysicsBase.h:68):
 * dead nodal loads, N x 3 original order, added to the residual scaled by mForceFraction. */
int sfem_set_nodal_loads(sfem_handle* h, const double* f);

/* ---- physics ---- */
/* FemPhysicsMatrixFree::ComputeGradients (Source/FemPhysicsMatrixFree.cpp:536-560), static:
 * r = f_int + m g ff + f_ext ff over free DOFs.  norm (optional) receives |r|_2 in FP64. */
int sfem_compute_gradients(sfem_handle* h, double* r, double* norm);
/* FemPhysicsMatrixFree::MatrixVectorMultiply (Source/FemPhysicsMatrixFree.cpp:523-534),
 * static: Kd = -ComputeForceDifferential(d) (:406-496).  FP64. */
int sfem_matvec(sfem_handle* h, const double* d, double* Kd);
/* FemPhysicsMatrixFree::DotProduct (Include/FemPhysicsMatrixFree.h:89). */
int sfem_dot(sfem_handle* h, const double* a, const double* b, double* out);
/* Per-DOF diagonal of the tangent: diagonal of the local stiffness matrices of
 * ElasticEnergy::ComputeLocalStiffnessMatrixFromDifferential (Source/ElasticEnergy.cpp:493-517)
 * summed per node (3 N_f). */
int sfem_jacobi_diagonal(sfem_handle* h, double* diag);
/* FemPhysicsBase::ComputeElasticEnergy (Source/FemPhysicsBase.cpp:203-212) and the total
 * potential (elastic - (m g + f_ext) . x, full gravity vector; cf. FemPhysicsMatrixFree::ComputeEnergy
 * :882-916 which uses g.y only). */
int sfem_energy(sfem_handle* h, double* elastic, double* total);
/* FemPhysicsBase::CheckForInversion (Source/FemPhysicsBase.cpp:93-117): elements with det F <= 0. */
int sfem_count_inverted(sfem_handle* h, int64_t* count);
/* ElasticEnergy::ComputeElementStress (Source/ElasticEnergy.cpp:114-257): PK1 per element,
 * E x 9 row-major, original element order. */
int sfem_element_stress(sfem_handle* h, double* P);
/* FemPhysicsBase::GetForceParamGrads (Source/FemPhysicsBase.cpp:162-187): free-DOF
 * d f / d mu, d f / d lambda, d f / d rho. */
int sfem_force_param_grads(sfem_handle* h, double* gmu, double* glambda, double* grho);

/* ---- solvers ---- */
/* SolveConjugateGradientMF (Math/IterativeSolvers.h:115-195) on K x = b, zero initial guess,
 * with the chosen preconditioner, in the handle's precision. b, x: free-DOF vectors. */
int sfem_pcg(sfem_handle* h, const double* b, double* x, const sfem_pcg_opts* opts, sfem_pcg_stats* stats);
/* Static equilibrium solve (FemPhysicsMatrixFree::Step(0) -> Solve -> SolveNewtonCG /
 * SolveNewtonLS, Source/FemPhysicsMatrixFree.cpp:325-331, 604-628, 733-781): globalized inexact
 * Newton with matrix-free PCG inner solves.  Updates the handle's positions. */
int sfem_newton_solve(sfem_handle* h, const sfem_newton_opts* opts, sfem_newton_stats* stats);
/* Record every line-search trial of the following Newton solves into caller-owned host memory:
 * trace[3k .. 3k+2] = (Newton iteration from 0, step length, FP64 residual norm at the trial) for
 * k < *count <= cap; *count is reset to 0 here and advanced by the solves.  trace = NULL stops it.
 * The trials are the ones NewtonSolverBackTrack::Solve (Include/NewtonSolver.h:179-348) evaluates,
 * so its bisection can be compared step by step. */
int sfem_set_newton_trace(sfem_handle* h, double* trace, int32_t cap, int32_t* count);
/* NonlinearConjugateGradientMinimizer::Solve (Include/NonlinearCG.h:51-114) with the
 * reference's constants; outer/inner iteration caps and absolute threshold as its fields. */
int sfem_nonlinear_cg(sfem_handle* h, int32_t outer_iters, int32_t inner_iters, double abs_tol,
                      int32_t* iters_done);

/* ---- differentiation (extension; the reference has only global mu/lambda/rho force
 * gradients, Source/ElasticEnergy.cpp:284-315) ---- */
/* Adjoint of the static equilibrium at the current state: solves K lam = dLdu (free DOFs)
 * and returns dL/dE_e (E x 1, original element order) and dL/df_ext (free DOFs). */
int sfem_adjoint(sfem_handle* h, const double* dLdu, double rel_tol, int32_t max_cg,
                 double* dLdE, double* dLdf);

/* ---- operator of the Krylov solves (MatrixVectorMultiply, Source/FemPhysicsMatrixFree.cpp:523-534) ----
 * SFEM_OP_MATRIX_FREE (default): the fused patch Hessian-vector product, re-forming each element's
 * tangent every iteration.  SFEM_OP_ASSEMBLED: the same tangent assembled in the handle's precision
 * (sliced ELL, 32 rows per slice) at the start of every Krylov solve (Newton step), then one streamed sparse
 * product per iteration; uses about 600 B per free node plus 480 B per element of device memory
 * (FP32; twice that in FP64), released again by sfem_set_operator(h, SFEM_OP_MATRIX_FREE).  Materials
 * 0-3 in either precision; batched instances and the other materials use the matrix-free product. */
#define SFEM_OP_MATRIX_FREE 0
#define SFEM_OP_ASSEMBLED 1
int sfem_set_operator(sfem_handle* h, int32_t op);
/* Cap on the device bytes the assembled operator may hold (0: no cap; default).  When the assembly
 * cannot get its memory (the cap, or cudaMalloc out of memory) the buffers it took are freed, the
 * Krylov solves use the matrix-free product, the call reports success and the handle does not retry
 * until sfem_set_operator or this function is called again.  No reference counterpart (the reference
 * allocates its sparse matrix on the host, ElasticEnergy.cpp:573-635). */
int sfem_set_operator_memory_limit(sfem_handle* h, int64_t bytes);
/* Device bytes the assembled operator holds, and 1 in *fallback after an assembly ran out of memory. */
int sfem_operator_info(sfem_handle* h, int64_t* bytes, int32_t* fallback);

/* ---- arithmetic of the nonlinear residual (ElasticEnergy::ComputeForces, Source/ElasticEnergy.cpp:170-186
 * neo-Hookean stress; the energy of :80-86 for the line search) ----
 * SFEM_RESIDUAL_TWO_TERM (default for SFEM_FP32 handles, neo-Hookean, no batched instances): the element
 * forces and energy in two-term FP32 arithmetic (about 48 significant bits, evaluated on H = F - I so
 * that no term of order one cancels), summed per node in the same arithmetic and converted to FP64 once;
 * element forces within about 1e-12 of their largest entry at any strain (the FP64 pass: about 1e-15 at
 * large strains, 1e-8 at strains of 1e-6, where F - F^-T cancels), on the FP32 pipes; it keeps the low
 * parts of X and V (40 B per element)
 * on the device, and a handle whose device has no room for them uses the FP64 pass from then on.
 * SFEM_RESIDUAL_FP64: FP64 instructions throughout (always so for SFEM_FP64 handles and the other
 * materials).  Returns SFEM_ERR_INVALID for other modes. */
#define SFEM_RESIDUAL_FP64 0
#define SFEM_RESIDUAL_TWO_TERM 1
int sfem_set_residual_arithmetic(sfem_handle* h, int32_t mode);

/* ---- assembled tangent (ElasticEnergy::AssembleStiffnessMatrix, Source/ElasticEnergy.cpp:573-635;
 * FemPhysicsMatrixFree::ComputeSystemMatrix :700-722 adds M/h^2 for implicit dynamics) ----
 * Block CSR over the free nodes in the reshuffled free order (3 x 3 blocks, row-major), FP64,
 * at the current state; the element blocks are the tangent's columns in closed form. */
int sfem_tangent_nnz(sfem_handle* h, int64_t* nnzb);
/* rowptr: n_free + 1, colidx: nnzb, vals: 9 nnzb */
int sfem_assemble_tangent(sfem_handle* h, int32_t* rowptr, int32_t* colidx, double* vals);
/* out = K d with the assembled tangent (checks against sfem_matvec) */
int sfem_tangent_matvec(sfem_handle* h, const double* d_free, double* out_free);

/* ---- dynamics (FemPhysicsMatrixFree::Step :297-324, SubStep :371-387, MatrixVectorMultiply
 * :523-534 and ComputeGradients :536-560 with mTimeStep != 0, Solve :589-597) ----
 * Time step h of the implicit (backward Euler) terms: with h > 0 the residual gains
 * (m/h) v - (m/h^2)(x - x_start) and the tangent m/h^2 (lumped masses), as the reference's
 * matrix-free class does; h = 0 restores the static problem. */
#define SFEM_SIM_EXPLICIT 2 /* SimulationType ST_EXPLICIT */
#define SFEM_SIM_IMPLICIT 3 /* SimulationType ST_IMPLICIT */
int sfem_set_time_step(sfem_handle* h, double dt);
int sfem_get_time_step(sfem_handle* h, double* dt);
/* node velocities, original node order (N x 3); fixed nodes stay at rest */
int sfem_set_velocities(sfem_handle* h, const double* vel);
int sfem_get_velocities(sfem_handle* h, double* vel);
/* x_start = current positions (the reference's pos0 = pos at the start of Step) */
int sfem_begin_step(sfem_handle* h);
/* Step(dt) with mNumSteps = substeps.  EXPLICIT: symplectic Euler substeps on the elastic forces
 * and gravity.  IMPLICIT: x_start = x, time step dt/substeps, per substep a Newton solve (opts)
 * then v = (x - x_start)/h; the time step stays set afterwards, as in the reference. */
int sfem_step(sfem_handle* h, double dt, int32_t sim_type, int32_t substeps, const sfem_newton_opts* opts,
              sfem_newton_stats* stats);

/* ---- learned preconditioner (extension: the reference has no learned components) ----
 * A linear message-passing network S on the free-node mesh graph (3 layers, width 64, BF16
 * weights and activations, FP32 accumulation on the tensor cores) defines the symmetric
 * positive definite preconditioner M(r) = D^-1/2 (c x + S^T S x), x = D^-1/2 r, c > 0; it
 * replaces Jacobi inside flexible (Polak-Ribiere) PCG when sfem_newton_opts.precond =
 * SFEM_PC_LEARNED.  FP32 handles only.  Parameter vector layout: sfem_gnn_num_params floats
 * [We(64x3) {Wl(64x128)} x3 log_c]. */
int sfem_gnn_num_params(int32_t* n);
int sfem_gnn_init(sfem_handle* h, uint64_t seed);
int sfem_gnn_get_params(sfem_handle* h, float* params);
int sfem_gnn_set_params(sfem_handle* h, const float* params);
/* M(r) at the current state (uses the current Jacobi diagonal); free-DOF vectors */
int sfem_gnn_apply(sfem_handle* h, const double* r_free, double* out_free);
/* training objective: 0 = energy norm of the error ||M(r) - e||_K^2 / (e . r) (default),
 * 1 = residual norm ||K M(r) - r||^2 / (r . r) */
int sfem_gnn_set_loss(sfem_handle* h, int32_t mode);
/* the loss of one residual/correction pair and its parameter gradient */
int sfem_gnn_loss_grad(sfem_handle* h, const double* r_free, const double* e_free, double* loss, float* grad);
/* residual/correction pairs (r_j, x_final - x_j) from a plain Jacobi-PCG solve of K x = b
 * (b_free NULL: the current nonlinear residual), one every `every` iterations, appended to
 * the handle's training set */
int sfem_gnn_collect(sfem_handle* h, const double* b_free, int32_t every, int32_t max_snaps, double rel_tol,
                     int32_t* n_added);
int sfem_gnn_dataset_size(sfem_handle* h, int32_t* n);
int sfem_gnn_clear_dataset(sfem_handle* h);
/* how M(r) is evaluated inside the solver and by sfem_gnn_apply: 0 (default) = the network
 * folded into its polynomial form S^T S x = sum_{j,k} (A^T)^j (A^k x) G_kj with 3x3 blocks
 * G_kj (exact, since S is linear; six passes over 3-vectors), 1 = the six BF16 tensor-core
 * layer kernels.  Training always runs the layer kernels. */
int sfem_gnn_set_inference(sfem_handle* h, int32_t mode);
/* how the polynomial passes find a node's neighbours: *form = 2 (a pattern table shared by
 * nodes with equal neighbour-delta lists, *patterns entries), 1 (16-bit deltas per node) or
 * 0 (32-bit indices); the three give the same neighbours in the same order */
int sfem_gnn_graph_form(sfem_handle* h, int32_t* form, int32_t* patterns);
/* pairs per Adam step (gradient averaged over them); default 1 */
int sfem_gnn_set_batch(sfem_handle* h, int32_t batch);
/* Adam on the collected pairs, `batch` seeded random pairs per step; losses: steps floats
 * (optional), the first pair's loss of each step */
int sfem_gnn_train(sfem_handle* h, int32_t steps, float lr, uint64_t seed, float* losses);

/* ---- instrumentation (no reference counterpart: the reference's PROFILE_SCOPE macros are
 * empty, Engine/Profiler.h:35-39) ---- */
typedef struct {
  double hvp_elem_ms;      /* summed CUDA-event time of sampled element Hessian-vector launches */
  double hvp_gather_ms;    /* summed time of the matching node gathers */
  int64_t samples;         /* number of sampled launches */
  int64_t hvp_launches;    /* all element Hessian-vector launches since profiling was enabled */
  double algo_bytes_hvp;   /* algorithmic bytes of one launch: E (16 + 10 s) + N (9 s) */
  int32_t precision;       /* precision of the sampled launches (SFEM_FP64 / SFEM_FP32) */
  int32_t reserved;
} sfem_profile;
/* enable != 0 resets the counters and samples one Hessian-vector product per poll interval
 * of every Krylov solve, timed with CUDA events on the handle's stream. */
int sfem_set_profiling(sfem_handle* h, int32_t enable);
int sfem_get_profile(const sfem_handle* h, sfem_profile* out);
/* Total number of kernels this library has launched in the process. */
int sfem_kernel_launches(int64_t* count);

/* ---- allocation-free reduction (no counterpart in the reference) ----
 * For callers that cannot call cudaMalloc where they need a reduction: code running inside a
 * CUDA stream capture (allocation is not capturable and synchronises the device), control
 * loops that forbid allocation after start-up, and host applications that plan all device
 * memory themselves.  Computes out_dev[0] = sum_i a_dev[i] * b_dev[i] (device pointers),
 * ordered on `stream`.  The sum is deterministic (the same bits on every run: fixed 2048-entry
 * tiles, the tile partials added in index order by the last block) but its order differs from
 * sfem_dot's, so the two can differ in the last bits.  Its scratch is a
 * fixed static device array (one partial per 2048 entries + a counter, 512 KiB), held by every
 * device that loads this library until the process exits; n above 134,217,728 is rejected
 * with SFEM_ERR_INVALID.  Every call shares the array and clears its counter first, so calls
 * that overlap on the GPU race: serialise them.  The first call on a device looks the array's
 * address up (cudaGetSymbolAddress) and should come before any stream capture.  That address is
 * kept for the life of the process: after cudaDeviceReset (or any release of the device's primary
 * context) it is stale, so do not call this entry point on that device again in the process. */
int sfem_dot_noalloc_dev(const double* a_dev, const double* b_dev, int64_t n, double* out_dev, void* stream);

/* ---- coarse space (extension; the reference's SolveConjugateGradientMF,
 * Math/IterativeSolvers.h:115-195, has none): the host-side factors of the two-level preconditioner
 * (sfem_set_coarse_space below), exposed for checking.
 * X: n points (3n doubles, e.g. free-node rest positions); aggregates are the cells of a uniform
 * grid of spacing `cell` anchored at the points' minimum corner, numbered in increasing cell order
 * (aid: n).  d: 3n, each point's offset from its aggregate's centroid.  R (optional, 36 * n_agg
 * doubles, row-major 6 x 6 per aggregate): the aggregate's rigid-body modes B_i = [I, -[d_i]x]
 * orthonormalised, P_i = B_i R_a, R_a = diag(I / sqrt(n_a), V L^-1/2) from the eigenpairs of the
 * aggregate's inertia tensor; rotations with eigenvalue <= rtol * the largest are dropped (zero
 * columns).  Call with R = NULL to learn n_agg.  No device work. */
int sfem_coarse_factors(const double* X, int64_t n, double cell, double rtol, int32_t* aid, double* d,
                        double* R, int64_t* n_agg);
/* The same aggregates with polynomial modes: per displacement component k the F features of the offset
 * (degree 1: F = 4, 1, dx, dy, dz, the affine motions u = t + A d_i; degree 2: F = 10, also dx^2, dy^2,
 * dz^2, dx dy, dy dz, dz dx), column F k + m of node i's block giving component k the feature f_m(d_i),
 * orthonormalised: R (optional, (3F)^2 * n_agg doubles, row-major per aggregate) = I (x) V L^-1/2 from
 * the eigenpairs of the features' Gram matrix (formed on d / the aggregate's largest |d|, the scaling
 * folded into R; column 3 j + k: component k of the j-th eigenvector, largest first), modes of eigenvalue
 * <= max(rtol, 1e-3) * the largest dropped (zero columns, last: the floor drops nearly dependent modes,
 * e.g. a quadratic feature along an aggregate's thin direction).  No device work. */
int sfem_coarse_factors_poly(const double* X, int64_t n, double cell, double rtol, int32_t degree, int32_t* aid,
                             double* d, double* R, int64_t* n_agg);

/* Two-level preconditioner for the learned flexible CG of FP32 handles (extension: the reference's
 * SolveConjugateGradientMF, Math/IterativeSolvers.h:115-195, has no coarse space):
 * z = M(r) + P Kc^-1 P^T r, P the rigid-body modes of grid-cell aggregates of the free nodes (cell:
 * the grid spacing; rtol as in sfem_coarse_factors), Kc = P^T K P from the FP64 tangent at the rest
 * state, inverted once here (dense, FP64 Cholesky on the host threads) and applied as one
 * matrix-vector product per iteration (W = R Kc^-1 R^T stored in FP16 times a power of two, FP32 sums).
 * cell <= 0 turns it off.  At most 2048 aggregates. */
int sfem_set_coarse_space(sfem_handle* h, double cell, double rtol);
/* The same with the aggregates' six rigid-body modes (modes = 6: sfem_set_coarse_space), twelve affine
 * modes (modes = 12) or thirty quadratic ones (modes = 30; sfem_coarse_factors_poly of degree 1 or 2).
 * At most 2048 aggregates and 12,288 coarse modes. */
int sfem_set_coarse_space_modes(sfem_handle* h, double cell, double rtol, int32_t modes);
/* z = P Kc^-1 P^T r alone (free DOFs, host arrays), for checking the coarse correction. */
int sfem_coarse_apply(sfem_handle* h, const double* r, double* z);
/* The coarse space's size and the wall-clock seconds of its setup (any pointer may be NULL):
 * n_agg aggregates, n_coarse kept modes (the order of Kc); seconds[0] the rest-state FP64 tangent
 * (pattern, assembly, copy to the host), seconds[1] Kc, seconds[2] the Cholesky factorisation, the
 * inverse and W.  Zeros when the handle has no coarse space. */
int sfem_coarse_info(sfem_handle* h, int32_t* n_agg, int32_t* n_coarse, double* seconds);

/* ---- device-pointer variants (stream-ordered on the handle's stream) ---- */
int sfem_compute_gradients_dev(sfem_handle* h, double* r_dev);
int sfem_matvec_dev(sfem_handle* h, const double* d_dev, double* Kd_dev);
int sfem_get_free_positions_dev(sfem_handle* h, double* pos_dev);
int sfem_set_free_positions_dev(sfem_handle* h, const double* pos_dev);
int sfem_set_element_youngs_dev(sfem_handle* h, const double* young_e_dev);
int sfem_set_nodal_loads_free_dev(sfem_handle* h, const double* f_free_dev);
int sfem_adjoint_dev(sfem_handle* h, const double* dLdu_dev, double rel_tol, int32_t max_cg,
                     double* dLdE_dev, double* dLdf_dev);

#ifdef __cplusplus
}
#endif

#endif /* SFEM_H */
