/*
 * TEST INFRASTRUCTURE ONLY -- the oracle.
 *
 * A plain-C (C99 + OpenMP) CPU restatement of SolidFEM's matrix-free
 * nonlinear elasticity path.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference legs load it, and only as the checker
 * or the timed CPU port; the product (solidfem_gb300) never links or calls it.
 *
 * Parity is pinned: tests/test_oracle_pin.py compares every function here
 * against the reference's own sources compiled unmodified
 * (oracle/Makefile.ref -> oracle/_ref/libsfem_ref.so) and against the golden
 * fixtures in tests/golden/ that were produced from that build.
 *
 * Arithmetic follows the reference operation by operation (3x3 row-major
 * matrices, the same association order, element-order serial scatters) so
 * that results agree bit for bit with the reference on x86-64 when compiled
 * with -ffp-contract=off.  References are to files of the SolidFEM project.
 *
 * Build: gcc -std=c99 -O2 -fopenmp -fPIC -ffp-contract=off -shared
 *        -o oracle/liboracle.so oracle/sfem_oracle.c -lm
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------- */
/* 3x3 algebra, Math/matrix3.h and Math/vector3.h semantics                */
/* ---------------------------------------------------------------------- */
typedef struct { double m[3][3]; } M3;
typedef struct { double v[3]; } V3;

static M3 m3_ident(void) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = (i == j) ? 1.0 : 0.0; return r; }
/* matrix from column vectors, matrix3.h:101-109 */
static M3 m3_cols(V3 a, V3 b, V3 c) { M3 r; for (int i = 0; i < 3; i++) { r.m[i][0] = a.v[i]; r.m[i][1] = b.v[i]; r.m[i][2] = c.v[i]; } return r; }
static V3 m3_col(const M3* a, int j) { V3 r; for (int i = 0; i < 3; i++) r.v[i] = a->m[i][j]; return r; }
static M3 m3_tr(M3 a) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = a.m[j][i]; return r; }
static M3 m3_add(M3 a, M3 b) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = a.m[i][j] + b.m[i][j]; return r; }
static M3 m3_sub(M3 a, M3 b) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = a.m[i][j] - b.m[i][j]; return r; }
static M3 m3_scale(double s, M3 a) { for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) a.m[i][j] *= s; return a; }
/* matrix3.h:330-340: C[i][j] = 0; C[i][j] += A[i][k] * B[k][j] */
static M3 m3_mul(M3 a, M3 b) {
  M3 c;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      c.m[i][j] = 0;
      for (int k = 0; k < 3; k++) c.m[i][j] += a.m[i][k] * b.m[k][j];
    }
  return c;
}
static V3 m3_mulv(M3 a, V3 v) {
  V3 r;
  for (int i = 0; i < 3; i++) { r.v[i] = 0; for (int j = 0; j < 3; j++) r.v[i] += a.m[i][j] * v.v[j]; }
  return r;
}
static double m3_trace(M3 a) { return a.m[0][0] + a.m[1][1] + a.m[2][2]; }
/* matrix3.h:206-212 */
static double m3_det(M3 a) {
  double a00 = a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1];
  double a01 = -a.m[1][0] * a.m[2][2] + a.m[2][0] * a.m[1][2];
  double a02 = a.m[1][0] * a.m[2][1] - a.m[2][0] * a.m[1][1];
  return a.m[0][0] * a00 + a.m[0][1] * a01 + a.m[0][2] * a02;
}
/* matrix3.h:234-249 (cofactor inverse) */
static M3 m3_inv(M3 a) {
  M3 r;
  r.m[0][0] = a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1];
  r.m[1][0] = -a.m[1][0] * a.m[2][2] + a.m[2][0] * a.m[1][2];
  r.m[2][0] = a.m[1][0] * a.m[2][1] - a.m[2][0] * a.m[1][1];
  r.m[0][1] = a.m[0][2] * a.m[2][1] - a.m[0][1] * a.m[2][2];
  r.m[1][1] = a.m[0][0] * a.m[2][2] - a.m[0][2] * a.m[2][0];
  r.m[2][1] = a.m[0][1] * a.m[2][0] - a.m[0][0] * a.m[2][1];
  r.m[0][2] = a.m[0][1] * a.m[1][2] - a.m[0][2] * a.m[1][1];
  r.m[1][2] = a.m[0][2] * a.m[1][0] - a.m[0][0] * a.m[1][2];
  r.m[2][2] = a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0];
  double det = a.m[0][0] * r.m[0][0] + a.m[0][1] * r.m[1][0] + a.m[0][2] * r.m[2][0];
  return m3_scale(1.0 / det, r);
}
/* matrix3.h:264-269 */
static M3 m3_skew(V3 v) {
  M3 r;
  r.m[0][0] = 0; r.m[0][1] = -v.v[2]; r.m[0][2] = v.v[1];
  r.m[1][0] = v.v[2]; r.m[1][1] = 0; r.m[1][2] = -v.v[0];
  r.m[2][0] = -v.v[1]; r.m[2][1] = v.v[0]; r.m[2][2] = 0;
  return r;
}
static double m3_ddot(M3 a, M3 b) { double s = 0; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) s += a.m[i][j] * b.m[i][j]; return s; }

static V3 v3(double x, double y, double z) { V3 r; r.v[0] = x; r.v[1] = y; r.v[2] = z; return r; }
static V3 v3_sub(V3 a, V3 b) { return v3(a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]); }
static V3 v3_scale(double s, V3 a) { return v3(s * a.v[0], s * a.v[1], s * a.v[2]); }
static double v3_dot(V3 a, V3 b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }
static V3 v3_normalized(V3 a) { double len = sqrt(v3_dot(a, a)); double s = 1.0 / len; for (int i = 0; i < 3; i++) a.v[i] *= s; return a; }
/* vector3.h:155-158 */
static V3 v3_cross(V3 a, V3 b) {
  return v3(a.v[1] * b.v[2] - b.v[1] * a.v[2], -a.v[0] * b.v[2] + a.v[2] * b.v[0], a.v[0] * b.v[1] - b.v[0] * a.v[1]);
}

/* Gram-Schmidt "polar" decomposition, Source/PolarDecomposition.cpp:37-47, 269-280 */
static void polar_qr(M3 F, M3* R, M3* U) {
  V3 r0 = v3_normalized(m3_col(&F, 0));
  V3 a1 = m3_col(&F, 1);
  V3 r1 = v3_normalized(v3_sub(a1, v3_scale(v3_dot(a1, r0), r0)));
  V3 r2 = v3_normalized(v3_cross(r0, r1));
  *R = m3_cols(r0, r1, r2);
  M3 V = m3_mul(m3_tr(*R), F);
  *U = m3_scale(0.5, m3_add(V, m3_tr(V)));
}

/* ---------------------------------------------------------------------- */
/* Problem                                                                */
/* ---------------------------------------------------------------------- */
/* MaterialModelType, Include/FemDataStructures.h:93-107 */
enum {
  MMT_LINEAR = 0, MMT_STVK = 1, MMT_COROTATIONAL = 2, MMT_NEO_HOOKEAN = 3, MMT_NEO_HOOKEAN_OGDEN = 4,
  MMT_DISTORTIONAL_LINEAR = 5, MMT_DISTORTIONAL_MOONEY = 6, MMT_DISTORTIONAL_NH2 = 7, MMT_DISTORTIONAL_NH3 = 8,
  MMT_DISTORTIONAL_BW = 9, MMT_DISTORTIONAL_OGDEN = 10, MMT_DISTORTIONAL_NH6 = 11, MMT_DISTORTIONAL_NH7 = 12
};

typedef struct {
  int n_nodes, n_tets, n_bcs, material;
  int tangent;       /* 0: the reference's force differential, 1: exact derivative of the force */
  double mu, lambda, young, density, grav[3], force_fraction;
  int* map;          /* original -> reshuffled */
  int* tets;         /* reshuffled indices, 4 per element */
  double* X;         /* Dm^-1 per element, 9 (row-major) */
  double* vol;       /* signed rest volume */
  double* escale;    /* optional per-element stiffness scale (E_e / E), may be NULL */
  double* pos;       /* current positions, reshuffled, 3N */
  double* pos0;      /* rest positions, reshuffled, 3N */
  double* inv_mass;  /* per reshuffled node */
  double* fext;      /* dead loads, reshuffled, 3N */
  int n_tris;        /* follower-pressure surface (original node indices), 3 per triangle */
  int* tris;
  double pressure;
  double time_step;  /* mTimeStep: 0 static, h > 0 backward-Euler terms */
  double* vel;       /* node velocities, reshuffled, 3N */
  double* xstart;    /* positions at the start of the step (the reference's pos0), reshuffled, 3N */
} orc_problem;

static M3 load_X(const orc_problem* p, int e) { M3 r; memcpy(r.m, p->X + 9 * (size_t)e, 9 * sizeof(double)); return r; }
static V3 node_v(const double* a, int i) { return v3(a[3 * (size_t)i], a[3 * (size_t)i + 1], a[3 * (size_t)i + 2]); }

/* Source/FemPhysicsBase.cpp:35-41 (Lame parameters) */
static void lame(double E, double nu, double* mu, double* lambda) {
  *lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
  *mu = 0.5 * E / (1.0 + nu);
}

/*
 * Construction: FemBody::Prepare orientation fix (Source/FemBody.cpp:127-156),
 * ReshuffleFixedNodes (Source/FemPhysicsMatrixFree.cpp:229-263) and the
 * per-element precompute of the constructor (:121-205).
 */
void* orc_create(const double* nodes, int n_nodes, const int* tets, int n_tets,
                 const int* fixed, int n_fixed, double young, double poisson,
                 double density, const double* gravity, int material) {
  orc_problem* p = (orc_problem*)calloc(1, sizeof(orc_problem));
  p->n_nodes = n_nodes; p->n_tets = n_tets; p->material = material;
  lame(young, poisson, &p->mu, &p->lambda);
  p->young = young;
  p->density = density;
  for (int i = 0; i < 3; i++) p->grav[i] = gravity[i];
  p->force_fraction = 1.0;
  char* is_fixed = (char*)calloc(n_nodes, 1);
  for (int i = 0; i < n_fixed; i++) is_fixed[fixed[i]] = 1;
  p->map = (int*)malloc(sizeof(int) * n_nodes);
  int k = 0;
  for (int i = 0; i < n_nodes; i++) if (is_fixed[i]) p->map[i] = k++;
  p->n_bcs = k;
  for (int i = 0; i < n_nodes; i++) if (!is_fixed[i]) p->map[i] = k++;
  p->pos = (double*)malloc(sizeof(double) * 3 * n_nodes);
  p->pos0 = (double*)malloc(sizeof(double) * 3 * n_nodes);
  p->fext = (double*)calloc(3 * (size_t)n_nodes, sizeof(double));
  p->vel = (double*)calloc(3 * (size_t)n_nodes, sizeof(double));
  p->xstart = (double*)malloc(sizeof(double) * 3 * n_nodes);
  for (int i = 0; i < n_nodes; i++)
    for (int c = 0; c < 3; c++) p->pos[3 * p->map[i] + c] = p->pos0[3 * p->map[i] + c] = nodes[3 * i + c];
  p->tets = (int*)malloc(sizeof(int) * 4 * (size_t)n_tets);
  p->X = (double*)malloc(sizeof(double) * 9 * (size_t)n_tets);
  p->vol = (double*)malloc(sizeof(double) * n_tets);
  double* masses = (double*)calloc(n_nodes, sizeof(double));
  for (int e = 0; e < n_tets; e++) {
    int t[4];
    for (int j = 0; j < 4; j++) t[j] = tets[4 * e + j];
    {
      V3 x0 = node_v(nodes, t[0]);
      M3 m = m3_cols(v3_sub(node_v(nodes, t[1]), x0), v3_sub(node_v(nodes, t[2]), x0), v3_sub(node_v(nodes, t[3]), x0));
      if (m3_det(m) / 6.0 < 0) { int s = t[0]; t[0] = t[1]; t[1] = s; }
    }
    for (int j = 0; j < 4; j++) p->tets[4 * e + j] = p->map[t[j]];
    const int* ti = p->tets + 4 * (size_t)e;
    V3 x0 = node_v(p->pos0, ti[0]);
    M3 m = m3_cols(v3_sub(node_v(p->pos0, ti[1]), x0), v3_sub(node_v(p->pos0, ti[2]), x0), v3_sub(node_v(p->pos0, ti[3]), x0));
    M3 X = m3_inv(m);
    memcpy(p->X + 9 * (size_t)e, X.m, 9 * sizeof(double));
    p->vol[e] = m3_det(m) / 6.0;
    double lumped = 0.25 * p->vol[e] * density;
    for (int j = 0; j < 4; j++) masses[ti[j]] += lumped;
  }
  p->inv_mass = (double*)malloc(sizeof(double) * n_nodes);
  for (int i = 0; i < n_nodes; i++) {
    p->inv_mass[i] = (i < p->n_bcs) ? 0.0 : 1.0;
    if (p->inv_mass[i] != 0 && masses[i] != 0) p->inv_mass[i] = 1.0 / masses[i];
  }
  free(masses);
  free(is_fixed);
  memcpy(p->xstart, p->pos, sizeof(double) * 3 * n_nodes);
  return p;
}

void orc_destroy(void* h) {
  orc_problem* p = (orc_problem*)h;
  free(p->tris);
  free(p->map); free(p->tets); free(p->X); free(p->vol); free(p->escale);
  free(p->pos); free(p->pos0); free(p->inv_mass); free(p->fext); free(p->vel); free(p->xstart); free(p);
}

int orc_num_bcs(void* h) { return ((orc_problem*)h)->n_bcs; }
int orc_num_free(void* h) { orc_problem* p = (orc_problem*)h; return p->n_nodes - p->n_bcs; }
void orc_reshuffle_map(void* h, int* out) { orc_problem* p = (orc_problem*)h; memcpy(out, p->map, sizeof(int) * p->n_nodes); }
void orc_tets(void* h, int* out) { orc_problem* p = (orc_problem*)h; memcpy(out, p->tets, sizeof(int) * 4 * (size_t)p->n_tets); }
void orc_set_force_fraction(void* h, double f) { ((orc_problem*)h)->force_fraction = f; }
/* dynamics: mTimeStep, node velocities and step-start positions (reshuffled order) */
void orc_set_time_step(void* h, double dt) { ((orc_problem*)h)->time_step = dt; }
void orc_set_velocities_shuffled(void* h, const double* v) { orc_problem* p = (orc_problem*)h; memcpy(p->vel, v, sizeof(double) * 3 * p->n_nodes); }
void orc_get_velocities_shuffled(void* h, double* v) { orc_problem* p = (orc_problem*)h; memcpy(v, p->vel, sizeof(double) * 3 * p->n_nodes); }
void orc_set_start_shuffled(void* h, const double* x) { orc_problem* p = (orc_problem*)h; memcpy(p->xstart, x, sizeof(double) * 3 * p->n_nodes); }
/* 0: the reference's force differential; 1: exact derivative of the force (differs for corotational). */
void orc_set_tangent(void* h, int mode) { ((orc_problem*)h)->tangent = mode; }
void orc_set_lame(void* h, double mu, double lambda) { orc_problem* p = (orc_problem*)h; p->mu = mu; p->lambda = lambda; }

/* Extension: per-element stiffness scale s_e = E_e / E (mu_e = s_e mu, lambda_e = s_e lambda). */
void orc_set_element_scale(void* h, const double* s) {
  orc_problem* p = (orc_problem*)h;
  if (!s) { free(p->escale); p->escale = NULL; return; }
  if (!p->escale) p->escale = (double*)malloc(sizeof(double) * p->n_tets);
  memcpy(p->escale, s, sizeof(double) * p->n_tets);
}
/* Extension: dead loads per ORIGINAL node (only free nodes matter). */
void orc_set_nodal_loads(void* h, const double* f_orig) {
  orc_problem* p = (orc_problem*)h;
  for (int i = 0; i < p->n_nodes; i++)
    for (int c = 0; c < 3; c++) p->fext[3 * (size_t)p->map[i] + c] = f_orig[3 * (size_t)i + c];
}
void orc_set_positions_shuffled(void* h, const double* x) { orc_problem* p = (orc_problem*)h; memcpy(p->pos, x, sizeof(double) * 3 * p->n_nodes); }
void orc_get_positions_shuffled(void* h, double* x) { orc_problem* p = (orc_problem*)h; memcpy(x, p->pos, sizeof(double) * 3 * p->n_nodes); }
void orc_get_positions(void* h, double* x) {
  orc_problem* p = (orc_problem*)h;
  for (int i = 0; i < p->n_nodes; i++) for (int c = 0; c < 3; c++) x[3 * (size_t)i + c] = p->pos[3 * (size_t)p->map[i] + c];
}
/* free-node block of positions (reshuffled order), 3 N_f */
void orc_set_free_positions(void* h, const double* x) { orc_problem* p = (orc_problem*)h; memcpy(p->pos + 3 * (size_t)p->n_bcs, x, sizeof(double) * 3 * (p->n_nodes - p->n_bcs)); }
void orc_get_free_positions(void* h, double* x) { orc_problem* p = (orc_problem*)h; memcpy(x, p->pos + 3 * (size_t)p->n_bcs, sizeof(double) * 3 * (p->n_nodes - p->n_bcs)); }

/* FemPhysicsMatrixFree::ComputeDeformationGradient, Source/FemPhysicsMatrixFree.cpp:354-368 */
static M3 def_grad(const orc_problem* p, int e) {
  const int* t = p->tets + 4 * (size_t)e;
  V3 x0 = node_v(p->pos, t[0]);
  M3 Ds = m3_cols(v3_sub(node_v(p->pos, t[1]), x0), v3_sub(node_v(p->pos, t[2]), x0), v3_sub(node_v(p->pos, t[3]), x0));
  return m3_mul(Ds, load_X(p, e));
}

static void elem_lame(const orc_problem* p, int e, double* mu, double* lambda) {
  double s = p->escale ? p->escale[e] : 1.0;
  *mu = p->escale ? s * p->mu : p->mu;
  *lambda = p->escale ? s * p->lambda : p->lambda;
}

/* ElasticEnergy::ComputeElementStress, Source/ElasticEnergy.cpp:114-257 (4 materials).
 * Pmu / Plambda are the mu- and lambda-parts for neo-Hookean (zero otherwise). */
/* the float literals of the reference's formulas as they convert to its real type */
#define C23 ((double)(2.0f / 3.0f))
#define C13 ((double)(1.0f / 3.0f))

/* E_e for the NH2 variant (the reference uses GetYoungsModulus(); per-element scales apply) */
static double elem_young(const orc_problem* p, int e) { return p->escale ? p->young * p->escale[e] : p->young; }

static M3 elem_stress(const orc_problem* p, int e, M3 F, M3* Pmu, M3* Plambda) {
  double mu, lambda;
  elem_lame(p, e, &mu, &lambda);
  M3 id = m3_ident(), zero = m3_scale(0.0, id);
  *Pmu = zero; *Plambda = zero;
  M3 R, U;
  if (p->material == MMT_COROTATIONAL) { polar_qr(F, &R, &U); F = U; }
  M3 strain;
  if (p->material == MMT_LINEAR || p->material == MMT_COROTATIONAL || p->material == MMT_DISTORTIONAL_LINEAR)
    strain = m3_sub(m3_scale(0.5, m3_add(F, m3_tr(F))), id);
  else
    strain = m3_scale(0.5, m3_sub(m3_mul(m3_tr(F), F), id));
  switch (p->material) {
    case MMT_STVK:
      return m3_mul(F, m3_add(m3_scale(2 * mu, strain), m3_scale(lambda * m3_trace(strain), id)));
    case MMT_LINEAR:
      return m3_add(m3_scale(2 * mu, strain), m3_scale(lambda * m3_trace(strain), id));
    case MMT_COROTATIONAL:
      return m3_mul(R, m3_add(m3_scale(2 * mu, strain), m3_scale(lambda * m3_trace(strain), id)));
    case MMT_NEO_HOOKEAN: {
      M3 Finv = m3_inv(F);
      double J = m3_det(F);
      M3 Finvtr = m3_tr(Finv);
      *Pmu = m3_sub(F, Finvtr);
      *Plambda = m3_scale(log(J), Finvtr);
      return m3_add(m3_scale(mu, *Pmu), m3_scale(lambda, *Plambda));
    }
    /* the other materials, ElasticEnergy.cpp:188-254 */
    case MMT_DISTORTIONAL_LINEAR:
      return m3_sub(m3_scale(2 * mu, strain), m3_scale((2 * mu / 3) * m3_trace(strain), id));
    case MMT_DISTORTIONAL_MOONEY:
      return m3_scale(mu, F);
    case MMT_DISTORTIONAL_NH2:
      return m3_scale(0.5 * elem_young(p, e), F);
    case MMT_DISTORTIONAL_NH3:
      return m3_scale(mu * pow(m3_det(F), -C23), F);
    default: break;
  }
  M3 Finvtr = m3_tr(m3_inv(F));
  double J = m3_det(F);
  switch (p->material) {
    case MMT_NEO_HOOKEAN_OGDEN:
      return m3_add(m3_scale(mu, m3_sub(F, Finvtr)), m3_scale(lambda * (J - 1) * J, Finvtr));
    case MMT_DISTORTIONAL_BW: {
      double I1 = m3_trace(m3_mul(m3_tr(F), F));
      return m3_scale(mu * pow(J, -C23), m3_sub(F, m3_scale(I1 / 3, Finvtr)));
    }
    case MMT_DISTORTIONAL_OGDEN:
      *Pmu = m3_sub(F, Finvtr);
      return m3_scale(mu, *Pmu);
    case MMT_DISTORTIONAL_NH6:
      return m3_scale(mu, m3_sub(F, m3_scale(J, Finvtr)));
    default: { /* MMT_DISTORTIONAL_NH7 */
      double lambda1 = -C23 * mu;
      return m3_add(m3_scale(mu, m3_sub(F, Finvtr)), m3_scale(lambda1 * log(J), Finvtr));
    }
  }
}

/* FemPhysicsMatrixFree::SetBoundaryConditionsSurface (Source/FemPhysicsMatrixFree.cpp:1051-1060):
 * triangles of original node indices and the applied (follower) pressure. */
void orc_set_pressure_surface(void* h, const int* tris, int n_tris, double pressure) {
  orc_problem* p = (orc_problem*)h;
  free(p->tris);
  p->tris = NULL;
  p->n_tris = n_tris;
  p->pressure = pressure;
  if (n_tris > 0) {
    p->tris = (int*)malloc(sizeof(int) * 3 * (size_t)n_tris);
    memcpy(p->tris, tris, sizeof(int) * 3 * (size_t)n_tris);
  }
}

/* FemPhysicsMatrixFree::ComputePressureForces (Source/FemPhysicsMatrixFree.cpp:967-1049), explicit
 * part: per triangle ff * (area/3) * pressure * unit normal of (p2-p1) x (p3-p1), added to its nodes. */
static void pressure_forces(const orc_problem* p, double* f) {
  for (int t = 0; t < p->n_tris; t++) {
    int i1 = p->map[p->tris[3 * t]], i2 = p->map[p->tris[3 * t + 1]], i3 = p->map[p->tris[3 * t + 2]];
    V3 p1 = node_v(p->pos, i1), p2 = node_v(p->pos, i2), p3 = node_v(p->pos, i3);
    V3 a = v3_sub(p2, p1), b = v3_sub(p3, p1);
    V3 nrm = v3_cross(a, b);
    double area = 0.5 * sqrt(v3_dot(nrm, nrm));
    nrm = v3_normalized(nrm);
    V3 traction = v3_scale(p->pressure, nrm);
    V3 force = v3_scale(p->force_fraction, v3_scale(area / 3.0, traction));
    int idx[3] = {i1, i2, i3};
    for (int k = 0; k < 3; k++)
      for (int c = 0; c < 3; c++) f[3 * (size_t)idx[k] + c] += force.v[c];
  }
}

/* ElasticEnergy::ComputeForces (Source/ElasticEnergy.cpp:259-282) into a full
 * reshuffled node array, serial element-order scatter, after the pressure forces
 * (the order of FemPhysicsMatrixFree::ComputeGradients, Source/FemPhysicsMatrixFree.cpp:540-543). */
static void internal_forces(const orc_problem* p, double* f) {
  memset(f, 0, sizeof(double) * 3 * p->n_nodes);
  pressure_forces(p, f);
  for (int e = 0; e < p->n_tets; e++) {
    M3 Pmu, Pl;
    M3 F = def_grad(p, e);
    M3 P = elem_stress(p, e, F, &Pmu, &Pl);
    M3 H = m3_mul(m3_scale(-p->vol[e], P), m3_tr(load_X(p, e)));
    const int* t = p->tets + 4 * (size_t)e;
    for (int j = 1; j < 4; j++)
      for (int c = 0; c < 3; c++) {
        f[3 * (size_t)t[j] + c] += H.m[c][j - 1];
        f[3 * (size_t)t[0] + c] -= H.m[c][j - 1];
      }
  }
}

/* FemPhysicsMatrixFree::ComputeGradients (Source/FemPhysicsMatrixFree.cpp:536-560),
 * static case, plus the dead-load extension.  r has 3 N_f entries. */
void orc_compute_gradients(void* h, double* r) {
  orc_problem* p = (orc_problem*)h;
  double* f = (double*)malloc(sizeof(double) * 3 * p->n_nodes);
  internal_forces(p, f);
  int nf = p->n_nodes - p->n_bcs;
  for (int i = 0; i < nf; i++) {
    int g = i + p->n_bcs;
    double mass = 1.0 / p->inv_mass[g];
    double s = mass * p->force_fraction;
    /* FemPhysicsMatrixFree.cpp:545-556: invH = 1/h, invHSqr = 1/(h h), both 0 for a static solve */
    double invH = p->time_step == 0 ? 0 : 1.0 / p->time_step;
    double invHSqr = p->time_step == 0 ? 0 : 1.0 / (p->time_step * p->time_step);
    for (int c = 0; c < 3; c++) {
      size_t k = 3 * (size_t)g + c;
      r[3 * (size_t)i + c] = f[k];
      r[3 * (size_t)i + c] += s * p->grav[c];
      if (p->time_step != 0) {
        r[3 * (size_t)i + c] += mass * invH * p->vel[k];
        r[3 * (size_t)i + c] -= mass * invHSqr * (p->pos[k] - p->xstart[k]);
      }
      r[3 * (size_t)i + c] += p->force_fraction * p->fext[k];
    }
  }
  free(f);
}

static V3 v3_add(V3 a, V3 b) { return v3(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }

/* Exact directional derivative of the corotational PK1 stress P = R (2 mu (U - I) + lambda tr(U - I) I)
 * with the Gram-Schmidt R of polar_qr and U = sym(R^T F) (the force of ElasticEnergy.cpp:164-167).
 * Extension: the reference's differential (FemPhysicsMatrixFree.cpp:441-456) assumes a true polar R. */
static M3 corot_exact_diff(double mu, double lambda, M3 F, M3 dF) {
  V3 c0 = m3_col(&F, 0), c1 = m3_col(&F, 1), dc0 = m3_col(&dF, 0), dc1 = m3_col(&dF, 1);
  double n0 = sqrt(v3_dot(c0, c0));
  V3 r0 = v3_scale(1.0 / n0, c0);
  V3 dr0 = v3_scale(1.0 / n0, v3_sub(dc0, v3_scale(v3_dot(r0, dc0), r0)));
  double a = v3_dot(c1, r0);
  V3 v1 = v3_sub(c1, v3_scale(a, r0));
  double n1 = sqrt(v3_dot(v1, v1));
  V3 r1 = v3_scale(1.0 / n1, v1);
  double da = v3_dot(dc1, r0) + v3_dot(c1, dr0);
  V3 dv1 = v3_sub(v3_sub(dc1, v3_scale(da, r0)), v3_scale(a, dr0));
  V3 dr1 = v3_scale(1.0 / n1, v3_sub(dv1, v3_scale(v3_dot(r1, dv1), r1)));
  V3 v2 = v3_cross(r0, r1);
  double n2 = sqrt(v3_dot(v2, v2));
  V3 r2 = v3_scale(1.0 / n2, v2);
  V3 dv2 = v3_add(v3_cross(dr0, r1), v3_cross(r0, dr1));
  V3 dr2 = v3_scale(1.0 / n2, v3_sub(dv2, v3_scale(v3_dot(r2, dv2), r2)));
  M3 R = m3_cols(r0, r1, r2), dR = m3_cols(dr0, dr1, dr2), id = m3_ident();
  M3 V = m3_mul(m3_tr(R), F);
  M3 U = m3_scale(0.5, m3_add(V, m3_tr(V)));
  M3 dV = m3_add(m3_mul(m3_tr(dR), F), m3_mul(m3_tr(R), dF));
  M3 dU = m3_scale(0.5, m3_add(dV, m3_tr(dV)));
  M3 strain = m3_sub(U, id);
  M3 S = m3_add(m3_scale(2 * mu, strain), m3_scale(lambda * m3_trace(strain), id));
  M3 dS = m3_add(m3_scale(2 * mu, dU), m3_scale(lambda * m3_trace(dU), id));
  return m3_add(m3_mul(dR, S), m3_mul(R, dS));
}

/* Force differential dP for each material, Source/FemPhysicsMatrixFree.cpp:436-470
 * (identical to ElasticEnergy::ComputeLocalForceDifferential, ElasticEnergy.cpp:367-411). */
static M3 stress_diff(const orc_problem* p, int e, M3 F, M3 dF) {
  double mu, lambda;
  elem_lame(p, e, &mu, &lambda);
  M3 id = m3_ident();
  switch (p->material) {
    case MMT_LINEAR:
      return m3_add(m3_scale(mu, m3_add(dF, m3_tr(dF))), m3_scale(lambda * m3_trace(dF), id));
    case MMT_COROTATIONAL: {
      if (p->tangent == 1) return corot_exact_diff(mu, lambda, F, dF);
      M3 R, S;
      polar_qr(F, &R, &S);
      M3 dS = m3_mul(m3_tr(R), dF);
      M3 dP = m3_add(m3_scale(2 * mu, dF), m3_scale(lambda * m3_trace(dS), R));
      double trS = m3_trace(S);
      M3 A = m3_sub(S, m3_scale(trS, id));
      V3 w = v3(dS.m[1][2] - dS.m[2][1], dS.m[0][2] - dS.m[2][0], dS.m[0][1] - dS.m[1][0]);
      V3 r = m3_mulv(m3_inv(A), w);
      M3 dR = m3_mul(R, m3_skew(r));
      return m3_add(dP, m3_scale(lambda * (trS - 3) - 2 * mu, dR));
    }
    case MMT_STVK: {
      M3 E = m3_scale(0.5, m3_sub(m3_mul(m3_tr(F), F), id));
      M3 dE = m3_scale(0.5, m3_add(m3_mul(m3_tr(dF), F), m3_mul(m3_tr(F), dF)));
      return m3_add(m3_mul(dF, m3_add(m3_scale(2 * mu, E), m3_scale(lambda * m3_trace(E), id))),
                    m3_mul(F, m3_add(m3_scale(2 * mu, dE), m3_scale(lambda * m3_trace(dE), id))));
    }
    case MMT_NEO_HOOKEAN: {
      M3 Finv = m3_inv(F);
      M3 Finvtr = m3_tr(Finv);
      double J = m3_det(F);
      M3 a = m3_scale(mu, dF);
      M3 b = m3_mul(m3_mul(m3_scale(mu - lambda * log(J), Finvtr), m3_tr(dF)), Finvtr);
      M3 c = m3_scale(lambda * m3_trace(m3_mul(Finv, dF)), Finvtr);
      return m3_add(m3_add(a, b), c);
    }
    /* the other materials: ElasticEnergy::ComputeLocalForceDifferential (ElasticEnergy.cpp:412-479),
     * the differential of the reference's assembled path (its matrix-free product covers only the
     * four materials above) */
    case MMT_DISTORTIONAL_LINEAR:
      return m3_sub(m3_scale(mu, m3_add(dF, m3_tr(dF))), m3_scale(C23 * mu * m3_trace(dF), id));
    case MMT_DISTORTIONAL_MOONEY:
      return m3_scale(mu, dF);
    case MMT_DISTORTIONAL_NH2:
      return m3_scale(0.5 * elem_young(p, e), dF);
    case MMT_DISTORTIONAL_NH3:
      return m3_scale(mu * pow(m3_det(F), -C23), dF);
    default: break;
  }
  M3 Finv = m3_inv(F);
  M3 Finvtr = m3_tr(Finv);
  double J = m3_det(F);
  double trFd = m3_trace(m3_mul(Finv, dF));
  switch (p->material) {
    case MMT_NEO_HOOKEAN_OGDEN: {
      M3 b = m3_mul(m3_mul(m3_scale(mu - lambda * (J - 1), Finvtr), m3_tr(dF)), Finvtr);
      return m3_add(m3_add(m3_scale(mu, dF), b), m3_scale(lambda * J * trFd, Finvtr));
    }
    case MMT_DISTORTIONAL_BW: {
      M3 C = m3_mul(m3_tr(F), F);
      double I1 = m3_trace(C);
      M3 Q = m3_sub(F, m3_scale(C13 * I1, Finvtr));
      M3 dC = m3_add(m3_mul(m3_tr(dF), F), m3_mul(m3_tr(F), dF));
      M3 inner = m3_sub(m3_scale(m3_trace(dC), Finvtr), m3_mul(m3_mul(m3_scale(I1, Finvtr), m3_tr(dF)), Finvtr));
      M3 dQ = m3_sub(dF, m3_scale(C13, inner));
      return m3_scale(mu * pow(J, -C23), m3_sub(dQ, m3_scale(C23 * trFd, Q)));
    }
    case MMT_DISTORTIONAL_OGDEN:
      return m3_add(m3_scale(mu, dF), m3_mul(m3_mul(m3_scale(mu, Finvtr), m3_tr(dF)), Finvtr));
    case MMT_DISTORTIONAL_NH6: {
      M3 a = m3_add(m3_scale(mu, dF), m3_mul(m3_mul(m3_scale(mu * J, Finvtr), m3_tr(dF)), Finvtr));
      return m3_sub(a, m3_scale(mu * J * trFd, Finvtr));
    }
    default: { /* MMT_DISTORTIONAL_NH7 */
      double lambda1 = -C23 * mu;
      M3 b = m3_mul(m3_mul(m3_scale(mu - lambda1 * log(J), Finvtr), m3_tr(dF)), Finvtr);
      return m3_add(m3_add(m3_scale(mu, dF), b), m3_scale(lambda1 * trFd, Finvtr));
    }
  }
}

/* FemPhysicsMatrixFree::ComputeForceDifferential + MatrixVectorMultiply
 * (Source/FemPhysicsMatrixFree.cpp:406-496, 523-534): out = -df (static).
 * Element loop in parallel (OpenMP, as :417), scatter serial in element order. */
void orc_matvec(void* h, const double* d, double* out) {
  orc_problem* p = (orc_problem*)h;
  int nf = p->n_nodes - p->n_bcs, nbc = p->n_bcs;
  double* dH = (double*)malloc(sizeof(double) * 9 * (size_t)p->n_tets);
  #pragma omp parallel for schedule(static)
  for (int e = 0; e < p->n_tets; e++) {
    const int* t = p->tets + 4 * (size_t)e;
    V3 x[4];
    for (int j = 0; j < 4; j++) x[j] = t[j] < nbc ? v3(0, 0, 0) : node_v(d, t[j] - nbc);
    M3 mat = m3_cols(v3_sub(x[1], x[0]), v3_sub(x[2], x[0]), v3_sub(x[3], x[0]));
    M3 X = load_X(p, e);
    M3 dF = m3_mul(mat, X);
    M3 F = def_grad(p, e);
    M3 dP = stress_diff(p, e, F, dF);
    M3 H = m3_mul(m3_scale(-p->vol[e], dP), m3_tr(X));
    memcpy(dH + 9 * (size_t)e, H.m, 9 * sizeof(double));
  }
  double* df = (double*)calloc(3 * (size_t)nf, sizeof(double));
  for (int e = 0; e < p->n_tets; e++) {
    const int* t = p->tets + 4 * (size_t)e;
    const double* H = dH + 9 * (size_t)e;
    double f3[3] = {0, 0, 0};
    for (int j = 1; j < 4; j++) {
      for (int c = 0; c < 3; c++) {
        double f = H[3 * c + (j - 1)];
        if (t[j] >= nbc) df[3 * (size_t)(t[j] - nbc) + c] += f;
        f3[c] -= f;
      }
    }
    if (t[0] >= nbc) for (int c = 0; c < 3; c++) df[3 * (size_t)(t[0] - nbc) + c] += f3[c];
  }
  /* MatrixVectorMultiply (FemPhysicsMatrixFree.cpp:523-534): M d / h^2 - df */
  double invHSqr = p->time_step == 0 ? 0 : 1.0 / (p->time_step * p->time_step);
  for (size_t i = 0; i < 3 * (size_t)nf; i++) {
    double mass = 1.0 / p->inv_mass[nbc + i / 3];
    out[i] = invHSqr * mass * d[i] - df[i];
  }
  free(df);
  free(dH);
}

/* FemPhysicsMatrixFree::SubStep (Source/FemPhysicsMatrixFree.cpp:371-387): elastic forces only,
 * then for every node with invMass != 0: vel += (h invMass) f + h g, pos += h vel. */
void orc_explicit_substep(void* h, double hs) {
  orc_problem* p = (orc_problem*)h;
  double* f = (double*)malloc(sizeof(double) * 3 * p->n_nodes);
  internal_forces(p, f);
  for (int i = 0; i < p->n_nodes; i++) {
    if (p->inv_mass[i] == 0) continue;
    for (int c = 0; c < 3; c++) {
      size_t k = 3 * (size_t)i + c;
      p->vel[k] += (hs * p->inv_mass[i]) * f[k] + hs * p->grav[c];
      p->pos[k] += hs * p->vel[k];
    }
  }
  free(f);
}

/* Per-DOF diagonal of the tangent over free DOFs: the diagonal entries of the
 * local stiffness of ElasticEnergy::ComputeLocalStiffnessMatrixFromDifferential
 * (Source/ElasticEnergy.cpp:493-517), K_local(i,i) = -df_i(e_i), summed per node
 * in element order. */
void orc_jacobi_diagonal(void* h, double* diag) {
  orc_problem* p = (orc_problem*)h;
  int nbc = p->n_bcs, nf = p->n_nodes - nbc;
  memset(diag, 0, sizeof(double) * 3 * (size_t)nf);
  double* kdall = (double*)malloc(sizeof(double) * 12 * (size_t)p->n_tets);
  /* element loop in parallel (as the reference's assembly loop, ElasticEnergy.cpp:589), scatter serial */
  #pragma omp parallel for schedule(static)
  for (int e = 0; e < p->n_tets; e++) {
    M3 F = def_grad(p, e);
    M3 X = load_X(p, e);
    double kd[12];
    for (int j = 0; j < 12; j++) {
      double b[12] = {0};
      b[j] = 1;
      V3 x0 = v3(b[0], b[1], b[2]);
      M3 mat = m3_cols(v3_sub(v3(b[3], b[4], b[5]), x0), v3_sub(v3(b[6], b[7], b[8]), x0), v3_sub(v3(b[9], b[10], b[11]), x0));
      M3 dF = m3_mul(mat, X);
      M3 dP = stress_diff(p, e, F, dF);
      M3 H = m3_mul(m3_scale(-p->vol[e], dP), m3_tr(X));
      int a = j / 3, c = j % 3;
      double dfv;
      if (a > 0) dfv = H.m[c][a - 1];
      else { double s = 0; for (int k = 0; k < 3; k++) s -= H.m[c][k]; dfv = s; }
      kd[j] = -dfv;
    }
    memcpy(kdall + 12 * (size_t)e, kd, sizeof(kd));
  }
  for (int e = 0; e < p->n_tets; e++) {
    const int* t = p->tets + 4 * (size_t)e;
    const double* kd = kdall + 12 * (size_t)e;
    for (int a = 0; a < 4; a++) {
      if (t[a] < nbc) continue;
      for (int c = 0; c < 3; c++) diag[3 * (size_t)(t[a] - nbc) + c] += kd[3 * a + c];
    }
  }
  free(kdall);
  if (p->time_step != 0) {  /* the M / h^2 term of the dynamic tangent */
    double invHSqr = 1.0 / (p->time_step * p->time_step);
    for (int i = 0; i < nf; i++)
      for (int c = 0; c < 3; c++) diag[3 * (size_t)i + c] += invHSqr * (1.0 / p->inv_mass[nbc + i]);
  }
}

/* PK1 stress of all elements at the current positions (E x 9). */
void orc_element_stress(void* h, double* P) {
  orc_problem* p = (orc_problem*)h;
  for (int e = 0; e < p->n_tets; e++) {
    M3 a, b;
    M3 S = elem_stress(p, e, def_grad(p, e), &a, &b);
    memcpy(P + 9 * (size_t)e, S.m, 9 * sizeof(double));
  }
}

/* ElasticEnergy::ComputeElementEnergy (Source/ElasticEnergy.cpp:40-112), summed
 * serially as FemPhysicsBase::ComputeElasticEnergy (Source/FemPhysicsBase.cpp:203-212). */
static double elem_energy(const orc_problem* p, int e) {
  double mu, lambda;
  elem_lame(p, e, &mu, &lambda);
  M3 id = m3_ident();
  M3 F = def_grad(p, e), R, U;
  if (p->material == MMT_COROTATIONAL) { polar_qr(F, &R, &U); F = U; }
  M3 strain;
  if (p->material == MMT_LINEAR || p->material == MMT_COROTATIONAL || p->material == MMT_DISTORTIONAL_LINEAR)
    strain = m3_sub(m3_scale(0.5, m3_add(F, m3_tr(F))), id);
  else
    strain = m3_scale(0.5, m3_sub(m3_mul(m3_tr(F), F), id));
  double en = 0;  /* ElasticEnergy.cpp:69-108: the materials without an energy there report 0 */
  if (p->material == MMT_LINEAR || p->material == MMT_COROTATIONAL || p->material == MMT_STVK) {
    double tr = m3_trace(strain);
    en = mu * m3_ddot(strain, strain) + 0.5 * lambda * tr * tr;
  } else if (p->material == MMT_NEO_HOOKEAN || p->material == MMT_NEO_HOOKEAN_OGDEN ||
             p->material == MMT_DISTORTIONAL_MOONEY || p->material == MMT_DISTORTIONAL_OGDEN) {
    double J = m3_det(F);
    double I1 = m3_trace(m3_mul(m3_tr(F), F));
    double lj = log(J);
    if (p->material == MMT_NEO_HOOKEAN) en = 0.5 * mu * (I1 - 3) - mu * lj + 0.5 * lambda * lj * lj;
    else if (p->material == MMT_NEO_HOOKEAN_OGDEN) en = 0.5 * mu * (I1 - 3) - mu * lj + 0.5 * lambda * (J - 1) * (J - 1);
    else if (p->material == MMT_DISTORTIONAL_MOONEY) en = 0.5 * mu * (I1 - 3);
    else en = 0.5 * mu * (I1 - 3) - mu * lj;
  }
  return p->vol[e] * en;
}
double orc_elastic_energy(void* h) {
  orc_problem* p = (orc_problem*)h;
  double s = 0;
  for (int e = 0; e < p->n_tets; e++) s += elem_energy(p, e);
  return s;
}
/* Total potential energy: elastic - sum_i (m_i g + f_ext,i) . x_i over free nodes
 * (the full gravity vector; the reference's ComputeEnergy uses g.y only,
 * Source/FemPhysicsMatrixFree.cpp:890). */
double orc_total_energy(void* h) {
  orc_problem* p = (orc_problem*)h;
  double s = orc_elastic_energy(h);
  for (int g = p->n_bcs; g < p->n_nodes; g++) {
    double mass = 1.0 / p->inv_mass[g];
    for (int c = 0; c < 3; c++)
      s -= p->force_fraction * (mass * p->grav[c] + p->fext[3 * (size_t)g + c]) * p->pos[3 * (size_t)g + c];
  }
  return s;
}

/* Number of elements with det F <= 0, FemPhysicsBase::CheckForInversion (Source/FemPhysicsBase.cpp:93-117). */
int orc_count_inverted(void* h) {
  orc_problem* p = (orc_problem*)h;
  int n = 0;
  for (int e = 0; e < p->n_tets; e++) if (m3_det(def_grad(p, e)) <= 0.0) n++;
  return n;
}

/* FemPhysicsBase::GetForceParamGrads (Source/FemPhysicsBase.cpp:162-187) with
 * ElasticEnergy::ComputeForceParamGrads (Source/ElasticEnergy.cpp:284-315). */
void orc_force_param_grads(void* h, double* gmu, double* glambda, double* grho) {
  orc_problem* p = (orc_problem*)h;
  size_t n3 = 3 * (size_t)p->n_nodes;
  double* fmu = (double*)calloc(n3, sizeof(double));
  double* fl = (double*)calloc(n3, sizeof(double));
  double* nv = (double*)calloc(p->n_nodes, sizeof(double));
  for (int e = 0; e < p->n_tets; e++) {
    M3 Pmu, Pl;
    elem_stress(p, e, def_grad(p, e), &Pmu, &Pl);
    const int* t = p->tets + 4 * (size_t)e;
    M3 Xt = m3_tr(load_X(p, e));
    M3 Hm = m3_mul(m3_scale(-p->vol[e], Pmu), Xt);
    M3 Hl = m3_mul(m3_scale(-p->vol[e], Pl), Xt);
    for (int j = 1; j < 4; j++)
      for (int c = 0; c < 3; c++) {
        fmu[3 * (size_t)t[j] + c] += Hm.m[c][j - 1];
        fmu[3 * (size_t)t[0] + c] -= Hm.m[c][j - 1];
      }
    for (int j = 1; j < 4; j++)
      for (int c = 0; c < 3; c++) {
        fl[3 * (size_t)t[j] + c] += Hl.m[c][j - 1];
        fl[3 * (size_t)t[0] + c] -= Hl.m[c][j - 1];
      }
    for (int l = 0; l < 4; l++) nv[t[l]] += 0.25 * p->vol[e];
  }
  int nbc = p->n_bcs, nf = p->n_nodes - nbc;
  for (int i = 0; i < nf; i++)
    for (int c = 0; c < 3; c++) {
      gmu[3 * (size_t)i + c] = fmu[3 * (size_t)(i + nbc) + c];
      glambda[3 * (size_t)i + c] = fl[3 * (size_t)(i + nbc) + c];
      grho[3 * (size_t)i + c] = nv[i + nbc] * p->grav[c];
    }
  free(fmu); free(fl); free(nv);
}

/* Per-element force vectors f_e (12 per element, local node order) of the internal
 * force at the current positions: used by the per-element adjoint gradient. */
void orc_element_forces(void* h, double* fe) {
  orc_problem* p = (orc_problem*)h;
  for (int e = 0; e < p->n_tets; e++) {
    M3 a, b;
    M3 P = elem_stress(p, e, def_grad(p, e), &a, &b);
    M3 H = m3_mul(m3_scale(-p->vol[e], P), m3_tr(load_X(p, e)));
    double* o = fe + 12 * (size_t)e;
    for (int c = 0; c < 3; c++) {
      o[c] = 0;
      for (int j = 1; j < 4; j++) { o[3 * j + c] = H.m[c][j - 1]; o[c] -= H.m[c][j - 1]; }
    }
  }
}

/* ---------------------------------------------------------------------- */
/* Solvers over the physics above                                          */
/* ---------------------------------------------------------------------- */
static double dotn(const double* a, const double* b, size_t n) { double s = 0; for (size_t i = 0; i < n; i++) s += a[i] * b[i]; return s; }

/* Jacobi-preconditioned CG on K x = b (zero initial guess), stopping when
 * |r| <= tol |b|.  The matrix-free CG of Math/IterativeSolvers.h:115-195
 * (Shewchuk's algorithm) with a per-DOF diagonal preconditioner.  Returns
 * iterations; *relres = final |r|/|b|. */
int orc_pcg(void* h, const double* b, double* x, const double* diag, double tol, int max_iters, double* relres) {
  orc_problem* p = (orc_problem*)h;
  size_t n = 3 * (size_t)(p->n_nodes - p->n_bcs);
  double* r = (double*)malloc(n * sizeof(double));
  double* z = (double*)malloc(n * sizeof(double));
  double* d = (double*)malloc(n * sizeof(double));
  double* q = (double*)malloc(n * sizeof(double));
  memset(x, 0, n * sizeof(double));
  memcpy(r, b, n * sizeof(double));
  double bn = sqrt(dotn(b, b, n));
  for (size_t i = 0; i < n; i++) { z[i] = diag ? r[i] / diag[i] : r[i]; d[i] = z[i]; }
  double delta = dotn(r, z, n), rn = bn;
  int it = 0;
  if (bn == 0) { *relres = 0; goto done; }
  for (; it < max_iters; it++) {
    orc_matvec(h, d, q);
    double alpha = delta / dotn(d, q, n);
    for (size_t i = 0; i < n; i++) { x[i] += alpha * d[i]; r[i] -= alpha * q[i]; }
    rn = sqrt(dotn(r, r, n));
    if (rn <= tol * bn) { it++; break; }
    for (size_t i = 0; i < n; i++) z[i] = diag ? r[i] / diag[i] : r[i];
    double delta1 = dotn(r, z, n);
    double beta = delta1 / delta;
    delta = delta1;
    for (size_t i = 0; i < n; i++) d[i] = z[i] + beta * d[i];
  }
  *relres = rn / bn;
done:
  free(r); free(z); free(d); free(q);
  return it;
}

/*
 * Inexact Newton with Jacobi-PCG inner solves (the same algorithm as the GPU
 * host driver's default): forcing term eta_k (Eisenstat-Walker choice 2,
 * gamma=0.9, exponent 2, eta_max, floored by eta_min and by the final target),
 * backtracking (halve up to 30 times, no inverted elements) on the total energy
 * (Armijo, 1e-4) for hyperelastic materials -- with the residual norm deciding
 * once the energy change is below FP64 resolution -- and on the residual norm
 * (|r(x+a d)| <= (1 - 1e-4 a) |r(x)|) for corotational.  Converges when |r| <= rtol |r0|.
 * stats[0]=newton its, [1]=total cg its, [2]=final |r|/|r0|, [3]=|r0|.
 */
int orc_newton_pcg(void* h, double rtol, int max_newton, int max_cg, double eta_max, double eta_min, double* stats) {
  orc_problem* p = (orc_problem*)h;
  size_t n = 3 * (size_t)(p->n_nodes - p->n_bcs);
  double* r = (double*)malloc(n * sizeof(double));
  double* dx = (double*)malloc(n * sizeof(double));
  double* diag = (double*)malloc(n * sizeof(double));
  double* x0 = (double*)malloc(n * sizeof(double));
  orc_compute_gradients(h, r);
  double r0 = sqrt(dotn(r, r, n)), rn = r0, rprev = r0, eta = eta_max;
  int k = 0, cg_total = 0, status = 1;
  if (r0 == 0) { status = 0; goto done; }
  for (; k < max_newton; k++) {
    if (rn <= rtol * r0) { status = 0; break; }
    if (k > 0) {
      double e2 = 0.9 * (rn / rprev) * (rn / rprev);
      double sg = 0.9 * eta * eta;
      if (sg > 0.1 && sg > e2) e2 = sg;
      eta = e2 < eta_max ? e2 : eta_max;
    }
    double floor_t = 0.5 * rtol * r0 / rn;
    if (eta < floor_t) eta = floor_t;
    if (eta < eta_min) eta = eta_min;
    if (eta > eta_max) eta = eta_max;
    orc_jacobi_diagonal(h, diag);
    double rr;
    cg_total += orc_pcg(h, r, dx, diag, eta, max_cg, &rr);
    orc_get_free_positions(h, x0);
    /* energy Armijo (hyperelastic) with the residual norm deciding once the energy change is
     * below FP64 resolution; residual-norm backtracking for corotational */
    const int armijo = p->material != MMT_COROTATIONAL;
    const double e_old = armijo ? orc_total_energy(h) : 0.0;
    const double slope = -dotn(r, dx, n);
    double a = 1.0;
    int ok = 0;
    for (int ls = 0; ls < 30; ls++) {
      for (size_t i = 0; i < n; i++) p->pos[3 * (size_t)p->n_bcs + i] = x0[i] + a * dx[i];
      if (orc_count_inverted(h) == 0) {
        orc_compute_gradients(h, r);
        double n2 = sqrt(dotn(r, r, n));
        int cond = 0;
        if (isfinite(n2)) {
          if (armijo) {
            const double e_el = orc_elastic_energy(h), e_new = orc_total_energy(h);
            cond = e_new < e_old + 1e-4 * a * slope;
            const double res = 1e-12 * (fabs(e_old) + fabs(e_el));
            if (!cond && fabs(e_new - e_old) <= res && fabs(a * slope) <= res) cond = n2 < rn;
          } else {
            cond = n2 <= (1 - 1e-4 * a) * rn;
          }
        }
        if (cond) { rprev = rn; rn = n2; ok = 1; break; }
      }
      a *= 0.5;
    }
    if (!ok) { orc_set_free_positions(h, x0); orc_compute_gradients(h, r); status = 2; k++; break; }
  }
  if (status == 1 && rn <= rtol * r0) status = 0;
done:
  stats[0] = k; stats[1] = cg_total; stats[2] = r0 > 0 ? rn / r0 : 0; stats[3] = r0;
  free(r); free(dx); free(diag); free(x0);
  return status;
}

/*
 * Adjoint gradient of L(u) at equilibrium with respect to per-element Young's
 * modulus E_e and dead loads.  With r(u; E, f) = f_int(u; E) + m g + f = 0 and
 * K = -dr/du symmetric, lambda solves K lambda = dL/du and
 *   dL/dE_e = lambda_e . f_int,e / E_e   (f_int,e is linear in E_e),
 *   dL/df   = lambda.
 * dLdu and dLdf are over free DOFs (reshuffled order); young_e gives E_e.
 */
int orc_adjoint(void* h, const double* dLdu, const double* young_e, double tol, int max_cg, double* dLdE, double* dLdf) {
  orc_problem* p = (orc_problem*)h;
  size_t n = 3 * (size_t)(p->n_nodes - p->n_bcs);
  int nbc = p->n_bcs;
  double* diag = (double*)malloc(n * sizeof(double));
  orc_jacobi_diagonal(h, diag);
  double rr;
  int its = orc_pcg(h, dLdu, dLdf, diag, tol, max_cg, &rr);
  double* fe = (double*)malloc(12 * sizeof(double) * (size_t)p->n_tets);
  orc_element_forces(h, fe);
  for (int e = 0; e < p->n_tets; e++) {
    const int* t = p->tets + 4 * (size_t)e;
    double s = 0;
    for (int a = 0; a < 4; a++) {
      if (t[a] < nbc) continue;
      for (int c = 0; c < 3; c++) s += dLdf[3 * (size_t)(t[a] - nbc) + c] * fe[12 * (size_t)e + 3 * a + c];
    }
    dLdE[e] = s / young_e[e];
  }
  free(fe); free(diag);
  return its;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
