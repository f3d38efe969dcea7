/*
 * fem-g GB300: C ABI of the host-side mirror of the reference's
 * Formulation/Field/Term interface (problem set-up and pre-processing).
 *
 * A problem here is what a GmshFEM user program builds: a mesh, a Field with
 * its function space and constraints, terms added with Formulation::integral
 * (src/problem/Formulation.cpp:219-746), then Formulation::pre()
 * (src/problem/Formulation.cpp:897-1039). The builder runs that pre() on the
 * host (DOF dictionary, Hilbert numbering, CSR pattern, element DOF map) and
 * exposes the descriptors fg_plan_create takes, so tests and benchmarks drive
 * the same C ABI a GmshFEM GpuFormulation would.
 */
#ifndef FEM_G_GB300_HOST_H
#define FEM_G_GB300_HOST_H

#include "fem_g_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  FG_PROBLEM_HELMHOLTZ = 0, /* -div grad u - k^2 c u = f, scalar */
  FG_PROBLEM_NAVIER = 1,    /* time-harmonic elastodynamics, 3-component field */
  FG_PROBLEM_MAXWELL = 2,   /* curl curl E - k^2 c E, hierarchical HCurl field of order `order` */
  FG_PROBLEM_COUPLED = 3    /* two scalar fields u, v (orders order, order2) coupled both ways:
                               grad u.grad tu - k^2 u tu + grad v.grad tv + 2 v tv
                               + (0.5 + x) u tv + (b . grad u) tv + 0.3 grad v.grad tu,
                               b = (1, -0.5 + 0.2i, 0.25); source: -f tu + (1 + x y) tv;
                               dirichlet: u fixed on the boundary curves (2D) */
};
enum { FG_SPACE_LAGRANGE = 0, FG_SPACE_HIERARCHICAL_H1 = 1, FG_SPACE_HCURL = 2 /* hierarchical HCurl; order 0: edge functions */ };
enum {
  FG_COEF_MODE_CONSTANT = 0,   /* mass coefficient -k^2 */
  FG_COEF_MODE_PER_ELEMENT = 1 /* mass coefficient -k^2 (1 + 0.3 xi_e), xi_e ~ N(0,1) per element */
};

typedef struct {
  int32_t kind;      /* FG_PROBLEM_* */
  int32_t dim;       /* 2: unit square of triangles, 3: unit cube of Kuhn tetrahedra */
  int32_t m;         /* cells per side */
  int32_t mesh_order;/* geometric order of the mesh: 1 or 2 */
  int32_t space;     /* FG_SPACE_* */
  int32_t order;     /* hierarchical order (ignored for Lagrange: mesh order) */
  int32_t gauss;     /* integration type "Gauss<gauss>" */
  double jitter;     /* interior node jitter, fraction of h */
  uint64_t seed;
  double k;          /* wavenumber (Helmholtz) */
  int32_t coef_mode; /* FG_COEF_MODE_* */
  int32_t dirichlet; /* 1: u = dirichlet_value on the boundary curves (2D) */
  double dirichlet_value;
  int32_t source;    /* 1: f = heaviside(0.01 - (x-.5)^2 - (y-.5)^2) as integral(-f, tf(u)) */
  double omega;      /* Navier: frequency of the mass term -omega^2 rho dof(u); <= 0: the mass
                        term is integral(dt2_dof(u), tf(u)) and the frequency is the assemble call's */
  double lame_sigma; /* Navier: lambda, mu lognormal(median 1, sigma) per element */
  int32_t upper;     /* 1: symmetric (upper-triangle) storage of the system matrix */
  int32_t order2;    /* FG_PROBLEM_COUPLED: hierarchical order of the field v (0: order) */
} fg_problem_config;

typedef struct fg_problem fg_problem;

int fg_problem_create(const fg_problem_config *cfg, fg_problem **out);
void fg_problem_destroy(fg_problem *p);

/* Descriptors of the (single) assembled element bucket; pointers stay valid
 * until fg_problem_destroy. */
int fg_problem_descs(const fg_problem *p, fg_mesh_desc *mesh, fg_rule_desc *rule, fg_space_desc *space,
                     fg_system_desc *sys, const fg_term_desc **terms, int32_t *n_terms,
                     const double **dirichlet);

/* Multi-field problems (FG_PROBLEM_COUPLED): the unknown fields in the
 * formulation's registration order (Formulation::_addField, the unknown of
 * each bilinear term by first appearance), each field's space on the bucket
 * and element DOF map (fillIndices); the terms by block (test field, unknown
 * field), linear terms in the block (k, k) of their test field k. A block
 * with test != unknown is assembled by a plan of fg_plan_create_coupled.
 * fg_problem_descs describes block 0 (the whole problem with one field). */
int32_t fg_problem_n_fields(const fg_problem *p);
int fg_problem_field(const fg_problem *p, int32_t k, fg_space_desc *space, const uint64_t **elem_dof_idx,
                     const int32_t **elem_dof_type);
int32_t fg_problem_n_blocks(const fg_problem *p);
int fg_problem_block(const fg_problem *p, int32_t b, int32_t *test_field, int32_t *unknown_field,
                     const fg_term_desc **terms, int32_t *n_terms);

/* The fields' DOF dictionaries, field after field, each in its iteration
 * order, as RawDof (src/dofs/Dof.h:44-50): numType, entity, numDof,
 * assembleType, coordinates. */
int64_t fg_problem_n_dofs(const fg_problem *p);
int fg_problem_raw_dofs(const fg_problem *p, uint64_t *num_type, uint64_t *entity, uint64_t *num_dof,
                        int32_t *assemble_type, float *xyz);
/* The DOFs in creation order (before numbering) with their keys and float
 * coordinates: the input of the numbering */
int fg_problem_created_dofs(const fg_problem *p, uint64_t *num_type, uint64_t *entity, int32_t *assemble_type,
                            float *xyz);
/* reserve() calls made on the DOF dictionary while creating DOFs
 * (DofsFactory::_generateFixedDofs / _generateUnknownDofs reserve once per
 * entity and element type): at[k] = DOFs created before call k, arg[k] its
 * argument. Returns the number of calls (fills at most cap entries). */
int64_t fg_problem_reserve_log(const fg_problem *p, uint64_t *at, uint64_t *arg, int64_t cap);
/* model bounding box (xmin, ymin, zmin, xmax, ymax, zmax) */
int fg_problem_bbox(const fg_problem *p, double *bbox);
/* wall seconds of the host pre(): DOFs, numbering, pattern */
double fg_problem_pre_seconds(const fg_problem *p);

/* GpuFormulation::assemble: plan (cached in the problem) + assemble through
 * the C ABI; precision 0 = FP64, 1 = mixed. values [nnz][2], rhs [n_rows][2].
 * Problems of one field (a multi-field problem's blocks go through their own
 * plans: FG_ERR_UNSUPPORTED). */
int fg_problem_assemble(fg_problem *p, int32_t precision, double *csr_values, double *rhs, void *stream);

/* The reference-element basis of the mirror's hierarchical spaces, as gmsh's
 * getBasisFunctions gives it for one orientation (the function spaces'
 * getBasisFunctions, src/field/FunctionSpaceHierarchicalH1.cpp:83-109,
 * FunctionSpaceHierarchicalHCurl.cpp:81-120): space FG_SPACE_HIERARCHICAL_H1
 * or FG_SPACE_HCURL, order, dim 2 (triangle) or 3 (tetrahedron), orientation
 * code from fg_basis_orientation, npts points uvw [npts][3] in reference
 * coordinates. val: [npts][n] (H1) or [npts][n][3] (HCurl); deriv:
 * [npts][n][3], gradients (H1) or curls (HCurl); either may be NULL.
 * Returns n, the functions per element, or -FG_ERR_ARG. */
int fg_basis_eval(int32_t space, int32_t order, int32_t dim, int32_t code, int64_t npts, const double *uvw, double *val,
                  double *deriv);
/* The orientation code of an element with these global vertex tags
 * ([dim + 1]): edge reversal bits, and in 3D the face permutations (not for
 * HCurl order 0), or -FG_ERR_ARG. */
int fg_basis_orientation(int32_t space, int32_t order, int32_t dim, const int64_t *vertex_tags);

#ifdef __cplusplus
}
#endif

#endif /* FEM_G_GB300_HOST_H */
