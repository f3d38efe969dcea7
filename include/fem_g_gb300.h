/*
 * fem-g GB300: C ABI of the GPU assembly path.
 *
 * The drop-in seam in the reference is the virtual
 * gmshfem::problem::Formulation<T>::assemble (src/problem/Formulation.h:196-199,
 * body src/problem/Formulation.cpp:1152-1215). A GPU formulation keeps the
 * reference's own pre() (DOF dictionary, Hilbert numbering, CSR pattern) and
 * replaces assemble() with the calls below:
 *
 *   fg_plan_create    replaces the per-bucket set-up of Formulation::_assembleDim
 *                     (src/problem/Formulation.cpp:1418-1493) and
 *                     Assembler::assemblyInitialization (src/term/Assembler.cpp:69-155):
 *                     geometry, basis tables, element DOF map, element->nonzero map;
 *   fg_assemble_fp64  replaces Assembler::assemble (src/term/Assembler.cpp:157-494):
 *                     BilinearTerm::evaluate (src/term/BilinearTerm.cpp:304-343),
 *                     LinearTerm::evaluate (src/term/LinearTerm.cpp:176-217),
 *                     MatrixFactory::addValues (src/system/MatrixFactory.cpp:233-448),
 *                     VectorFactory::addValues / addValuesDC
 *                     (src/system/VectorFactory.cpp:122-210), in FP64;
 *   fg_assemble_mixed same computation with FP64 geometry and a 3xTF32
 *                     tensor-core element contraction accumulated in FP32;
 *   fg_batch_*        many independent problems assembled in one persistent,
 *                     graph-captured launch.
 *
 * Conventions: complex values are interleaved (re, im) doubles, the layout of
 * std::complex<double>. CSR rows are test DOFs, columns unknown DOFs, as
 * in MatrixFactory (row index = numDof-1 of the test function DOF). All calls
 * return an FG_* status and never throw; fg_last_error() describes the last
 * failure on the calling thread.
 */
#ifndef FEM_G_GB300_H
#define FEM_G_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
enum {
  FG_OK = 0,
  FG_ERR_ARG = 1,         /* invalid argument or inconsistent descriptor */
  FG_ERR_OOM = 2,         /* device or host allocation failed */
  FG_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  FG_ERR_INDEX = 4,       /* an element DOF has no place in the CSR pattern */
  FG_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  FG_ERR_UNSUPPORTED = 6, /* a term/space combination this build does not handle */
  FG_ERR_NO_DEVICE = 7    /* no CUDA device */
};

/* DOF assemble types: same values as gmshfem::dofs::AssembleType (src/dofs/Dof.h:27-35) */
enum {
  FG_AT_UNDEFINED = 0,
  FG_AT_FIXED = 1,
  FG_AT_UNKNOWN = 2,
  FG_AT_UNKNOWN_BUBBLE = 3,
  FG_AT_UNKNOWN_GLOBAL = 4,
  FG_AT_LINKED = 5,
  FG_AT_LINKED_BUBBLE = 6
};

/* ---------------------------------------------------------------- inputs */

/* One element bucket: the elements of one type on one entity (ElementBucket,
 * src/problem/ElementBucket.h:20-43, built from gmsh nodes) */
typedef struct {
  int32_t dim;               /* topological dimension of the elements: 2 or 3 */
  int32_t nodes_per_element; /* geometric nodes per element: 3, 6, 4 or 10 */
  int64_t n_nodes;
  const double *node_xyz;    /* [n_nodes][3] */
  int64_t n_elements;
  const int64_t *elem_nodes; /* [n_elements][nodes_per_element], 0-based */
} fg_mesh_desc;

/* Quadrature rule and the geometric basis on it (GetGaussInfo,
 * src/field/FunctionSpaceInterface.cpp:470-481; gmsh getJacobians) */
typedef struct {
  int32_t nq;
  const double *weights;  /* [nq] */
  const double *geo_val;  /* [nq][nodes_per_element] */
  const double *geo_grad; /* [nq][nodes_per_element][3] reference gradients */
} fg_rule_desc;

/* Function space on the bucket: reference basis per orientation, in the
 * reference's layout bf[(o*nq + q)*ncomp*n + dof*ncomp + comp]
 * (src/term/BilinearTerm.cpp:316) */
enum {
  FG_FORM_0 = 0, /* H1 (Form0): scalar values, gradients mapped by J^-T (FieldEvaluator<Form0/Form1>) */
  FG_FORM_1 = 1  /* HCurl (Form1): vector values mapped by J^-T, curls mapped by J / det
                    (FieldEvaluator<Form1> / <Form2>, src/term/evaluator/FieldEvaluator.h:59-105) */
};
typedef struct {
  int32_t n_basis;      /* basis functions per element (per component of a compound field) */
  int32_t multiplicity; /* 1 (Field) or 3 (CompoundField, DOF = basis*3 + component) */
  int32_t n_orientations;
  const double *basis_val;         /* FG_FORM_0: [n_orientations][nq][n_basis]; FG_FORM_1: [...][n_basis][3] */
  const double *basis_grad;        /* FG_FORM_0: gradients, FG_FORM_1: curls, [n_orientations][nq][n_basis][3] */
  const int32_t *elem_orientation; /* [n_elements] dense orientation, NULL if n_orientations == 1 */
  int32_t form;                    /* FG_FORM_*; for FG_FORM_1 the derivative terms are curl-curl */
} fg_space_desc;

/* Pattern and element DOF map produced by the reference's pre():
 * MatrixFactory _ai/_aj (src/system/MatrixFactory.cpp:188-213) and the
 * IndiceBucket of FieldInterface::fillIndices (src/field/FieldInterface.cpp:1012-1076) */
typedef struct {
  uint64_t n_rows;              /* unknown DOFs */
  const uint64_t *ai;           /* [n_rows + 1] */
  const uint64_t *aj;           /* [ai[n_rows]] */
  const uint64_t *elem_dof_idx; /* [n_elements][n_basis*multiplicity]: numDof - 1 */
  const int32_t *elem_dof_type; /* same shape: FG_AT_* */
  uint64_t n_fixed;             /* fixed DOFs (size of the Dirichlet value array) */
  int32_t upper;                /* 1: symmetric or hermitian storage (the formulation's symmetric()
                                   or hermitian() option): the pattern holds the upper triangle and
                                   entries below the diagonal are not added
                                   (MatrixFactory::addPattern/addValues, "jIndex < iIndex") */
  uint64_t n_linked;            /* linked DOFs (FG_AT_LINKED and FG_AT_LINKED_BUBBLE; elem_dof_idx holds
                                   their index below), e.g. periodic or Bloch conditions */
  const uint64_t *linked_row;   /* [n_linked] the row of each linked DOF's master (MatrixFactory _indicesLC) */
  const double *linked_value;   /* [n_linked][2] its coefficient c (_valuesLC): a linked row adds into its
                                   master's row times conj(c), a linked column into its master's column
                                   times c (MatrixFactory.cpp:233-448, VectorFactory.cpp:122-210).
                                   A linked bubble (the interior DOF of an element linked to one of
                                   another element) adds the same way; its master is a bubble row. */
} fg_system_desc;

/* Coefficient expression: a complex-valued program over the physical point
 * (x, y, z) of a quadrature point and per-element arrays, in reverse Polish
 * order. Mirrors the expression trees of src/function/ (ScalarFunction::evaluate,
 * src/function/ScalarFunction.cpp:203-223) for the operators listed. */
enum {
  FG_OP_CONST = 0,     /* push (re, im) */
  FG_OP_X = 1,         /* push x of the point */
  FG_OP_Y = 2,
  FG_OP_Z = 3,
  FG_OP_ELEM = 4,      /* push elem_values[arg][element] */
  FG_OP_ADD = 5,
  FG_OP_SUB = 6,
  FG_OP_MUL = 7,
  FG_OP_DIV = 8,
  FG_OP_NEG = 9,
  FG_OP_HEAVISIDE = 10, /* 1 if Re>0, 0 if Re<0, 0.5 if Re==0 (unaryOperations.h:1008-1021) */
  FG_OP_FIELD = 11,     /* push u(x) = sum_j phi_j(x) u_e[j]: a scalar field of the bucket's own H1 space
                           at the point (field node, fieldOperations.h:160-170); elem_values[arg] is then
                           [n_elements][nb][2], the field's values at each element's local DOFs */
  /* unary operators on the top of the stack, complex (principal branches), as the reference's
     scalar operators on std::complex<double> (src/function/scalarUnaryOperators.h:27-120,
     executionTree/unaryOperations.h) */
  FG_OP_SQRT = 12,
  FG_OP_EXP = 13,
  FG_OP_LN = 14,    /* natural logarithm: the reference's ln() */
  FG_OP_LOG10 = 15, /* decimal logarithm: the reference's log() */
  FG_OP_POW = 16,   /* a^arg, arg >= 0 an integer (pow(a, n)) */
  FG_OP_SIN = 17,
  FG_OP_COS = 18,
  FG_OP_TAN = 19,
  FG_OP_SINH = 20,
  FG_OP_COSH = 21,
  FG_OP_TANH = 22,
  FG_OP_ASIN = 23,
  FG_OP_ACOS = 24,
  FG_OP_ATAN = 25,
  FG_OP_ASINH = 26,
  FG_OP_ACOSH = 27,
  FG_OP_ATANH = 28,
  FG_OP_ABS = 29,   /* |a| */
  FG_OP_CONJ = 30,
  FG_OP_REAL = 31,
  FG_OP_IMAG = 32,
  FG_OP_CBRT = 33,  /* a^(1/3): real cube root for a > 0, principal complex root otherwise */
  FG_OP_ATAN2 = 34, /* binary: atan2(Re a, Re b) of the two topmost (scalarBinaryOperators.h:21, real arguments) */
  FG_OP_POINT = 35  /* push elem_values[arg][element * nq + q]: the coefficient at every integration point of the
                       bucket, element-major ([n_elements * nq][2] complex), e.g. a Function the caller evaluates with
                       the reference's own evaluator (EquationEvaluator::initialize, EquationEvaluator.h:155-168)
                       instead of describing it; point-dependent, so FP64 paths only */
};
typedef struct {
  int32_t op;
  int32_t arg;
  double re, im;
} fg_instr;

#define FG_EXPR_MAX_CODE 32
#define FG_EXPR_MAX_ARRAYS 4
typedef struct {
  int32_t n_code;
  fg_instr code[FG_EXPR_MAX_CODE];
  int32_t n_arrays;
  const double *elem_values[FG_EXPR_MAX_ARRAYS]; /* [n_elements][2] complex */
} fg_expr;

/* Terms of one formulation on the bucket (one field, one quadrature rule) */
enum {
  FG_TERM_GRAD_GRAD = 0, /* integral(c * grad(dof(u)), grad(tf(u))) */
  FG_TERM_MASS = 1,      /* integral(c * dof(u), tf(u)) */
  FG_TERM_ELASTIC = 2,   /* integral(C * grad(dof(u)), grad(tf(u))), C isotropic Tensor4 (lambda, mu) */
  FG_TERM_SOURCE = 3,    /* integral(f, tf(u)) : right-hand side */
  FG_TERM_GRAD_GRAD_TENSOR = 4, /* integral(c * D * grad(dof(u)), grad(tf(u))), D a symmetric 3x3 tensor of
                                   coefficient programs (TensorFunction * grad, EquationEvaluator tensor-left);
                                   scalar H1 fields; on HCurl fields the curls: integral(c * D * curl, curl) */
  FG_TERM_MASS_TENSOR = 5,       /* integral(c * D * dof(u), tf(u)) for HCurl fields (D symmetric, as above) */
  FG_TERM_GRAD_GRAD_TENSOR_FULL = 6, /* integral(c * D * grad(dof(u)), grad(tf(u))) with a general (not symmetric)
                                        3x3 TensorFunction D: tensor[9], row-major D_00 D_01 ... D_22; scalar H1 fields;
                                        the element matrix is not symmetric (FP64 paths only) */
  FG_TERM_ADVECTION = 7,             /* integral(c * b * grad(dof(u)), tf(u)) with a VectorFunction b: tensor[3],
                                        b_x b_y b_z; scalar H1 fields; not symmetric (FP64 paths only) */
  FG_TERM_VECTOR_GRAD_TEST = 8,      /* integral(c * b * dof(u), grad(tf(u))) with a VectorFunction b: tensor[3];
                                        scalar H1 fields; not symmetric (FP64 paths only) */
  FG_TERM_SOURCE_GRAD = 9            /* integral(f, grad(tf(u))) with a VectorFunction f: tensor[3], coef multiplies
                                        it; right-hand side; scalar H1 fields (FP64 paths only) */
};
enum { FG_DT_NONE = 0, FG_DT_1 = 1, FG_DT_2 = 2 }; /* dof, dt_dof, dt2_dof */

/* Jacobian modificator of the term's domain on this bucket's entity
 * (domain::JacobiansModificator, src/domain/JacobiansModificator.h:16-30,
 * applied per term in Assembler::_assembleBilinear/_assembleLinear,
 * src/term/Assembler.cpp:178-228 and :386-436). At every integration point x
 * the Jacobian becomes J * jac(x) and the determinant det * det(jac(x)):
 * transformation shells that stretch [r_min, r_max) to [r_min, infinity),
 * and the axisymmetric measure r dr dz. An integration point whose shell
 * radius lies outside [r_min, r_max] (10 machine epsilons of slack) is an
 * argument error, reported after the element kernel (the reference throws). */
enum {
  FG_JACMOD_NONE = 0,
  FG_JACMOD_AXISYMMETRY = 1,       /* Axisymmetry.cpp:33-56: J(2,2) = x, det *= x */
  FG_JACMOD_AXISYMMETRY_SHELL = 2, /* AxisymmetryShell.cpp:37-95: r about (0, center[1]), times x */
  FG_JACMOD_POLAR_SHELL = 3,       /* PolarShell.cpp:37-93: 2D, r about (center[0], center[1]) */
  FG_JACMOD_CYLINDRICAL_SHELL = 4, /* CylindricalShell.cpp:37-101: r about the axis through center */
  FG_JACMOD_SPHERICAL_SHELL = 5    /* SphericalShell.cpp:37-95: r about center */
};
typedef struct {
  int32_t kind;     /* FG_JACMOD_* */
  int32_t axis;     /* cylindrical shell: the axis (0, 1 or 2) */
  int32_t exponent; /* shells: the exponent of the stretching (1 by default in the reference) */
  int32_t pad_;
  double r_min, r_max;
  double center[3];
} fg_jacmod;

typedef struct {
  int32_t kind; /* FG_TERM_* */
  int32_t dt;   /* FG_DT_*: with any dt term the AFrequency module applies */
  fg_expr coef; /* c, f, or lambda for FG_TERM_ELASTIC */
  fg_expr coef2; /* mu for FG_TERM_ELASTIC */
  fg_jacmod jacmod; /* all zero: none */
  const fg_expr *tensor; /* FG_TERM_GRAD_GRAD_TENSOR, FG_TERM_MASS_TENSOR: [6] programs of D_xx, D_yy, D_zz, D_xy, D_xz, D_yz;
                            FG_TERM_GRAD_GRAD_TENSOR_FULL: [9] of D row-major; FG_TERM_ADVECTION,
                            FG_TERM_VECTOR_GRAD_TEST, FG_TERM_SOURCE_GRAD: [3] of the vector */
} fg_term_desc;

/* ------------------------------------------------------------- plan / run */

typedef struct fg_plan fg_plan;

/* Builds the device-resident plan for one element bucket: uploads geometry
 * and basis tables, checks every element DOF against the pattern and builds
 * the element->nonzero map used by the deterministic CSR reduction. */
int fg_plan_create(const fg_mesh_desc *mesh, const fg_rule_desc *rule, const fg_space_desc *space,
                   const fg_system_desc *sys, fg_plan **out);
/* Plan for the terms of one bucket whose unknown field differs from their
 * test field (a BilinearTerm with _field[0] != _field[1],
 * src/term/BilinearTerm.cpp:156-273, scattered by MatrixFactory::addValues
 * with the test field's indices as rows and the unknown field's as columns,
 * src/term/Assembler.cpp:256). `space` and sys->elem_dof_idx / elem_dof_type
 * describe the TEST field (the rows); `unknown_space` and unknown_dof_idx /
 * unknown_dof_type ([n_elements][unknown n_basis], numDof - 1 and FG_AT_*)
 * the unknown field (the columns); ai/aj is the formulation's shared pattern.
 * Both fields scalar H1 (FG_FORM_0, multiplicity 1) on the same elements and
 * rule; no linked DOFs. Terms: FG_TERM_GRAD_GRAD, FG_TERM_MASS,
 * FG_TERM_GRAD_GRAD_TENSOR_FULL, FG_TERM_ADVECTION and FG_TERM_VECTOR_GRAD_TEST (with dt factors), no
 * field-value coefficients; linear terms go to the test field's own plan.
 * Assembled by fg_assemble_fp64 / fg_assemble_fp64_static into element
 * matrices of n_test x n_unknown. Set fg_plan_set_accumulate(plan, 1) so that
 * the block adds into the rows the test field's own plan writes. Fixed
 * unknown DOFs lift into the right-hand side through the entry that
 * VectorFactory::addValuesDC reads, values[j * n_unknown + i]
 * (src/system/VectorFactory.cpp:184): the transposed entry when both fields
 * have as many DOFs per element; with different counts that read falls
 * outside the element matrix, and such a call returns FG_ERR_UNSUPPORTED. */
int fg_plan_create_coupled(const fg_mesh_desc *mesh, const fg_rule_desc *rule, const fg_space_desc *space,
                           const fg_system_desc *sys, const fg_space_desc *unknown_space,
                           const uint64_t *unknown_dof_idx, const int32_t *unknown_dof_type, fg_plan **out);
void fg_plan_destroy(fg_plan *plan);
/* Bound on the tensor-core contraction's wait for each chain of MMAs, in
 * seconds (default about 2; process-wide, read at each launch, and at capture
 * time by batch graphs). When a wait runs out, the kernel records a timeout,
 * waits once more (bounded) for the MMAs it issued to retire, frees its TMEM
 * and returns; the call (host outputs) or the next call on the plan (device
 * outputs) returns FG_ERR_TIMEOUT and the device stays usable. 0 makes the
 * first wait give up at once, which tests that path. */
int fg_set_wait_limit(double seconds);
/* plan statistics: nnz, elements, element DOFs, quadrature points, orientations */
int fg_plan_info(const fg_plan *plan, int64_t *nnz, int64_t *n_elements, int32_t *n_dofs, int32_t *nq, int32_t *n_orient);

/* Error report of the mixed path (per element and global, against an FP64
 * evaluation of the same element matrices on the device) */
typedef struct {
  double max_elem_rel_fro;  /* max over elements of ||Ke_mixed - Ke_fp64||_F / ||Ke_fp64||_F */
  double mean_elem_rel_fro;
  double global_rel_fro;    /* ||A_mixed - A_fp64||_F / ||A_fp64||_F over the CSR values */
} fg_err_report;

/* Upload the terms once (coefficient arrays copied to the device) so later
 * assemble calls may pass terms == NULL and reuse them, like the reference's
 * term initialisation (BilinearTerm::assemblyInitialization,
 * src/term/BilinearTerm.cpp:156-273) followed by repeated assembly. */
int fg_plan_bind_terms(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, double frequency);

/* Assemble the system. csr_values ([nnz][2]) and rhs ([n_rows][2]) may be host
 * or device pointers (detected); the values are overwritten (the reference
 * adds into a zeroed module). dirichlet: [n_fixed][2] values of the fixed DOFs
 * (may be NULL when n_fixed == 0). frequency: omega of the AFrequency module,
 * used when a term has dt != 0. rhs may be NULL. stream: a cudaStream_t or NULL.
 * terms == NULL uses the terms bound by fg_plan_bind_terms. With device
 * outputs the call returns once the work is queued on the stream; with host
 * outputs it returns after the results are copied back. */
int fg_assemble_fp64(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, double frequency,
                     const double *dirichlet, double *csr_values, double *rhs, void *stream);
/* No counterpart in the reference. fg_assemble_fp64 with bound terms, but it
 * allocates nothing: its element-matrix and element-vector scratch is a
 * file-scope device array of FG_STATIC_SCRATCH_BYTES per device (64 MiB), and
 * csr_values, rhs (may be NULL) and dirichlet (NULL when n_fixed == 0) must be
 * device memory. For callers that may not call cudaMalloc/cudaFree once set
 * up: cudaFree synchronizes the whole device, which stalls a caller that
 * overlaps the assembly of one step with the solve of the previous one on
 * other streams, and a solver that owns the device memory pool allows no
 * allocation from outside it. Requires fg_plan_bind_terms first. Returns
 * FG_ERR_UNSUPPORTED when the scratch, E * (1 or 2 for complex) * n^2 * 8
 * bytes plus E * n * 16 bytes with a source term and rhs, exceeds the array;
 * FG_ERR_ARG for host outputs or no bound terms. The first call on a device
 * resolves the array's address (cudaGetSymbolAddress, that device current);
 * under CUDA's lazy module loading (the default) that is also when the driver
 * loads the code module holding the array and its 64 MiB of device memory,
 * kept until exit. Make that first call during set-up, before any stream
 * capture. FG_FP64_FACTORED plans build their reference tensors in
 * fg_plan_set_fp64_method, so no later call allocates. The array is shared by all plans on a
 * device: calls in flight at the same time on one device race on it. */
#define FG_STATIC_SCRATCH_BYTES ((size_t)64 << 20)
int fg_assemble_fp64_static(fg_plan *plan, const double *dirichlet, double *csr_values, double *rhs, void *stream);
/* FP64 element-matrix method of a plan. FG_FP64_QUADRATURE (default, the
 * plain method): the quadrature loop of BilinearTerm::evaluate. FG_FP64_FACTORED:
 * where it is exact (affine elements, element-constant coefficients,
 * one-component fields) the factorization Ke = sum_k D_e[k] T_o[k] of the
 * mixed path, kept in FP64 on the CUDA cores; the quadrature loop elsewhere. */
enum { FG_FP64_QUADRATURE = 0, FG_FP64_FACTORED = 1 };
int fg_plan_set_fp64_method(fg_plan *plan, int32_t method);
/* Buckets (element types, entities, boundary terms) that share rows add into
 * one system, as _assembleDim adds every bucket into one module
 * (src/problem/Formulation.cpp:1418-1493). With accumulate = 1 the assemble
 * calls of this plan add its contributions to csr_values and rhs instead of
 * overwriting them; both must then be device memory (FG_ERR_ARG otherwise).
 * Batches, the multi-frequency calls and the mixed error report refuse such
 * a plan. Default 0. */
int fg_plan_set_accumulate(fg_plan *plan, int32_t accumulate);
/* Mixed precision: FP64 geometry, 3xTF32 tcgen05 contraction with FP32
 * accumulation, FP64 CSR reduction. report may be NULL (no error report).
 * By default the contraction writes FP32 element matrices that a separate
 * deterministic reduction reads. With fg_plan_set_mixed_fused(plan, 1), where
 * it applies (one-component H1 fields whose element orientations only flip
 * basis signs, affine elements, real element-constant coefficients, no fixed
 * or linked DOFs, no error report), the contraction and the reduction run
 * fused in one kernel over blocks of consecutive CSR rows, and no element
 * matrix is written to device memory. */
int fg_assemble_mixed(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, double frequency,
                      const double *dirichlet, double *csr_values, double *rhs, void *stream,
                      fg_err_report *report);

/* Fused mixed path on (1) or off (0, the default) for this plan. */
int fg_plan_set_mixed_fused(fg_plan *plan, int32_t on);
/* Whether the fused mixed path applies to the plan (building its block
 * records on first use), its number of row blocks, the mean elements per
 * block and the contractions per element (>= 1: an element whose DOF rows
 * fall in several blocks is contracted in each). When it does not apply,
 * fg_last_error() says why. */
int fg_plan_fused_info(fg_plan *plan, int32_t *applies, int32_t *blocks, double *elems_per_block,
                       double *contractions_per_element);

/* The system at n_freq angular frequencies in one pass: what n_freq calls of
 * fg_assemble_fp64 (mixed == 0) or fg_assemble_mixed (mixed != 0) with
 * frequency = omegas[f] produce, i.e. what the reference's assemble() gives
 * after each change of the formulation's frequency (AFrequency module,
 * src/term/Assembler.cpp:263-305; src/system/MatrixModule.cpp:100-171). The
 * terms are split by time derivative into at most three groups whose element
 * matrices are integrated once; the row-owner reduction then writes
 *   values[f] = K + (-i omega_f) C + (-omega_f^2) M
 * for every frequency. csr_values: [n_freq][nnz][2]; rhs: [n_freq][n_rows][2]
 * or NULL; host or device memory (detected); dirichlet as in fg_assemble_fp64. */
int fg_assemble_multi_freq(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, const double *omegas,
                           int32_t n_freq, int32_t mixed, const double *dirichlet, double *csr_values, double *rhs,
                           void *stream);

/* The system as separate matrices sharing the pattern, the reference's
 * assemble(separate = true) with the MK, CK or MCK module
 * (src/problem/Formulation.cpp:1096-1149, src/term/Assembler.cpp:306-347,
 * src/system/MatrixModule.cpp:180-395): K from the terms without time
 * derivative, C from the dt terms, M from the dt2 terms, each without the
 * frequency factor; the right-hand side holds the sources and the Dirichlet
 * lifting with K alone. An output may be NULL when the formulation has no
 * term of that kind; host or device memory (detected). */
int fg_assemble_separate(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, int32_t mixed, const double *dirichlet,
                         double *k_values, double *c_values, double *m_values, double *rhs, void *stream);

/* -------------------------------------------------------------- batching */

typedef struct fg_batch fg_batch;
/* A batch of independent plans assembled by one persistent kernel launch
 * captured in a CUDA graph; tile shapes per (element type, order, rule) come
 * from the built-in autotuner on the first run. */
int fg_batch_create(fg_plan *const *plans, const fg_term_desc *const *terms, const int32_t *n_terms,
                    int32_t n_problems, int32_t mixed, fg_batch **out);
/* values[p] / rhs[p]: device or host output arrays per problem (NULL rhs allowed).
 * While the kernel timer is on (fg_profile_enable), a run issues the graph's
 * launches one by one instead of the graph, so that each kernel is timed. */
int fg_batch_run(fg_batch *batch, double *const *csr_values, double *const *rhs, void *stream);
void fg_batch_destroy(fg_batch *batch);
/* JSON description of the shapes the autotuner chose in the first run
 * (reduction lanes and warps per class, MMA width per contraction class);
 * empty before it. Valid until the next call on the batch. */
const char *fg_batch_tuning(const fg_batch *batch);

/* --------------------------------------------------------- symbolic phase */

/* GPU symbolic assembly of one element bucket's CSR pattern, the part of the
 * reference's pre() done by MatrixFactory::addPattern
 * (src/system/MatrixFactory.cpp:459-539) and finalizePattern (:188-213) when
 * the test and unknown DOFs are one field: row I (an Unknown, Unknown bubble
 * or Unknown global DOF) holds the sorted unique Unknown DOFs of the elements
 * that have I, Fixed DOFs take no column, and the bubble rows of an element
 * after its first alias that row. elem_dof_idx / elem_dof_type as in
 * fg_system_desc ([n_elements][n_dofs]). ai: [n_rows + 1], the caller's;
 * *aj: [ai[n_rows]] allocated by the call (free it with fg_host_free).
 * upper = 1: symmetric storage, only the columns J >= I of a row (for an
 * aliased bubble row, those of the first bubble's row). linked_row
 * ([n_linked], as in fg_system_desc): an FG_AT_LINKED DOF is a row and a
 * column of its master; an FG_AT_LINKED_BUBBLE DOF is a bubble row of its
 * master's, and the bubble rows of the master element and of the linked one
 * share one pattern (the columns of both elements; with upper = 1, each
 * element's from its own first bubble's row); NULL when there are none. */
int fg_pattern_build(const uint64_t *elem_dof_idx, const int32_t *elem_dof_type, int64_t n_elements, int32_t n_dofs,
                     uint64_t n_rows, uint64_t *ai, uint64_t **aj, int32_t upper, const uint64_t *linked_row,
                     uint64_t n_linked);

/* GPU Hilbert order of n points (float [n][dim], dim 2 or 3) in the box
 * [mn, mx]: the stable order of the keys of src/reorder/Hilbert.cpp:174-288
 * (perm[k] = index of the k-th point). */
int fg_hilbert_order(int32_t dim, uint64_t n, const float *pts, const float *mn, const float *mx, uint32_t *perm);
/* GPU DOF numbering, DofsManager::reorderWithHilbert(true)
 * (src/dofs/DofsManager.cpp:118-331): the DOFs in dictionary iteration order
 * (xyz [n_dofs][3] float, FG_AT_* types); Unknown DOFs get 1..nu-nb in
 * Hilbert order, Unknown bubble DOFs nu-nb+1..nu; the other entries of
 * num_dof are left as they are. bbox: xmin, ymin, zmin, xmax, ymax, zmax. */
int fg_hilbert_numbering(int32_t dim, const double *bbox, uint64_t n_dofs, const float *xyz, const int32_t *assemble_type,
                         uint64_t *num_dof);

/* ----------------------------------------------------------------- misc */

const char *fg_last_error(void);
/* number of kernel launches issued by this library since load (for the
 * launch count a benchmark reports) */
int64_t fg_launch_count(void);
/* Kernel timer: while enabled, every kernel this library launches is
 * bracketed by CUDA events on its launch stream. fg_profile_read synchronizes
 * the recorded events and returns, per kernel name, the launch count and the
 * summed device milliseconds (names separated by '\n' in names[name_bytes]);
 * it returns the number of kernels and clears the record. */
int fg_profile_enable(int on);
int fg_profile_read(char *names, int32_t name_bytes, int64_t *launches, double *total_ms, int32_t cap);

/* page-locked host buffers for end-to-end transfers */
int fg_host_alloc(void **ptr, size_t bytes);
void fg_host_free(void *ptr);

#ifdef __cplusplus
}
#endif

#endif /* FEM_G_GB300_H */
