/*
 * CPU oracle for the GmshFEM assembly path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithms, used by the tests, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline legs as the checker.
 * The product (libfemg.so) never links or calls this code.
 *
 * Each function cites the reference code it restates (paths inside the
 * reference project GmshFEM 1.0.0, directory fem-master/).
 *
 * Parity pinning: the reference has no golden element matrices or CSR
 * fixtures (its tests need gmsh + PETSc). The numbering pieces (robin-hood
 * iteration order, Hilbert keys and sort) are pinned against the reference's
 * own robin_hood.h and Hilbert.cpp compiled in oracle/_ref; the matrix
 * pieces (evaluate, addValues, addValuesDC) are pinned against exact
 * closed-form element matrices (P1 stiffness/mass) in the tests.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* ---------------------------------------------------------------- types */

enum { AT_UNDEFINED = 0, AT_FIXED = 1, AT_UNKNOWN = 2, AT_UNKNOWN_BUBBLE = 3, AT_UNKNOWN_GLOBAL = 4 };
enum {
  TERM_GRAD_GRAD = 0,
  TERM_MASS = 1,
  TERM_ELASTIC = 2,
  TERM_SOURCE = 3,
  TERM_GRAD_GRAD_TENSOR = 4,
  TERM_MASS_TENSOR = 5,
  TERM_GRAD_GRAD_TENSOR_FULL = 6,
  TERM_ADVECTION = 7,
  TERM_VECTOR_GRAD_TEST = 8,
  TERM_SOURCE_GRAD = 9
};
enum { OP_CONST = 0, OP_X, OP_Y, OP_Z, OP_ELEM, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_NEG, OP_HEAVISIDE, OP_FIELD,
       OP_SQRT, OP_EXP, OP_LN, OP_LOG10, OP_POW, OP_SIN, OP_COS, OP_TAN, OP_SINH, OP_COSH, OP_TANH, OP_ASIN, OP_ACOS,
       OP_ATAN, OP_ASINH, OP_ACOSH, OP_ATANH, OP_ABS, OP_CONJ, OP_REAL, OP_IMAG, OP_CBRT, OP_ATAN2, OP_POINT };

/* same memory layout as fg_instr / fg_expr / fg_term_desc of the C ABI, so
 * the tests can pass the product's term descriptors unchanged */
typedef struct {
  int32_t op, arg;
  double re, im;
} or_instr;
typedef struct {
  int32_t n_code;
  or_instr code[32];
  int32_t n_arrays;
  const double *elem_values[4];
} or_expr;
typedef struct {
  int32_t kind, axis, exponent, pad_;
  double r_min, r_max, center[3];
} or_jacmod;
typedef struct {
  int32_t kind, dt;
  or_expr coef, coef2;
  or_jacmod jacmod;
  const or_expr *tensor; /* TERM_GRAD_GRAD_TENSOR, TERM_MASS_TENSOR: D_xx, D_yy, D_zz, D_xy, D_xz, D_yz;
                            TERM_GRAD_GRAD_TENSOR_FULL: D row-major [9]; TERM_ADVECTION, TERM_VECTOR_GRAD_TEST,
                            TERM_SOURCE_GRAD: the vector [3] */
} or_term;

typedef struct {
  int dim, nn, nq, nb, mult;
  int64_t E;
  const double *xyz;      /* [nodes][3] */
  const int64_t *enodes;  /* [E][nn] */
  const double *w;        /* [nq] */
  const double *geo_val;  /* [nq][nn] */
  const double *geo_grad; /* [nq][nn][3] */
  const double *bval;     /* [no][nq][nb] */
  const double *bgrad;    /* [no][nq][nb][3] */
  const int32_t *orient;  /* [E] (NULL: one table, Lagrange's isConstantByElements) */
  int32_t form;           /* 0: H1 (bval scalar, bgrad gradients); 1: HCurl (bval [..][nb][3] values, bgrad curls) */
  int32_t upper;          /* symmetric()/hermitian() storage: columns J >= I only */
  const uint64_t *linked_row; /* [n_linked] master row of a linked DOF (MatrixFactory _indicesLC), or NULL */
  const double *linked_value; /* [n_linked][2] its coefficient (_valuesLC) */
} or_bucket;

enum { AT_LINKED = 5, AT_LINKED_BUBBLE = 6 };

/* Row (or column) of an element DOF and its scale: Unknown-like DOFs are
 * their own row with scale 1; a linked DOF is its master's row with its
 * coefficient (MatrixFactory.cpp:241-246, :254-259). Returns 0 for the DOFs
 * that take no row (fixed, undefined). */
static int or_dof_row(const or_bucket *b, int t, uint64_t idx, uint64_t *row, cplx *scale) {
  if (t == AT_UNKNOWN || t == AT_UNKNOWN_BUBBLE || t == AT_UNKNOWN_GLOBAL) {
    *row = idx;
    *scale = 1.0;
    return 1;
  }
  if ((t == AT_LINKED || t == AT_LINKED_BUBBLE) && b->linked_row) {
    *row = b->linked_row[idx];
    *scale = b->linked_value[2 * idx] + I * b->linked_value[2 * idx + 1];
    return 1;
  }
  return 0;
}

/* -------------------------------------------------------- expressions */

/* Function::evaluate for the operator subset of the ABI
 * (src/function/ScalarFunction.cpp:203-223; nullary x/y/z/constant
 * src/function/executionTree/nullaryOperations.h:284-345,1399-1484; heaviside
 * src/function/executionTree/unaryOperations.h:1008-1021; the other unary
 * operators or_unary above) */
/* phi: the bucket's scalar basis values at the point (nb of them), for the
 * field-node op: u(x) = sum_j phi_j u_e[j] with the element's DOF values u_e
 * (fieldOperations.h:160-170, Form0 field evaluated on the gauss points) */
/* z^p for a real power p, as std::pow(complex<double>, double) computes it:
 * x^p for a real positive z, else |z|^p e^(i p arg z) through the logarithm */
static cplx or_pow_real(cplx z, double p) {
  if (cimag(z) == 0.0 && creal(z) > 0.0) return pow(creal(z), p);
  cplx t = clog(z);
  double r = exp(p * creal(t)), th = p * cimag(t);
  return r * cos(th) + I * (r * sin(th));
}

/* The scalar unary operators of src/function/scalarUnaryOperators.h:27-120
 * (executionTree/unaryOperations.h) on std::complex<double>, whose functions
 * are the C99 complex ones: log() is the decimal logarithm (std::log10),
 * ln() the natural one; pow(a, n) multiplies for n <= 4 (Pow::operator(),
 * unaryOperations.h:1517-1549) and uses std::pow beyond; cbrt is
 * std::pow(a, 1/3) for complex scalars. */
static cplx or_unary(int op, int arg, cplx z) {
  switch (op) {
    case OP_NEG: return -z;
    case OP_HEAVISIDE: {
      double r = creal(z);
      return r > 0.0 ? 1.0 : (r < 0.0 ? 0.0 : 0.5);
    }
    case OP_SQRT: return csqrt(z);
    case OP_EXP: return cexp(z);
    case OP_LN: return clog(z);
    case OP_LOG10: return clog(z) / log(10.0);
    case OP_POW:
      if (arg == 1) return z;
      if (arg == 2) return z * z;
      if (arg == 3) return z * z * z;
      if (arg == 4) {
        cplx z2 = z * z;
        return z2 * z2;
      }
      return or_pow_real(z, (double)arg);
    case OP_CBRT: return or_pow_real(z, 1.0 / 3.0);
    case OP_SIN: return csin(z);
    case OP_COS: return ccos(z);
    case OP_TAN: return ctan(z);
    case OP_SINH: return csinh(z);
    case OP_COSH: return ccosh(z);
    case OP_TANH: return ctanh(z);
    case OP_ASIN: return casin(z);
    case OP_ACOS: return cacos(z);
    case OP_ATAN: return catan(z);
    case OP_ASINH: return casinh(z);
    case OP_ACOSH: return cacosh(z);
    case OP_ATANH: return catanh(z);
    case OP_ABS: return cabs(z);
    case OP_CONJ: return conj(z);
    case OP_REAL: return creal(z);
    case OP_IMAG: return cimag(z);
  }
  return z;
}

static cplx eval_expr(const or_expr *ex, int64_t e, const double *x, const double *phi, int nb, int q, int nq) {
  cplx st[16];
  int sp = 0;
  for (int k = 0; k < ex->n_code; ++k) {
    const or_instr *in = &ex->code[k];
    switch (in->op) {
      case OP_CONST: st[sp++] = in->re + I * in->im; break;
      case OP_X: st[sp++] = x[0]; break;
      case OP_Y: st[sp++] = x[1]; break;
      case OP_Z: st[sp++] = x[2]; break;
      case OP_ELEM: st[sp++] = ex->elem_values[in->arg][2 * e] + I * ex->elem_values[in->arg][2 * e + 1]; break;
      /* the coefficient at point q of element e, from a table the caller filled */
      case OP_POINT: {
        const double *v = ex->elem_values[in->arg] + 2 * ((size_t)e * nq + q);
        st[sp++] = v[0] + I * v[1];
        break;
      }
      case OP_FIELD: {
        const double *u = ex->elem_values[in->arg] + 2 * (size_t)e * nb;
        cplx s = 0.0;
        for (int j = 0; phi && j < nb; ++j) s += phi[j] * (u[2 * j] + I * u[2 * j + 1]);
        st[sp++] = s;
        break;
      }
      case OP_ADD:
      case OP_SUB:
      case OP_MUL:
      case OP_DIV:
      case OP_ATAN2: {
        cplx b = st[--sp];
        cplx a = st[sp - 1];
        if (in->op == OP_ADD) a = a + b;
        else if (in->op == OP_SUB) a = a - b;
        else if (in->op == OP_MUL) a = a * b;
        else if (in->op == OP_DIV) a = a / b;
        else a = atan2(creal(a), creal(b)); /* scalarBinaryOperators.h:21, real arguments */
        st[sp - 1] = a;
        break;
      }
      default: st[sp - 1] = or_unary(in->op, in->arg, st[sp - 1]);
    }
  }
  return st[0];
}

/* --------------------------------------------------------- geometry */

/* gmsh getJacobians as consumed by the reference (src/term/Assembler.cpp:131-139,
 * column-major 3x3 Map in src/term/evaluator/FieldEvaluator.h:69): J(r,c) =
 * sum_k x_k[r] dN_k/du_c stored at J[3c + r]; 2D elements complete the third
 * column with the unit normal. Returns det. */
static double or_jacobian(const or_bucket *b, int64_t e, int q, double *J, double *xq) {
  memset(J, 0, 9 * sizeof(double));
  xq[0] = xq[1] = xq[2] = 0.0;
  for (int k = 0; k < b->nn; ++k) {
    const double *X = b->xyz + 3 * b->enodes[e * b->nn + k];
    for (int c = 0; c < b->dim; ++c) {
      double g = b->geo_grad[((size_t)q * b->nn + k) * 3 + c];
      for (int r = 0; r < 3; ++r) J[3 * c + r] += X[r] * g;
    }
    double v = b->geo_val[(size_t)q * b->nn + k];
    for (int r = 0; r < 3; ++r) xq[r] += v * X[r];
  }
  if (b->dim == 2) {
    double nx = J[1] * J[5] - J[2] * J[4], ny = J[2] * J[3] - J[0] * J[5], nz = J[0] * J[4] - J[1] * J[3];
    double l = sqrt(nx * nx + ny * ny + nz * nz);
    J[6] = nx / l;
    J[7] = ny / l;
    J[8] = nz / l;
  }
#define M(r, c) J[3 * (c) + (r)]
  return M(0, 0) * (M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1)) - M(0, 1) * (M(1, 0) * M(2, 2) - M(1, 2) * M(2, 0)) +
         M(0, 2) * (M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0));
#undef M
}

/* Jacobian modificators, restated from the reference's five implementations:
 *   Axisymmetry      src/domain/Axisymmetry.cpp:33-56
 *   AxisymmetryShell src/domain/AxisymmetryShell.cpp:37-95
 *   PolarShell       src/domain/PolarShell.cpp:37-93
 *   CylindricalShell src/domain/CylindricalShell.cpp:37-101
 *   SphericalShell   src/domain/SphericalShell.cpp:37-95
 * applied by Assembler::_assembleBilinear / _assembleLinear to the term's
 * Jacobians and determinants (src/term/Assembler.cpp:208-228, :416-436).
 * Row-major storage as gmsh returns it: jac[9i + 3k + l] = dx_l/du_k, which is
 * the J[3c + r] layout used here. Returns 0, or 1 when the radius lies
 * outside the shell (the reference throws). */
enum { JM_NONE = 0, JM_AXI, JM_AXI_SHELL, JM_POLAR, JM_CYL, JM_SPH };
static int or_jacmod_apply(const or_jacmod *m, const double *x, double *J, double *det) {
  const double eps = 2.220446049250313e-16;
  if (m->kind == JM_NONE) return 0;
  if (m->kind == JM_AXI) {
    double R = x[0];
    if (R == 0.) R = eps;
    J[8] = R;
    *det *= R;
    return 0;
  }
  double R, dRdx[3] = {0., 0., 0.}, S = x[0];
  int two = m->kind == JM_AXI_SHELL || m->kind == JM_POLAR;
  if (m->kind == JM_AXI_SHELL) {
    R = sqrt(x[0] * x[0] + (x[1] - m->center[1]) * (x[1] - m->center[1]));
  } else {
    double R2 = 0.;
    for (int j = 0; j < (two ? 2 : 3); ++j) {
      if (m->kind == JM_CYL && j == m->axis) continue;
      R2 += (x[j] - m->center[j]) * (x[j] - m->center[j]);
    }
    R = sqrt(R2);
  }
  if (R < m->r_min - 10. * eps || R > m->r_max + 10. * eps) return 1;
  if (R >= m->r_max) R = m->r_max - 10 * eps;
  if (m->kind == JM_AXI_SHELL) {
    if (S == 0.) S = eps;
    dRdx[0] = x[0] / R;
    dRdx[1] = (x[1] - m->center[1]) / R;
  } else {
    for (int j = 0; j < (two ? 2 : 3); ++j) dRdx[j] = (m->kind == JM_CYL && j == m->axis) ? 0. : (x[j] - m->center[j]) / R;
  }
  const double f = pow((m->r_min * (m->r_max - m->r_min)) / (R * (m->r_max - R)), m->exponent);
  const double theta = m->exponent * (m->r_max - 2. * R) / (m->r_max - R);
  double jac[3][3], nj[9];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) jac[a][b] = f * ((a == b ? 1.0 : 0.0) - theta * dRdx[a] * dRdx[b]);
  if (!two) {
    if (m->kind == JM_CYL) jac[m->axis][m->axis] = 1.;
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) nj[k * 3 + l] = J[k * 3 + 0] * jac[0][l] + J[k * 3 + 1] * jac[1][l] + J[k * 3 + 2] * jac[2][l];
    *det *= m->kind == JM_CYL ? f * f * (1.0 - theta) : f * f * f * (1.0 - theta);
  } else {
    for (int k = 0; k < 2; ++k)
      for (int l = 0; l < 2; ++l) nj[k * 3 + l] = J[k * 3 + 0] * jac[0][l] + J[k * 3 + 1] * jac[1][l];
    nj[2] = nj[5] = nj[6] = nj[7] = 0.;
    if (m->kind == JM_POLAR) {
      nj[8] = 1.;
      *det *= f * f * (1.0 - theta);
    } else {
      nj[8] = S * f;
      *det *= S * (f * f * f * (1.0 - theta));
    }
  }
  memcpy(J, nj, sizeof(nj));
  return 0;
}
static int or_jacmod_err = 0;

/* FieldEvaluator<Form1>: J^T.inverse() * bf (src/term/evaluator/FieldEvaluator.h:67-70);
 * out G[3][nb] */
static void or_form1(const double *J, const double *bf, int nb, double *G) {
  /* K = J^T; Kinv = K^-1 by cofactors */
  double K[3][3], Ki[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) K[r][c] = J[3 * r + c]; /* K(r,c) = J(c,r) */
  double det = K[0][0] * (K[1][1] * K[2][2] - K[1][2] * K[2][1]) - K[0][1] * (K[1][0] * K[2][2] - K[1][2] * K[2][0]) +
               K[0][2] * (K[1][0] * K[2][1] - K[1][1] * K[2][0]);
  Ki[0][0] = (K[1][1] * K[2][2] - K[1][2] * K[2][1]) / det;
  Ki[0][1] = (K[0][2] * K[2][1] - K[0][1] * K[2][2]) / det;
  Ki[0][2] = (K[0][1] * K[1][2] - K[0][2] * K[1][1]) / det;
  Ki[1][0] = (K[1][2] * K[2][0] - K[1][0] * K[2][2]) / det;
  Ki[1][1] = (K[0][0] * K[2][2] - K[0][2] * K[2][0]) / det;
  Ki[1][2] = (K[0][2] * K[1][0] - K[0][0] * K[1][2]) / det;
  Ki[2][0] = (K[1][0] * K[2][1] - K[1][1] * K[2][0]) / det;
  Ki[2][1] = (K[0][1] * K[2][0] - K[0][0] * K[2][1]) / det;
  Ki[2][2] = (K[0][0] * K[1][1] - K[0][1] * K[1][0]) / det;
  for (int d = 0; d < nb; ++d)
    for (int r = 0; r < 3; ++r) G[r * nb + d] = Ki[r][0] * bf[3 * d] + Ki[r][1] * bf[3 * d + 1] + Ki[r][2] * bf[3 * d + 2];
}

/* -------------------------------------------------- element matrices */

/* Element matrix of one element, A_e column-major (Eigen): Ae[j + i*n] = A_e(j, i)
 * with j the unknown (lhs) index and i the test (rhs) index.
 *   BilinearTerm::evaluate, Hermitian product (src/term/BilinearTerm.cpp:314-326):
 *     A_e += w_q det_q * expressionLhs^T * conj(expressionRhs)
 *   with expressionLhs = c(e,q) * field (EquationEvaluator Left scalar,
 *   src/term/evaluator/EquationEvaluator.h:170-173), expressionRhs = field,
 *   field = FieldEvaluator<Form0> (bf values) or <Form1> (J^-T grad bf);
 *   the Tensor4 compound case (src/term/evaluator/EquationEvaluator.h:1222-1297,
 *   CompoundFieldEvaluator<Form1,3> src/term/evaluator/FieldEvaluator.h:149-188)
 *   for an isotropic C = lambda d_ij d_kl + mu (d_ik d_jl + d_il d_jk).
 *   Module combination (src/term/Assembler.cpp:263-305): AModule adds every
 *   term; AFrequency adds -w^2 * (dt2 terms) and -i w * (dt1 terms).
 * Also the element right-hand side of LinearTerm::evaluate (Hermitian,
 * src/term/LinearTerm.cpp:182-191): b_e += w det conj(phi) f(q). */
static void or_element(const or_bucket *b, const or_term *terms, int nterms, double freq, int64_t e, cplx *Ae, cplx *be, cplx *tmp,
                       double *G, double *phi, int bilinear) {
  const int nb = b->nb, mult = b->mult, n = nb * mult, nq = b->nq;
  const int o = b->orient ? b->orient[e] : 0;
  int frequencyModule = 0;
  for (int t = 0; t < nterms; ++t)
    if (terms[t].dt) frequencyModule = 1;
  for (int k = 0; k < n * n; ++k) Ae[k] = 0.0;
  if (be)
    for (int k = 0; k < n; ++k) be[k] = 0.0;
  for (int t = 0; t < nterms; ++t) {
    const or_term *T = &terms[t];
    cplx *target = (frequencyModule && T->dt) ? tmp : Ae;
    const int linear = T->kind == TERM_SOURCE || T->kind == TERM_SOURCE_GRAD;
    if (!linear && !bilinear) continue;
    if (T->kind == TERM_SOURCE_GRAD) {
      /* a VectorFunction f tested against grad(tf(u)): b_e[i] += w det conj(G_i) . (c f)
       * (LinearTerm::evaluate, src/term/LinearTerm.cpp:182-191, with FieldEvaluator<Form1>) */
      if (!be || b->form == 1) continue;
      for (int q = 0; q < nq; ++q) {
        double J[9], xq[3];
        double det = or_jacobian(b, e, q, J, xq);
        if (or_jacmod_apply(&T->jacmod, xq, J, &det)) or_jacmod_err = 1;
        const double *bf = b->bval + ((size_t)o * nq + q) * nb;
        const cplx c = eval_expr(&T->coef, e, xq, bf, nb, q, nq);
        cplx fv[3];
        for (int k = 0; k < 3; ++k) fv[k] = c * eval_expr(&T->tensor[k], e, xq, bf, nb, q, nq);
        or_form1(J, b->bgrad + ((size_t)o * nq + q) * nb * 3, nb, G);
        for (int i = 0; i < nb; ++i) be[i] += b->w[q] * det * (conj(G[i]) * fv[0] + conj(G[nb + i]) * fv[1] + conj(G[2 * nb + i]) * fv[2]);
      }
      continue;
    }
    if (T->kind == TERM_SOURCE) {
      if (!be || b->form == 1) continue; /* scalar sources only (H1 test functions) */
      for (int q = 0; q < nq; ++q) {
        double J[9], xq[3];
        double det = or_jacobian(b, e, q, J, xq);
        if (or_jacmod_apply(&T->jacmod, xq, J, &det)) or_jacmod_err = 1;
        const double *bf = b->bval + ((size_t)o * nq + q) * nb;
        cplx f = eval_expr(&T->coef, e, xq, bf, nb, q, nq);
        for (int i = 0; i < nb; ++i)
          for (int c = 0; c < mult; ++c) be[i * mult + c] += b->w[q] * det * conj(bf[i]) * f;
      }
      continue;
    }
    if (target == tmp)
      for (int k = 0; k < n * n; ++k) tmp[k] = 0.0;
    for (int q = 0; q < nq; ++q) {
      double J[9], xq[3];
      double det = or_jacobian(b, e, q, J, xq);
      if (or_jacmod_apply(&T->jacmod, xq, J, &det)) or_jacmod_err = 1;
      const double wd = b->w[q] * det;
      const double *ph = b->form == 0 ? b->bval + ((size_t)o * nq + q) * nb : NULL;
      cplx c = eval_expr(&T->coef, e, xq, ph, nb, q, nq);
      if (T->kind == TERM_MASS && b->form == 1) {
        /* FieldEvaluator<Form1>: J^-T applied to the vector values */
        or_form1(J, b->bval + ((size_t)o * nq + q) * nb * 3, nb, G);
        for (int ii = 0; ii < n; ++ii)
          for (int jj = 0; jj < n; ++jj) {
            cplx s = 0.0;
            for (int r = 0; r < 3; ++r) s += (c * G[r * nb + jj]) * conj(G[r * nb + ii]);
            target[jj + ii * n] += wd * s;
          }
      } else if (T->kind == TERM_GRAD_GRAD && b->form == 1) {
        /* the curl of a Form1 field is a Form2 field: FieldEvaluator<Form2>,
         * J / det applied to the reference curls (FieldEvaluator.h:93-96) */
        const double *cf = b->bgrad + ((size_t)o * nq + q) * nb * 3;
        for (int i = 0; i < nb; ++i)
          for (int r = 0; r < 3; ++r) G[r * nb + i] = (J[r] * cf[3 * i] + J[3 + r] * cf[3 * i + 1] + J[6 + r] * cf[3 * i + 2]) / det;
        for (int ii = 0; ii < n; ++ii)
          for (int jj = 0; jj < n; ++jj) {
            cplx s = 0.0;
            for (int r = 0; r < 3; ++r) s += (c * G[r * nb + jj]) * conj(G[r * nb + ii]);
            target[jj + ii * n] += wd * s;
          }
      } else if (T->kind == TERM_MASS) {
        const double *bf = b->bval + ((size_t)o * nq + q) * nb;
        for (int k = 0; k < nb; ++k) phi[k] = bf[k];
        /* compound Form0: 3 x 3nb field, component c of dof i at row c */
        for (int ii = 0; ii < n; ++ii)
          for (int jj = 0; jj < n; ++jj) {
            if (ii % mult != jj % mult) continue;
            target[jj + ii * n] += wd * (c * phi[jj / mult]) * conj(phi[ii / mult]);
          }
      } else if (T->kind == TERM_GRAD_GRAD_TENSOR || T->kind == TERM_MASS_TENSOR) {
        /* tensor-left evaluator (EquationEvaluator, TensorFunction * field): the unknown's
         * field is c D G_j, tested against G_i, with G the physical gradients (H1),
         * curls (HCurl, grad-grad kind: J / det on the reference curls) or
         * values (HCurl, mass kind: J^-T on the reference values) */
        static const int ab[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
        cplx D[3][3];
        for (int k = 0; k < 6; ++k) {
          const cplx d = c * eval_expr(&T->tensor[k], e, xq, ph, nb, q, nq);
          D[ab[k][0]][ab[k][1]] = D[ab[k][1]][ab[k][0]] = d;
        }
        if (b->form == 1 && T->kind == TERM_GRAD_GRAD_TENSOR) {
          const double *cf = b->bgrad + ((size_t)o * nq + q) * nb * 3;
          for (int i = 0; i < nb; ++i)
            for (int r = 0; r < 3; ++r) G[r * nb + i] = (J[r] * cf[3 * i] + J[3 + r] * cf[3 * i + 1] + J[6 + r] * cf[3 * i + 2]) / det;
        } else if (b->form == 1) {
          or_form1(J, b->bval + ((size_t)o * nq + q) * nb * 3, nb, G);
        } else {
          or_form1(J, b->bgrad + ((size_t)o * nq + q) * nb * 3, nb, G);
        }
        for (int ii = 0; ii < n; ++ii)
          for (int jj = 0; jj < n; ++jj) {
            cplx s = 0.0;
            for (int r = 0; r < 3; ++r)
              for (int t = 0; t < 3; ++t) s += D[r][t] * G[t * nb + jj] * G[r * nb + ii];
            target[jj + ii * n] += wd * s;
          }
      } else if (T->kind == TERM_GRAD_GRAD_TENSOR_FULL) {
        /* a general TensorFunction: the unknown's field is c D G_j (row-major D) */
        cplx D[3][3];
        for (int k = 0; k < 9; ++k) D[k / 3][k % 3] = c * eval_expr(&T->tensor[k], e, xq, ph, nb, q, nq);
        or_form1(J, b->bgrad + ((size_t)o * nq + q) * nb * 3, nb, G);
        for (int ii = 0; ii < n; ++ii)
          for (int jj = 0; jj < n; ++jj) {
            cplx s = 0.0;
            for (int r = 0; r < 3; ++r)
              for (int t = 0; t < 3; ++t) s += D[r][t] * G[t * nb + jj] * G[r * nb + ii];
            target[jj + ii * n] += wd * s;
          }
      } else if (T->kind == TERM_VECTOR_GRAD_TEST) {
        /* VectorFunction b times dof(u), tested against grad(tf(u)): (c b phi_j) . conj(G_i) */
        cplx bv[3];
        for (int k = 0; k < 3; ++k) bv[k] = c * eval_expr(&T->tensor[k], e, xq, ph, nb, q, nq);
        or_form1(J, b->bgrad + ((size_t)o * nq + q) * nb * 3, nb, G);
        const double *bf = b->bval + ((size_t)o * nq + q) * nb;
        for (int ii = 0; ii < n; ++ii)
          for (int jj = 0; jj < n; ++jj) {
            cplx s = bv[0] * conj(G[ii]) + bv[1] * conj(G[nb + ii]) + bv[2] * conj(G[2 * nb + ii]);
            target[jj + ii * n] += wd * s * bf[jj];
          }
      } else if (T->kind == TERM_ADVECTION) {
        /* VectorFunction b times grad(dof u), tested against tf(u): (c b . G_j) conj(phi_i) */
        cplx bv[3];
        for (int k = 0; k < 3; ++k) bv[k] = c * eval_expr(&T->tensor[k], e, xq, ph, nb, q, nq);
        or_form1(J, b->bgrad + ((size_t)o * nq + q) * nb * 3, nb, G);
        const double *bf = b->bval + ((size_t)o * nq + q) * nb;
        for (int ii = 0; ii < n; ++ii)
          for (int jj = 0; jj < n; ++jj) {
            cplx s = bv[0] * G[jj] + bv[1] * G[nb + jj] + bv[2] * G[2 * nb + jj];
            target[jj + ii * n] += wd * s * conj(bf[ii]);
          }
      } else if (T->kind == TERM_GRAD_GRAD) {
        or_form1(J, b->bgrad + ((size_t)o * nq + q) * nb * 3, nb, G);
        for (int ii = 0; ii < n; ++ii)
          for (int jj = 0; jj < n; ++jj) {
            if (ii % mult != jj % mult) continue;
            const int i = ii / mult, j = jj / mult;
            cplx s = 0.0;
            for (int r = 0; r < 3; ++r) s += (c * G[r * nb + j]) * conj(G[r * nb + i]);
            target[jj + ii * n] += wd * s;
          }
      } else if (T->kind == TERM_ELASTIC) {
        /* (C : grad u) : grad v with grad u_{a,k} = d u_a / d x_k: for unknown
         * DOF (j, beta) the field is the 3x3 matrix D with D[beta][k] = G[k][j];
         * C : D = lambda tr(D) I + mu (D + D^T) */
        cplx lam = c, mu = eval_expr(&T->coef2, e, xq, ph, nb, q, nq);
        or_form1(J, b->bgrad + ((size_t)o * nq + q) * nb * 3, nb, G);
        for (int ii = 0; ii < n; ++ii)
          for (int jj = 0; jj < n; ++jj) {
            const int i = ii / 3, al = ii % 3, j = jj / 3, be2 = jj % 3;
            /* sum_{a,k} (C:Dj)[a][k] * Di[a][k], Di[a][k] = (a == al) G[k][i] */
            cplx s = 0.0;
            for (int k = 0; k < 3; ++k) {
              /* (C:Dj)[al][k] = lambda tr(Dj) d(al,k) + mu (Dj[al][k] + Dj[k][al]) */
              cplx trDj = G[be2 * nb + j];
              cplx CD = (al == k ? lam * trDj : 0.0) + mu * ((al == be2 ? G[k * nb + j] : 0.0) + (k == be2 ? G[al * nb + j] : 0.0));
              s += CD * G[k * nb + i];
            }
            target[jj + ii * n] += wd * s;
          }
      }
    }
    if (target == tmp) {
      cplx factor = T->dt == 2 ? -freq * freq : -I * freq;
      for (int k = 0; k < n * n; ++k) Ae[k] += factor * tmp[k];
    }
  }
}

/* Element matrices in the product's layout Ke[e][i][j] (i test, j unknown),
 * for direct per-element comparison; be[e][i]. */
int or_element_matrices(const or_bucket *b, const or_term *terms, int nterms, double freq, double *ke, double *be) {
  const int n = b->nb * b->mult;
#pragma omp parallel
  {
    cplx *Ae = malloc(sizeof(cplx) * n * n), *tmp = malloc(sizeof(cplx) * n * n), *bl = malloc(sizeof(cplx) * n);
    double *G = malloc(sizeof(double) * 3 * b->nb), *phi = malloc(sizeof(double) * b->nb);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < b->E; ++e) {
      or_element(b, terms, nterms, freq, e, Ae, be ? bl : NULL, tmp, G, phi, 1);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          cplx v = Ae[j + i * n];
          ke[2 * (((size_t)e * n + i) * n + j)] = creal(v);
          ke[2 * (((size_t)e * n + i) * n + j) + 1] = cimag(v);
        }
      if (be)
        for (int i = 0; i < n; ++i) {
          be[2 * ((size_t)e * n + i)] = creal(bl[i]);
          be[2 * ((size_t)e * n + i) + 1] = cimag(bl[i]);
        }
    }
    free(Ae);
    free(tmp);
    free(bl);
    free(G);
    free(phi);
  }
  return 0;
}

/* ------------------------------------------------------------- scatter */

static uint64_t lower_bound_u64(const uint64_t *a, uint64_t lo, uint64_t hi, uint64_t v) {
  while (lo < hi) {
    uint64_t mid = lo + (hi - lo) / 2;
    if (a[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

static void atomic_add_c(double *p, cplx v) {
#pragma omp atomic update
  p[0] += creal(v);
#pragma omp atomic update
  p[1] += cimag(v);
}

/* Full assembly: Assembler::_assembleBilinear / _assembleLinear
 * (src/term/Assembler.cpp:157-479) with
 *   MatrixFactory::addValues (src/system/MatrixFactory.cpp:233-448): row =
 *     test DOF, column = unknown DOF, values[i*n + j] = A_e(j, i), position by
 *     std::lower_bound in the CSR row, Fixed columns flag the lifting;
 *   VectorFactory::addValuesDC (src/system/VectorFactory.cpp:178-210):
 *     b[row] += values[j*n + i] * valuesDC[fixed]  (note the transposed read);
 *   VectorFactory::addValues (src/system/VectorFactory.cpp:122-145).
 * values [nnz][2] and rhs [n_rows][2] are accumulated (zero them first). */
int or_assemble(const or_bucket *b, const or_term *terms, int nterms, double freq, const uint64_t *ai, const uint64_t *aj,
                const uint64_t *edof, const int32_t *etype, const double *dirichlet, double *values, double *rhs) {
  const int n = b->nb * b->mult;
  int hasSource = 0;
  for (int t = 0; t < nterms; ++t)
    if (terms[t].kind == TERM_SOURCE || terms[t].kind == TERM_SOURCE_GRAD) hasSource = 1;
  int err = 0;
  or_jacmod_err = 0;
#pragma omp parallel
  {
    cplx *Ae = malloc(sizeof(cplx) * n * n), *tmp = malloc(sizeof(cplx) * n * n), *bl = malloc(sizeof(cplx) * n);
    double *G = malloc(sizeof(double) * 3 * b->nb), *phi = malloc(sizeof(double) * b->nb);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < b->E; ++e) {
      /* _assembleBilinear: bilinear terms only */
      or_element(b, terms, nterms, freq, e, Ae, NULL, tmp, G, phi, 1);
      const uint64_t *idx = edof + (size_t)e * n;
      const int32_t *typ = etype + (size_t)e * n;
      int haveDC = 0;
      for (int i = 0; i < n; ++i) {
        const int ti = typ[i];
        if (ti == AT_FIXED) {
          haveDC = 1;
          continue;
        }
        uint64_t row, col;
        cplx si, sj;
        if (!or_dof_row(b, ti, idx[i], &row, &si)) continue;
        for (int j = 0; j < n; ++j) {
          const int tj = typ[j];
          if (tj == AT_FIXED) {
            haveDC = 1;
            continue;
          }
          if (!or_dof_row(b, tj, idx[j], &col, &sj)) continue;
          if (b->upper && col < row) continue; /* upper triangular matrix (MatrixFactory.cpp:265) */
          const uint64_t pos = lower_bound_u64(aj, ai[row], ai[row + 1], col);
          /* the reference adds at the lower_bound position unchecked (MatrixFactory.cpp:267-268);
           * with upper storage an aliased bubble row can miss columns, which then land on
           * the next column of the row */
          if (pos == ai[row + 1] || (aj[pos] != col && !b->upper)) {
#pragma omp atomic write
            err = 1;
            continue;
          }
          /* linked rows scale by conj(coefficient), linked columns by the coefficient */
          atomic_add_c(values + 2 * pos, conj(si) * sj * Ae[i * n + j]);
        }
      }
      if (haveDC && rhs) {
        /* addValuesDC, transposed read (VectorFactory.cpp:178-210) */
        for (int i = 0; i < n; ++i) {
          uint64_t row;
          cplx si;
          if (!or_dof_row(b, typ[i], idx[i], &row, &si)) continue;
          for (int j = 0; j < n; ++j)
            if (typ[j] == AT_FIXED) {
              cplx uD = dirichlet[2 * idx[j]] + I * dirichlet[2 * idx[j] + 1];
              atomic_add_c(rhs + 2 * row, conj(si) * Ae[j * n + i] * uD);
            }
        }
      }
    }
    if (hasSource && rhs) {
#pragma omp barrier
#pragma omp for schedule(static)
      for (int64_t e = 0; e < b->E; ++e) {
        /* _assembleLinear: linear terms only */
        or_element(b, terms, nterms, freq, e, Ae, bl, tmp, G, phi, 0);
        const uint64_t *idx = edof + (size_t)e * n;
        const int32_t *typ = etype + (size_t)e * n;
        for (int i = 0; i < n; ++i) {
          uint64_t row;
          cplx si;
          /* VectorFactory::addValues (VectorFactory.cpp:122-145) */
          if (or_dof_row(b, typ[i], idx[i], &row, &si)) atomic_add_c(rhs + 2 * row, conj(si) * bl[i]);
        }
      }
    }
    free(Ae);
    free(tmp);
    free(bl);
    free(G);
    free(phi);
  }
  return or_jacmod_err ? 2 : err;
}

/* ------------------------------------------------ two-field terms */

/* Element matrix of a term whose unknown and test fields differ
 * (BilinearTerm::assemblyInitialization with _field[0] != _field[1],
 * src/term/BilinearTerm.cpp:156-273: the rule of the unknown field's space,
 * both fields' basis functions at its points; evaluate, :304-343, with
 * expressionLhs from the unknown field's evaluator and expressionRhs from the
 * test field's). Scalar H1 fields (Form0, one component) on both sides.
 * Ae[i * nU + j] = A_e(j, i): i the test DOF, j the unknown DOF, the
 * column-major layout of the reference's nU x nT A_e. */
static void or_element_coupled(const or_bucket *bt, const or_bucket *bu, const or_term *terms, int nterms, double freq,
                               int64_t e, cplx *Ae, cplx *tmp, double *GT, double *GU) {
  const int nT = bt->nb, nU = bu->nb, nq = bt->nq;
  const int oT = bt->orient ? bt->orient[e] : 0, oU = bu->orient ? bu->orient[e] : 0;
  int frequencyModule = 0;
  for (int t = 0; t < nterms; ++t)
    if (terms[t].dt) frequencyModule = 1;
  for (int k = 0; k < nT * nU; ++k) Ae[k] = 0.0;
  for (int t = 0; t < nterms; ++t) {
    const or_term *T = &terms[t];
    if (T->kind == TERM_SOURCE || T->kind == TERM_SOURCE_GRAD) continue;
    cplx *target = (frequencyModule && T->dt) ? tmp : Ae;
    if (target == tmp)
      for (int k = 0; k < nT * nU; ++k) tmp[k] = 0.0;
    for (int q = 0; q < nq; ++q) {
      double J[9], xq[3];
      double det = or_jacobian(bt, e, q, J, xq);
      if (or_jacmod_apply(&T->jacmod, xq, J, &det)) or_jacmod_err = 1;
      const double wd = bt->w[q] * det;
      const double *phT = bt->bval + ((size_t)oT * nq + q) * nT;
      const double *phU = bu->bval + ((size_t)oU * nq + q) * nU;
      /* field nodes read the unknown field's values (the coefficient's field
       * is evaluated with the unknown's element DOFs) */
      const cplx c = eval_expr(&T->coef, e, xq, phU, nU, q, nq);
      or_form1(J, bt->bgrad + ((size_t)oT * nq + q) * nT * 3, nT, GT);
      or_form1(J, bu->bgrad + ((size_t)oU * nq + q) * nU * 3, nU, GU);
      if (T->kind == TERM_MASS) {
        for (int i = 0; i < nT; ++i)
          for (int j = 0; j < nU; ++j) target[j + i * nU] += wd * (c * phU[j]) * conj(phT[i]);
      } else if (T->kind == TERM_GRAD_GRAD) {
        for (int i = 0; i < nT; ++i)
          for (int j = 0; j < nU; ++j) {
            cplx s = 0.0;
            for (int r = 0; r < 3; ++r) s += (c * GU[r * nU + j]) * conj(GT[r * nT + i]);
            target[j + i * nU] += wd * s;
          }
      } else if (T->kind == TERM_GRAD_GRAD_TENSOR_FULL) {
        cplx D[3][3];
        for (int k = 0; k < 9; ++k) D[k / 3][k % 3] = c * eval_expr(&T->tensor[k], e, xq, phU, nU, q, nq);
        for (int i = 0; i < nT; ++i)
          for (int j = 0; j < nU; ++j) {
            cplx s = 0.0;
            for (int r = 0; r < 3; ++r)
              for (int u = 0; u < 3; ++u) s += D[r][u] * GU[u * nU + j] * GT[r * nT + i];
            target[j + i * nU] += wd * s;
          }
      } else if (T->kind == TERM_VECTOR_GRAD_TEST) {
        cplx bv[3];
        for (int k = 0; k < 3; ++k) bv[k] = c * eval_expr(&T->tensor[k], e, xq, phU, nU, q, nq);
        for (int i = 0; i < nT; ++i)
          for (int j = 0; j < nU; ++j) {
            cplx s = bv[0] * GT[i] + bv[1] * GT[nT + i] + bv[2] * GT[2 * nT + i];
            target[j + i * nU] += wd * s * phU[j];
          }
      } else if (T->kind == TERM_ADVECTION) {
        cplx bv[3];
        for (int k = 0; k < 3; ++k) bv[k] = c * eval_expr(&T->tensor[k], e, xq, phU, nU, q, nq);
        for (int i = 0; i < nT; ++i)
          for (int j = 0; j < nU; ++j) {
            cplx s = bv[0] * GU[j] + bv[1] * GU[nU + j] + bv[2] * GU[2 * nU + j];
            target[j + i * nU] += wd * s * conj(phT[i]);
          }
      }
    }
    if (target == tmp) {
      cplx factor = T->dt == 2 ? -freq * freq : -I * freq;
      for (int k = 0; k < nT * nU; ++k) Ae[k] += factor * tmp[k];
    }
  }
}

/* Assembly of two-field terms into the shared CSR (Assembler::_assembleBilinear,
 * src/term/Assembler.cpp:157-359, with the test field's indices as rows and
 * the unknown field's as columns): MatrixFactory::addValues(nT, nU, test,
 * unknown, values) adds values[i * nU + j] at (row of test DOF i, column of
 * unknown DOF j) (src/system/MatrixFactory.cpp:233-307); for fixed unknown
 * DOFs VectorFactory::addValuesDC(nT, nU, ...) adds values[j * nU + i] *
 * valuesDC (src/system/VectorFactory.cpp:178-210), the transposed entry when
 * nT == nU. With nT != nU that read leaves the nT x nU element matrix, so no
 * value is defined: such a call returns 4 and adds nothing. Scalar H1 fields;
 * Unknown and Fixed DOFs (linked DOFs: returns 5). values [nnz][2] and rhs
 * [n_rows][2] are accumulated. */
int or_assemble_coupled(const or_bucket *bt, const or_bucket *bu, const or_term *terms, int nterms, double freq,
                        const uint64_t *ai, const uint64_t *aj, const uint64_t *edofT, const int32_t *etypeT,
                        const uint64_t *edofU, const int32_t *etypeU, const double *dirichlet, double *values, double *rhs) {
  const int nT = bt->nb, nU = bu->nb;
  if (bt->form != 0 || bu->form != 0 || bt->mult != 1 || bu->mult != 1) return 6;
  for (int64_t k = 0; k < bt->E * nT; ++k)
    if (etypeT[k] == AT_LINKED || etypeT[k] == AT_LINKED_BUBBLE) return 5;
  int anyFixed = 0;
  for (int64_t k = 0; k < bu->E * nU; ++k) {
    if (etypeU[k] == AT_LINKED || etypeU[k] == AT_LINKED_BUBBLE) return 5;
    if (etypeU[k] == AT_FIXED) anyFixed = 1;
  }
  if (anyFixed && rhs && nT != nU) return 4;
  int err = 0;
  or_jacmod_err = 0;
#pragma omp parallel
  {
    cplx *Ae = malloc(sizeof(cplx) * nT * nU), *tmp = malloc(sizeof(cplx) * nT * nU);
    double *GT = malloc(sizeof(double) * 3 * nT), *GU = malloc(sizeof(double) * 3 * nU);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < bt->E; ++e) {
      or_element_coupled(bt, bu, terms, nterms, freq, e, Ae, tmp, GT, GU);
      const uint64_t *it = edofT + (size_t)e * nT, *iu = edofU + (size_t)e * nU;
      const int32_t *tt = etypeT + (size_t)e * nT, *tu = etypeU + (size_t)e * nU;
      int haveDC = 0;
      for (int i = 0; i < nT; ++i) {
        if (tt[i] == AT_FIXED) {
          haveDC = 1;
          continue;
        }
        if (tt[i] != AT_UNKNOWN && tt[i] != AT_UNKNOWN_BUBBLE && tt[i] != AT_UNKNOWN_GLOBAL) continue;
        const uint64_t row = it[i];
        for (int j = 0; j < nU; ++j) {
          if (tu[j] == AT_FIXED) {
            haveDC = 1;
            continue;
          }
          if (tu[j] != AT_UNKNOWN && tu[j] != AT_UNKNOWN_BUBBLE && tu[j] != AT_UNKNOWN_GLOBAL) continue;
          const uint64_t col = iu[j];
          if (bt->upper && col < row) continue;
          const uint64_t pos = lower_bound_u64(aj, ai[row], ai[row + 1], col);
          if (pos == ai[row + 1] || (aj[pos] != col && !bt->upper)) {
#pragma omp atomic write
            err = 1;
            continue;
          }
          atomic_add_c(values + 2 * pos, Ae[i * nU + j]);
        }
      }
      if (haveDC && rhs) {
        for (int i = 0; i < nT; ++i) {
          if (tt[i] != AT_UNKNOWN && tt[i] != AT_UNKNOWN_BUBBLE && tt[i] != AT_UNKNOWN_GLOBAL) continue;
          for (int j = 0; j < nU; ++j)
            if (tu[j] == AT_FIXED) {
              cplx uD = dirichlet[2 * iu[j]] + I * dirichlet[2 * iu[j] + 1];
              atomic_add_c(rhs + 2 * it[i], Ae[j * nU + i] * uD);
            }
        }
      }
    }
    free(Ae);
    free(tmp);
    free(GT);
    free(GU);
  }
  return or_jacmod_err ? 2 : err;
}

/* --------------------------------------------------------------- pattern */

/* MatrixFactory::addPattern (src/system/MatrixFactory.cpp:459-539) for a
 * non-symmetric matrix, element by element in order (the reference builds
 * rows under per-row locks; the resulting sorted sets do not depend on
 * order), then finalizePattern (:188-213). Bubble rows of one element alias
 * the first bubble row's column vector (:505-536).
 * Output: ai [n_rows+1]; aj allocated here (free with or_free). */
typedef struct {
  uint64_t *v;
  uint64_t n, cap;
} u64vec;

static void vec_insert_sorted(u64vec *r, uint64_t x) {
  uint64_t pos = lower_bound_u64(r->v, 0, r->n, x);
  if (pos < r->n && r->v[pos] == x) return;
  if (r->n == r->cap) {
    r->cap = r->cap ? 2 * r->cap : 16;
    r->v = realloc(r->v, r->cap * sizeof(uint64_t));
  }
  memmove(r->v + pos + 1, r->v + pos, (r->n - pos) * sizeof(uint64_t));
  r->v[pos] = x;
  r->n++;
}

int or_pattern(int64_t E, int n, const uint64_t *edof, const int32_t *etype, uint64_t n_rows, uint64_t *ai, uint64_t **aj_out,
               int upper, const uint64_t *linked_row) {
  for (int64_t k = 0; k < E * n; ++k)
    if ((etype[k] == AT_LINKED || etype[k] == AT_LINKED_BUBBLE) && !linked_row) return 3; /* not restated */
  /* rows[v] are the column lists; a row's pattern is the list ptr[r] points at
   * (the reference's array of vector pointers, MatrixFactory _pattern) */
  u64vec *rows = calloc(n_rows, sizeof(u64vec));
  int64_t *ptr = malloc(n_rows * sizeof(int64_t));
  for (uint64_t r = 0; r < n_rows; ++r) ptr[r] = (int64_t)r;
  for (int64_t e = 0; e < E; ++e) {
    const uint64_t *idx = edof + (size_t)e * n;
    const int32_t *typ = etype + (size_t)e * n;
    int64_t bubble = -1;
    for (int i = 0; i < n; ++i) {
      const int ti = typ[i];
      uint64_t Ir, Jc;
      /* a linked row is its master's row (MatrixFactory.cpp:468-470) */
      if (ti == AT_LINKED || ti == AT_LINKED_BUBBLE) Ir = linked_row[idx[i]];
      else if (ti == AT_UNKNOWN || ti == AT_UNKNOWN_GLOBAL || ti == AT_UNKNOWN_BUBBLE) Ir = idx[i];
      else continue;
      /* the element's first bubble row (unknown or linked) takes its columns
       * into the list its row points at; the element's later bubble rows are
       * pointed at that list (MatrixFactory.cpp:505-535). A linked bubble's
       * master row is a bubble row of the master element, so the two
       * elements' bubble rows end up on one list with both their columns. */
      int64_t dst = ptr[Ir];
      if (ti == AT_UNKNOWN_BUBBLE || ti == AT_LINKED_BUBBLE) {
        if (bubble >= 0) {
          ptr[Ir] = bubble;
          continue;
        }
        bubble = dst;
      }
      for (int j = 0; j < n; ++j) {
        const int tj = typ[j];
        if (tj == AT_LINKED || tj == AT_LINKED_BUBBLE) Jc = linked_row[idx[j]];
        else if (tj == AT_UNKNOWN || tj == AT_UNKNOWN_GLOBAL || tj == AT_UNKNOWN_BUBBLE) Jc = idx[j];
        else continue;
        if (upper && Jc < Ir) continue; /* upper triangular matrix (MatrixFactory.cpp:491) */
        vec_insert_sorted(&rows[dst], Jc);
      }
    }
  }
  ai[0] = 0;
  for (uint64_t r = 0; r < n_rows; ++r) ai[r + 1] = ai[r] + rows[ptr[r]].n;
  uint64_t *aj = malloc((ai[n_rows] ? ai[n_rows] : 1) * sizeof(uint64_t));
  for (uint64_t r = 0; r < n_rows; ++r) {
    const u64vec *src = &rows[ptr[r]];
    memcpy(aj + ai[r], src->v, src->n * sizeof(uint64_t));
  }
  for (uint64_t r = 0; r < n_rows; ++r) free(rows[r].v);
  free(rows);
  free(ptr);
  *aj_out = aj;
  return 0;
}

void or_free(void *p) { free(p); }

/* ----------------------------------------------------------- Hilbert */

/* Hilbert<T_dim, T_N> (src/reorder/Hilbert.cpp:17-125 tables, :128-143 key,
 * :174-288 apply): Gray-code state machine, key of the float coordinates
 * scaled into 2^(bits-1) cells (unfused multiply-add, the x86 build's path
 * without FP_FAST_FMAF), then a stable radix sort on the 64-bit key: top 11
 * bits bucketed, then 7 byte passes inside each bucket. */
typedef struct {
  int dim, N;
  uint8_t nextED[24][8];
  uint8_t tiED[24][8];
} or_hilbert_tables;

static void or_hilbert_init(or_hilbert_tables *h, int dim) {
  const int N = 1 << dim;
  const unsigned mask = (~0u) ^ ((~0u) << dim);
  uint8_t gray[8], tgc[8][3][8], inv[8], tinv[8][3][8], ee[8], dd[8], nE[8][3][8], nD[8][3][8];
  h->dim = dim;
  h->N = N;
  for (int i = 0; i < N; ++i) gray[i] = (uint8_t)(i ^ (i >> 1));
  for (int e = 0; e < N; ++e)
    for (int d = 0; d < dim; ++d)
      for (int i = 0; i < N; ++i) {
        unsigned k = (unsigned)(i ^ e);
        tgc[e][d][i] = (uint8_t)((k >> (d + 1)) | ((k << (dim - d - 1)) & mask));
      }
  inv[0] = 0;
  for (int i = 1; i < N; ++i) {
    inv[i] = (uint8_t)i;
    for (int j = 1; j < dim; ++j) inv[i] ^= (uint8_t)(i >> j);
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < dim; ++j)
      for (int k = 0; k < N; ++k) tinv[i][j][k] = inv[tgc[i][j][k]];
  ee[0] = 0;
  for (int i = 1; i < N; ++i) ee[i] = gray[2 * ((i - 1) / 2)];
  dd[0] = 0;
  for (int i = 1; i < N; ++i) {
    if (i < N / 2) dd[i] = (i % 2 == 0) ? gray[i - 1] % dim : gray[i] % dim;
    else dd[i] = dd[N - i - 1];
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < dim; ++j)
      for (int k = 0; k < N; ++k) {
        uint8_t l = ee[tinv[i][j][k]];
        nE[i][j][k] = (uint8_t)(i ^ (((l << (j + 1)) & mask) | (l >> (dim - j - 1))));
        nD[i][j][k] = (uint8_t)((j + dd[tinv[i][j][k]] + 1) % dim);
      }
  memset(h->nextED, 0, sizeof(h->nextED));
  memset(h->tiED, 0, sizeof(h->tiED));
  for (int i = 0; i < N * dim; ++i)
    for (int j = 0; j < N; ++j) {
      int e = i & (int)mask, d = i >> dim;
      if (d >= dim) continue;
      h->nextED[i][j] = (uint8_t)((nD[e][d][j] << dim) | nE[e][d][j]);
      h->tiED[i][j] = tinv[e][d][j];
    }
}

static uint64_t or_hilbert_index(const or_hilbert_tables *h, const uint32_t *el, int begBit) {
  uint64_t key = 0;
  uint8_t ed = 0;
  for (int m = begBit; m >= 0; m--) {
    uint8_t l = 0;
    for (int n = h->dim - 1; n >= 0; n--) l ^= (uint8_t)(((el[n] >> m) & 0x1) << n);
    key <<= h->dim;
    key ^= h->tiED[ed][l];
    ed = h->nextED[ed][l];
  }
  return key;
}

/* keys of n float points (dim 2 or 3) into out_keys */
int or_hilbert_keys(int dim, int64_t n, const float *pts, const float *mn, const float *mx, uint64_t *out_keys) {
  or_hilbert_tables h;
  or_hilbert_init(&h, dim);
  const unsigned nbrBits = (unsigned)floor(64.0 / dim);
  const unsigned twoPow = 1u << (nbrBits - 1);
  float scale[3], scaleMin[3];
  for (int i = 0; i < dim; ++i) {
    scale[i] = twoPow / (mx[i] - mn[i]);
    scaleMin[i] = -mn[i] * scale[i];
  }
  for (int64_t i = 0; i < n; ++i) {
    uint32_t u[3];
    for (int j = 0; j < dim; ++j) {
      volatile float p = pts[i * dim + j] * scale[j];
      u[j] = (uint32_t)(p + scaleMin[j]);
    }
    out_keys[i] = or_hilbert_index(&h, u, (int)nbrBits - 1);
  }
  return 0;
}

/* stable order of the keys: bucket by the top 11 bits, then 7 LSD byte passes
 * (the radix sort of Hilbert::apply with one thread) */
int or_hilbert_sort(int64_t n, const uint64_t *keys, uint32_t *perm) {
  const int nb = 2048, shift = 64 - 11;
  uint64_t *hist = calloc(nb + 1, sizeof(uint64_t));
  uint32_t *a = malloc((n ? n : 1) * sizeof(uint32_t)), *c = malloc((n ? n : 1) * sizeof(uint32_t));
  for (int64_t i = 0; i < n; ++i) hist[(keys[i] >> shift) + 1]++;
  for (int b = 0; b < nb; ++b) hist[b + 1] += hist[b];
  {
    uint64_t *fill = malloc(nb * sizeof(uint64_t));
    memcpy(fill, hist, nb * sizeof(uint64_t));
    for (int64_t i = 0; i < n; ++i) c[fill[keys[i] >> shift]++] = (uint32_t)i;
    free(fill);
  }
  uint64_t local[8 * 256];
  for (int b = 0; b < nb; ++b) {
    const uint64_t off = hist[b], cnt = hist[b + 1] - hist[b];
    if (cnt == 0) continue;
    uint32_t *src = c + off, *dst = a + off;
    memset(local, 0, sizeof(local));
    for (uint64_t j = 0; j < cnt; ++j)
      for (int k = 0; k < 8; ++k) local[((keys[src[j]] >> (k * 8)) & 0xFF) + 256 * k]++;
    uint64_t sum[8] = {0};
    for (int j = 0; j < 256; ++j)
      for (int k = 0; k < 8; ++k) {
        uint64_t t = sum[k] + local[256 * k + j];
        local[256 * k + j] = sum[k];
        sum[k] = t;
      }
    for (int k = 0; k < 7; ++k) {
      for (uint64_t j = 0; j < cnt; ++j) dst[local[((keys[src[j]] >> (k * 8)) & 0xFF) + 256 * k]++] = src[j];
      uint32_t *t = src;
      src = dst;
      dst = t;
    }
    /* after 7 passes the sorted bucket sits in the buffer that started as the
     * destination */
    if (src != a + off) memcpy(a + off, src, cnt * sizeof(uint32_t));
  }
  memcpy(perm, a, n * sizeof(uint32_t));
  free(hist);
  free(a);
  free(c);
  return 0;
}

/* DofsManager::reorderWithHilbert(true) (src/dofs/DofsManager.cpp:118-241):
 * DOFs given in dictionary iteration order (float coords, assemble types);
 * unknown non-bubble DOFs get numDof 1.. in Hilbert order, bubbles last.
 * num_dof is written for unknown DOFs only. */
int or_reorder_hilbert(int dim, const double *bbox, int64_t n, const float *xyz, const int32_t *atype, uint64_t n_unknown,
                       uint64_t n_bubble, uint64_t *num_dof) {
  float mn[3], mx[3];
  for (int c = 0; c < dim; ++c) {
    mn[c] = (float)(bbox[c] - 0.000001 * fabs(bbox[c]));
    mx[c] = (float)(bbox[3 + c] + 0.000001 * fabs(bbox[3 + c]));
  }
  for (int pass = 0; pass < 2; ++pass) {
    const int want = pass == 0 ? AT_UNKNOWN : AT_UNKNOWN_BUBBLE;
    int64_t cnt = 0;
    for (int64_t i = 0; i < n; ++i)
      if (atype[i] == want) ++cnt;
    float *pts = malloc((cnt ? cnt : 1) * dim * sizeof(float));
    int64_t *ids = malloc((cnt ? cnt : 1) * sizeof(int64_t));
    uint64_t *keys = malloc((cnt ? cnt : 1) * sizeof(uint64_t));
    uint32_t *perm = malloc((cnt ? cnt : 1) * sizeof(uint32_t));
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i)
      if (atype[i] == want) {
        for (int c = 0; c < dim; ++c) pts[k * dim + c] = xyz[3 * i + c];
        ids[k++] = i;
      }
    or_hilbert_keys(dim, cnt, pts, mn, mx, keys);
    or_hilbert_sort(cnt, keys, perm);
    for (int64_t r = 0; r < cnt; ++r) num_dof[ids[perm[r]]] = pass == 0 ? (uint64_t)r + 1 : n_unknown - n_bubble + (uint64_t)r + 1;
    free(pts);
    free(ids);
    free(keys);
    free(perm);
  }
  return 0;
}

/* ----------------------------------------------------- robin-hood order */

/* Slot order of robin_hood::unordered_map<Dof*, T> (vendored robin-hood
 * 3.8.0: detail::Table doInsert, insert_move, shiftUp, increase_size,
 * try_increase_info, reserve, iteration) keyed by Dof::hash
 * (src/dofs/Dof.h:87-92). ops: a script of reserve(c) (op_kind 0, arg c) and
 * insert(DOF arg) (op_kind 1) events; order_out receives the DOF ids in
 * iteration order; returns the element count. */
typedef struct {
  uint32_t *keys;
  uint64_t *hashes;
  uint8_t *info;
  size_t mask, num, maxAllowed;
  uint32_t inc, shift;
} or_rh;

static uint64_t rh_rotr(uint64_t x, unsigned r) { return (x >> r) | (x << (64 - r)); }
static uint64_t rh_mix(uint64_t x) {
  uint64_t h1 = x * UINT64_C(0xA24BAED4963EE407);
  uint64_t h2 = rh_rotr(x, 32) * UINT64_C(0x9FB21C651E98DF25);
  return rh_rotr(h1 + h2, 32);
}
static size_t rh_max(size_t n) { return n * 80 / 100; }
static size_t rh_buf(size_t n) { size_t m = rh_max(n); return n + (m < 0xFF ? m : 0xFF); }

static void rh_init(or_rh *t, size_t maxElements) {
  size_t nb = rh_buf(maxElements);
  free(t->keys);
  free(t->hashes);
  free(t->info);
  t->num = 0;
  t->mask = maxElements - 1;
  t->maxAllowed = rh_max(maxElements);
  t->keys = calloc(nb, sizeof(uint32_t));
  t->hashes = calloc(nb, sizeof(uint64_t));
  t->info = calloc(nb + 8, 1);
  t->info[nb] = 1;
  t->inc = 32;
  t->shift = 59;
}

static void rh_shift_up(or_rh *t, size_t start, size_t ins) {
  for (size_t i = start; i != ins; --i) {
    t->keys[i] = t->keys[i - 1];
    t->hashes[i] = t->hashes[i - 1];
  }
  for (size_t i = start; i != ins; --i) {
    t->info[i] = (uint8_t)(t->info[i - 1] + t->inc);
    if (t->info[i] + t->inc > 0xFF) t->maxAllowed = 0;
  }
}

static int rh_try_increase_info(or_rh *t) {
  if (t->inc <= 2) return 0;
  t->inc >>= 1;
  ++t->shift;
  size_t nb = rh_buf(t->mask + 1);
  for (size_t i = 0; i < nb; i += 8)
    for (size_t b = i; b < i + 8; ++b) t->info[b] >>= 1;
  t->info[nb] = 1;
  t->maxAllowed = rh_max(t->mask + 1);
  return 1;
}

static void rh_insert_move(or_rh *t, uint32_t id, uint64_t hash) {
  if (t->maxAllowed == 0) rh_try_increase_info(t);
  uint64_t h = rh_mix(hash);
  uint32_t info = t->inc + (uint32_t)(h >> t->shift);
  size_t idx = (size_t)h & t->mask;
  while (info <= t->info[idx]) {
    ++idx;
    info += t->inc;
  }
  size_t ins = idx;
  uint8_t insInfo = (uint8_t)info;
  if (insInfo + t->inc > 0xFF) t->maxAllowed = 0;
  while (t->info[idx] != 0) {
    ++idx;
    info += t->inc;
  }
  if (idx != ins) rh_shift_up(t, idx, ins);
  t->keys[ins] = id;
  t->hashes[ins] = hash;
  t->info[ins] = insInfo;
  t->num++;
}

static void rh_rehash(or_rh *t, size_t nbk) {
  size_t oldBuf = rh_buf(t->mask + 1);
  uint32_t *ok = t->keys;
  uint64_t *oh = t->hashes;
  uint8_t *oi = t->info;
  int had = ok != NULL;
  t->keys = NULL;
  t->hashes = NULL;
  t->info = NULL;
  rh_init(t, nbk);
  if (had && oldBuf > 1)
    for (size_t i = 0; i < oldBuf; ++i)
      if (oi[i]) rh_insert_move(t, ok[i], oh[i]);
  free(ok);
  free(oh);
  free(oi);
}

static void rh_increase(or_rh *t) {
  if (t->keys == NULL) {
    rh_init(t, 8);
    return;
  }
  if (t->num < rh_max(t->mask + 1) && rh_try_increase_info(t)) return;
  rh_rehash(t, (t->mask + 1) * 2);
}

static uint64_t dof_hash(uint64_t numType, uint64_t entity) {
  uint64_t seed = entity + 0x9e3779b9ull;
  seed ^= numType + 0x9e3779b9ull + (seed << 6) + (seed >> 2);
  return seed;
}

int64_t or_robin_order(int64_t n_ops, const int32_t *op_kind, const uint64_t *op_arg, const uint64_t *num_type,
                       const uint64_t *entity, uint32_t *order_out) {
  or_rh t;
  memset(&t, 0, sizeof(t));
  static uint8_t dummy[8];
  (void)dummy;
  for (int64_t k = 0; k < n_ops; ++k) {
    if (op_kind[k] == 0) {
      size_t c = op_arg[k] > t.num ? op_arg[k] : t.num, ns = 8;
      while (rh_max(ns) < c) ns *= 2;
      rh_rehash(&t, ns);
      continue;
    }
    const uint32_t id = (uint32_t)op_arg[k];
    const uint64_t hsh = dof_hash(num_type[id], entity[id]);
    for (;;) {
      if (t.keys == NULL) {
        rh_increase(&t);
        continue;
      }
      uint64_t h = rh_mix(hsh);
      uint32_t info = t.inc + (uint32_t)(h >> t.shift);
      size_t idx = (size_t)h & t.mask;
      while (info < t.info[idx]) {
        ++idx;
        info += t.inc;
      }
      int found = 0;
      while (info == t.info[idx]) {
        uint32_t o = t.keys[idx];
        if (num_type[o] == num_type[id] && entity[o] == entity[id]) {
          found = 1;
          break;
        }
        ++idx;
        info += t.inc;
      }
      if (found) break;
      if (t.num >= t.maxAllowed) {
        rh_increase(&t);
        continue;
      }
      size_t ins = idx;
      uint32_t insInfo = info;
      if (insInfo + t.inc > 0xFF) t.maxAllowed = 0;
      while (t.info[idx] != 0) {
        ++idx;
        info += t.inc;
      }
      if (idx != ins) rh_shift_up(&t, idx, ins);
      t.keys[ins] = id;
      t.hashes[ins] = hsh;
      t.info[ins] = (uint8_t)insInfo;
      t.num++;
      break;
    }
  }
  int64_t cnt = 0;
  if (t.keys) {
    size_t nb = rh_buf(t.mask + 1);
    for (size_t i = 0; i < nb; ++i)
      if (t.info[i]) order_out[cnt++] = t.keys[i];
  }
  free(t.keys);
  free(t.hashes);
  free(t.info);
  return cnt;
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
