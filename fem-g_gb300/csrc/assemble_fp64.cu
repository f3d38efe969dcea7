// Plain FP64 / complex<double> assembly.
//
// K1-K3 + K5 (element kernel, one warp per element): for each quadrature
// point the warp forms the Jacobian, its inverse and determinant (gmsh
// getJacobians, src/term/Assembler.cpp:131-139), evaluates the coefficient
// programs at the physical point (EquationEvaluator::initialize,
// src/term/evaluator/EquationEvaluator.h:155-168), maps the reference
// gradients with J^-T (FieldEvaluator<Form1>, src/term/evaluator/FieldEvaluator.h:67-70)
// and accumulates Ke += w det (c L)^T conj(R) (BilinearTerm::evaluate,
// src/term/BilinearTerm.cpp:314-326) with the AFrequency factors
// (src/term/Assembler.cpp:283-295), and b_e += w det conj(phi) f
// (LinearTerm::evaluate, src/term/LinearTerm.cpp:182-191). The tensor
// grad-grad term (a TensorFunction times grad(dof), the left-order evaluator
// src/term/evaluator/EquationEvaluator.h:134-173 with a degree-2 function)
// maps the unknown's gradients by w det c D before the product; D is
// symmetric here. Ke is symmetric for these terms, so each lane owns
// upper-triangle entries.
//
// The element matrices and vectors then go through the deterministic CSR
// reduction of gather.cu.
#include "common.cuh"

namespace femg {

constexpr int kWarpsPerBlockElem = 4;

struct ElemWarpSmem {
  double X[kMaxNodes * 3];
  double J0[9], J[9], Jinv[9];
  double det0, det;
  double2 a, b, s;  // w det c_gradgrad, w det c_mass, w det f
  double2 Aw[6];    // w det times the diffusion tensor (tensor grad-grad term)
  double G[3][kMaxDofs];
  double phi[kMaxDofs];
  double Gs[2][3][kMaxDofs];
  double phis[2][kMaxDofs];
};

template <int MAXENT, bool CPLX>
__global__ void __launch_bounds__(32 * kWarpsPerBlockElem)
    k_element_fp64(const PlanDev p, const DevTerms *__restrict__ terms, double *__restrict__ ke, double2 *__restrict__ be) {
  __shared__ ElemWarpSmem smem[kWarpsPerBlockElem];
  __shared__ uint8_t pairI[kMaxDofs * (kMaxDofs + 1) / 2], pairJ[kMaxDofs * (kMaxDofs + 1) / 2];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int n = p.nb;  // scalar field here: n == nb
  const int nEnt = n * (n + 1) / 2;
  for (int k = threadIdx.x; k < nEnt; k += blockDim.x) {
    // k -> (i, j), i <= j, row-major over the upper triangle
    int i = 0, rem = k;
    while (rem >= n - i) {
      rem -= n - i;
      ++i;
    }
    pairI[k] = (uint8_t)i;
    pairJ[k] = (uint8_t)(i + rem);
  }
  __syncthreads();
  ElemWarpSmem &S = smem[warp];
  const int64_t stride = (int64_t)gridDim.x * kWarpsPerBlockElem;
  for (int64_t e = (int64_t)blockIdx.x * kWarpsPerBlockElem + warp; e < p.E; e += stride) {
    const int o = p.orient ? p.orient[e] : 0;
    for (int t = lane; t < p.nn * 3; t += 32) S.X[t] = p.xyz[3 * (int64_t)p.enodes[e * p.nn + t / 3] + t % 3];
    __syncwarp();
    double accR[MAXENT], accI[MAXENT];
#pragma unroll
    for (int m = 0; m < MAXENT; ++m) {
      accR[m] = 0.0;
      accI[m] = 0.0;
    }
    double2 bacc[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    // one pass over the points per group of terms sharing a Jacobian modificator
    const int nG = terms->nMod > 1 ? terms->nMod : 1;
    for (int gq = 0; gq < nG * p.nq; ++gq) {
      const int g = gq / p.nq, q = gq - g * p.nq;
      if (lane == 0) {
        double xq[3];
        pointGeometry(p, terms, g, q, S.X, S.J0, S.det0, S.J, S.det, S.Jinv, xq);
        double2 cgg = make_double2(0.0, 0.0), cm = make_double2(0.0, 0.0), f = make_double2(0.0, 0.0);
        const double *phq = p.bval + ((size_t)o * p.nq + q) * p.nb;  // for field-node coefficients
        for (int t = 0; t < terms->n; ++t) {
          const DevTerm &T = terms->t[t];
          if (T.mod != g) continue;
          const double2 v = evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq);
          if (T.kind == FG_TERM_GRAD_GRAD) cgg = cadd(cgg, cmul(T.factor, v));
          else if (T.kind == FG_TERM_MASS) cm = cadd(cm, cmul(T.factor, v));
          else if (T.kind == FG_TERM_SOURCE) f = cadd(f, v);
        }
        const double wd = p.w[q] * S.det;
        S.a = make_double2(wd * cgg.x, wd * cgg.y);
        S.b = make_double2(wd * cm.x, wd * cm.y);
        S.s = make_double2(wd * f.x, wd * f.y);
        if (terms->tensorTerm >= 0) {
          double2 A[6];
          diffusionTensor(terms, g, e, xq, cgg, A, phq, p.nb, q, p.nq);
          for (int k = 0; k < 6; ++k) S.Aw[k] = make_double2(wd * A[k].x, wd * A[k].y);
        }
      }
      __syncwarp();
      const size_t base = ((size_t)o * p.nq + q) * p.nb;
      const bool tensor = terms->tensorTerm >= 0;
      for (int i = lane; i < n; i += 32) {
        const double g0 = p.bgrad[3 * (base + i)], g1 = p.bgrad[3 * (base + i) + 1], g2 = p.bgrad[3 * (base + i) + 2];
        const double ph = p.bval[base + i];
        double G[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          G[r] = S.Jinv[r] * g0 + S.Jinv[3 + r] * g1 + S.Jinv[6 + r] * g2;
          S.G[r][i] = G[r];
        }
        if (tensor) {
          // (w det A) G with A symmetric: rows (00 01 02), (01 11 12), (02 12 22)
          const int row[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            S.Gs[0][r][i] = S.Aw[row[r][0]].x * G[0] + S.Aw[row[r][1]].x * G[1] + S.Aw[row[r][2]].x * G[2];
            if (CPLX) S.Gs[1][r][i] = S.Aw[row[r][0]].y * G[0] + S.Aw[row[r][1]].y * G[1] + S.Aw[row[r][2]].y * G[2];
          }
        } else {
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            S.Gs[0][r][i] = S.a.x * G[r];
            if (CPLX) S.Gs[1][r][i] = S.a.y * G[r];
          }
        }
        S.phi[i] = ph;
        S.phis[0][i] = S.b.x * ph;
        if (CPLX) S.phis[1][i] = S.b.y * ph;
        // b_e[i] += w det conj(phi_i) f
        const int slot = i >> 5;
        bacc[slot].x += S.s.x * ph;
        bacc[slot].y += S.s.y * ph;
      }
      __syncwarp();
#pragma unroll
      for (int m = 0; m < MAXENT; ++m) {
        const int k = lane + 32 * m;
        if (k < nEnt) {
          const int i = pairI[k], j = pairJ[k];
          accR[m] += S.G[0][i] * S.Gs[0][0][j] + S.G[1][i] * S.Gs[0][1][j] + S.G[2][i] * S.Gs[0][2][j] + S.phi[i] * S.phis[0][j];
          if (CPLX)
            accI[m] += S.G[0][i] * S.Gs[1][0][j] + S.G[1][i] * S.Gs[1][1][j] + S.G[2][i] * S.Gs[1][2][j] + S.phi[i] * S.phis[1][j];
        }
      }
      __syncwarp();
    }
    // Ke layout [E][ncomp][n][n], row = local test index, column = local unknown index
    const int ncomp = CPLX ? 2 : 1;
    double *K = ke + (size_t)e * ncomp * n * n;
#pragma unroll
    for (int m = 0; m < MAXENT; ++m) {
      const int k = lane + 32 * m;
      if (k < nEnt) {
        const int i = pairI[k], j = pairJ[k];
        K[i * n + j] = accR[m];
        K[j * n + i] = accR[m];
        if (CPLX) {
          K[n * n + i * n + j] = accI[m];
          K[n * n + j * n + i] = accI[m];
        }
      }
    }
    if (be)
      for (int i = lane; i < n; i += 32) be[(size_t)e * n + i] = bacc[i >> 5];
    __syncwarp();
  }
}

// Scalar H1 field with terms whose element matrix is not symmetric: a general
// TensorFunction D in integral(c D grad(dof u), grad(tf u)) and the advection
// integral(c b . grad(dof u), tf(u)) with a VectorFunction b, beside the
// symmetric terms. One warp per element; at each point lane 0 forms
//   M = w det (c_gg I + A_sym + c_full D)   (the unknown's gradient map),
//   v = w det c_adv b,  m = w det c_mass,
// the lanes map the unknown's gradients (U_j = M G_j, a_j = v . G_j + m phi_j)
// and each lane owns entries (i, j) of the full n x n matrix:
//   Ke[i][j] += G_i . U_j + phi_i a_j
// (BilinearTerm::evaluate's Hermitian product with real test functions,
// src/term/BilinearTerm.cpp:314-326: the test side is conj(field), the
// unknown side carries the coefficient).
struct FullWarpSmem {
  double X[kMaxNodes * 3];
  double J0[9], J[9], Jinv[9];
  double det0, det;
  double2 M[9], v[3], m, s;
  double2 vb[3], sg[3];      // w det c b (vector times dof, tested against gradients), w det f (vector source)
  double G[3][kMaxDofs];     // test functions: physical gradients
  double phi[kMaxDofs];      // and values
  double U[2][3][kMaxDofs];  // unknown functions: M G_j (real, imaginary parts)
  double a[2][kMaxDofs];     // and v . G_j + m phi_j
};

// Full (non-symmetric) element matrices: Ke[i][j] = sum_q G_i . (M G_j) +
// phi_i (v . G_j + m phi_j) with the test function i (rows) and the unknown
// function j (columns), M the scaled diffusion tensor (isotropic, symmetric
// and general parts), v the advection vector, m the mass coefficient. A
// two-field plan takes the test functions from the test field's tables and
// the unknown functions from the unknown field's (BilinearTerm with
// _field[0] != _field[1], src/term/BilinearTerm.cpp:304-343): Ke is n x nc.
template <int MAXENT, bool CPLX>
__global__ void __launch_bounds__(32 * kWarpsPerBlockElem)
    k_element_full_fp64(const PlanDev p, const DevTerms *__restrict__ terms, double *__restrict__ ke, double2 *__restrict__ be) {
  __shared__ FullWarpSmem smem[kWarpsPerBlockElem];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int n = p.nb, nU = p.nbU;
  const int nEnt = n * nU;
  FullWarpSmem &S = smem[warp];
  const int64_t stride = (int64_t)gridDim.x * kWarpsPerBlockElem;
  for (int64_t e = (int64_t)blockIdx.x * kWarpsPerBlockElem + warp; e < p.E; e += stride) {
    const int o = p.orient ? p.orient[e] : 0;
    const int oU = p.orientU ? p.orientU[e] : 0;
    for (int t = lane; t < p.nn * 3; t += 32) S.X[t] = p.xyz[3 * (int64_t)p.enodes[e * p.nn + t / 3] + t % 3];
    __syncwarp();
    double accR[MAXENT], accI[MAXENT];
#pragma unroll
    for (int k = 0; k < MAXENT; ++k) {
      accR[k] = 0.0;
      accI[k] = 0.0;
    }
    double2 bacc[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    const int nG = terms->nMod > 1 ? terms->nMod : 1;
    for (int gq = 0; gq < nG * p.nq; ++gq) {
      const int g = gq / p.nq, q = gq - g * p.nq;
      if (lane == 0) {
        double xq[3];
        pointGeometry(p, terms, g, q, S.X, S.J0, S.det0, S.J, S.det, S.Jinv, xq);
        const double *phq = p.bval + ((size_t)o * p.nq + q) * p.nb;
        double2 cgg = make_double2(0.0, 0.0), cm = make_double2(0.0, 0.0), f = make_double2(0.0, 0.0);
        for (int t = 0; t < terms->n; ++t) {
          const DevTerm &T = terms->t[t];
          if (T.mod != g) continue;
          if (T.kind == FG_TERM_GRAD_GRAD) cgg = cadd(cgg, cmul(T.factor, evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq)));
          else if (T.kind == FG_TERM_MASS) cm = cadd(cm, cmul(T.factor, evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq)));
          else if (T.kind == FG_TERM_SOURCE) f = cadd(f, evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq));
        }
        const double wd = p.w[q] * S.det;
        double2 A6[6];
        diffusionTensor(terms, g, e, xq, cgg, A6, phq, p.nb, q, p.nq);  // c_gg I (+ the symmetric tensor term)
        const int sym[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
        double2 M[9];
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) M[3 * r + c] = A6[sym[r][c]];
        if (terms->tensorFullTerm >= 0 && terms->t[terms->tensorFullTerm].mod == g) {
          const DevTerm &T = terms->t[terms->tensorFullTerm];
          const double2 fc = cmul(T.factor, evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq));
          for (int k = 0; k < 9; ++k) M[k] = cadd(M[k], cmul(fc, evalExpr(terms->tensorFull[k], e, xq, phq, p.nb, q, p.nq)));
        }
        double2 v[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
        if (terms->advectTerm >= 0 && terms->t[terms->advectTerm].mod == g) {
          const DevTerm &T = terms->t[terms->advectTerm];
          const double2 fc = cmul(T.factor, evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq));
          for (int k = 0; k < 3; ++k) v[k] = cmul(fc, evalExpr(terms->advect[k], e, xq, phq, p.nb, q, p.nq));
        }
        double2 vb[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
        if (terms->vecGradTerm >= 0 && terms->t[terms->vecGradTerm].mod == g) {
          const DevTerm &T = terms->t[terms->vecGradTerm];
          const double2 fc = cmul(T.factor, evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq));
          for (int k = 0; k < 3; ++k) vb[k] = cmul(fc, evalExpr(terms->vecGrad[k], e, xq, phq, p.nb, q, p.nq));
        }
        double2 sg[3] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
        if (terms->srcGradTerm >= 0 && terms->t[terms->srcGradTerm].mod == g) {
          const DevTerm &T = terms->t[terms->srcGradTerm];
          const double2 fc = evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq);
          for (int k = 0; k < 3; ++k) sg[k] = cmul(fc, evalExpr(terms->srcGrad[k], e, xq, phq, p.nb, q, p.nq));
        }
        for (int k = 0; k < 9; ++k) S.M[k] = make_double2(wd * M[k].x, wd * M[k].y);
        for (int k = 0; k < 3; ++k) S.v[k] = make_double2(wd * v[k].x, wd * v[k].y);
        for (int k = 0; k < 3; ++k) S.vb[k] = make_double2(wd * vb[k].x, wd * vb[k].y);
        for (int k = 0; k < 3; ++k) S.sg[k] = make_double2(wd * sg[k].x, wd * sg[k].y);
        S.m = make_double2(wd * cm.x, wd * cm.y);
        S.s = make_double2(wd * f.x, wd * f.y);
      }
      __syncwarp();
      const size_t base = ((size_t)o * p.nq + q) * p.nb;
      for (int i = lane; i < n; i += 32) {
        const double g0 = p.bgrad[3 * (base + i)], g1 = p.bgrad[3 * (base + i) + 1], g2 = p.bgrad[3 * (base + i) + 2];
        const double ph = p.bval[base + i];
#pragma unroll
        for (int r = 0; r < 3; ++r) S.G[r][i] = S.Jinv[r] * g0 + S.Jinv[3 + r] * g1 + S.Jinv[6 + r] * g2;
        S.phi[i] = ph;
        const int slot = i >> 5;
        bacc[slot].x += S.s.x * ph + S.sg[0].x * S.G[0][i] + S.sg[1].x * S.G[1][i] + S.sg[2].x * S.G[2][i];
        bacc[slot].y += S.s.y * ph + S.sg[0].y * S.G[0][i] + S.sg[1].y * S.G[1][i] + S.sg[2].y * S.G[2][i];
      }
      const size_t baseU = ((size_t)oU * p.nq + q) * nU;
      for (int j = lane; j < nU; j += 32) {
        const double g0 = p.bgradU[3 * (baseU + j)], g1 = p.bgradU[3 * (baseU + j) + 1], g2 = p.bgradU[3 * (baseU + j) + 2];
        const double ph = p.bvalU[baseU + j];
        double G[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) G[r] = S.Jinv[r] * g0 + S.Jinv[3 + r] * g1 + S.Jinv[6 + r] * g2;
        // U_j = M G_j + vb phi_j: the unknown's vector field, tested against G_i
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          S.U[0][r][j] = S.M[3 * r].x * G[0] + S.M[3 * r + 1].x * G[1] + S.M[3 * r + 2].x * G[2] + S.vb[r].x * ph;
          if (CPLX) S.U[1][r][j] = S.M[3 * r].y * G[0] + S.M[3 * r + 1].y * G[1] + S.M[3 * r + 2].y * G[2] + S.vb[r].y * ph;
        }
        S.a[0][j] = S.v[0].x * G[0] + S.v[1].x * G[1] + S.v[2].x * G[2] + S.m.x * ph;
        if (CPLX) S.a[1][j] = S.v[0].y * G[0] + S.v[1].y * G[1] + S.v[2].y * G[2] + S.m.y * ph;
      }
      __syncwarp();
#pragma unroll
      for (int m = 0; m < MAXENT; ++m) {
        const int k = lane + 32 * m;
        if (k < nEnt) {
          const int i = k / nU, j = k - i * nU;
          accR[m] += S.G[0][i] * S.U[0][0][j] + S.G[1][i] * S.U[0][1][j] + S.G[2][i] * S.U[0][2][j] + S.phi[i] * S.a[0][j];
          if (CPLX)
            accI[m] += S.G[0][i] * S.U[1][0][j] + S.G[1][i] * S.U[1][1][j] + S.G[2][i] * S.U[1][2][j] + S.phi[i] * S.a[1][j];
        }
      }
      __syncwarp();
    }
    const int ncomp = CPLX ? 2 : 1;
    double *K = ke + (size_t)e * ncomp * nEnt;
#pragma unroll
    for (int m = 0; m < MAXENT; ++m) {
      const int k = lane + 32 * m;
      if (k < nEnt) {
        K[k] = accR[m];
        if (CPLX) K[nEnt + k] = accI[m];
      }
    }
    if (be)
      for (int i = lane; i < n; i += 32) be[(size_t)e * n + i] = bacc[i >> 5];
    __syncwarp();
  }
}

// Compound (3-component) field with the isotropic Tensor4 term
// integral(C * grad(dof(u)), grad(tf(u))) and the mass term: the Tensor4
// evaluator of the reference (src/term/evaluator/EquationEvaluator.h:1267-1276,
// CompoundFieldEvaluator<Form1,3> src/term/evaluator/FieldEvaluator.h:171-182)
// with C_ijkl = lambda d_ij d_kl + mu (d_ik d_jl + d_il d_jk) gives, for the
// test DOF (i, a) and the unknown DOF (j, b) (local index = basis * 3 + component),
//   Ke = w det [ lambda dj_b di_a + mu d_ab (gi . gj) + mu dj_a di_b ] + w det c_m d_ab phi_i phi_j
// with g = J^-T grad phi. Lanes own scalar basis pairs (i <= j) and their 3x3
// blocks; the element matrix is symmetric.
struct ElasticWarpSmem {
  double X[kMaxNodes * 3];
  double J0[9], J[9], Jinv[9];
  double det0, det;
  double2 lam, mu, cm, s;  // scaled by w det
  double G[3][kMaxDofs / 3 + 1];
  double phi[kMaxDofs / 3 + 1];
};

template <int MAXP, bool CPLX>
__global__ void __launch_bounds__(32 * kWarpsPerBlockElem)
    k_element_elastic_fp64(const PlanDev p, const DevTerms *__restrict__ terms, double *__restrict__ ke, double2 *__restrict__ be) {
  __shared__ ElasticWarpSmem smem[kWarpsPerBlockElem];
  __shared__ uint8_t pairI[256], pairJ[256];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int ns = p.nb, n = 3 * ns;
  const int nPairs = ns * (ns + 1) / 2;
  for (int k = threadIdx.x; k < nPairs; k += blockDim.x) {
    int i = 0, rem = k;
    while (rem >= ns - i) {
      rem -= ns - i;
      ++i;
    }
    pairI[k] = (uint8_t)i;
    pairJ[k] = (uint8_t)(i + rem);
  }
  __syncthreads();
  ElasticWarpSmem &S = smem[warp];
  const int64_t stride = (int64_t)gridDim.x * kWarpsPerBlockElem;
  for (int64_t e = (int64_t)blockIdx.x * kWarpsPerBlockElem + warp; e < p.E; e += stride) {
    const int o = p.orient ? p.orient[e] : 0;
    for (int t = lane; t < p.nn * 3; t += 32) S.X[t] = p.xyz[3 * (int64_t)p.enodes[e * p.nn + t / 3] + t % 3];
    __syncwarp();
    double accR[MAXP][9], accI[MAXP][9];
#pragma unroll
    for (int m = 0; m < MAXP; ++m)
#pragma unroll
      for (int b = 0; b < 9; ++b) {
        accR[m][b] = 0.0;
        accI[m][b] = 0.0;
      }
    const int nG = terms->nMod > 1 ? terms->nMod : 1;
    for (int gq = 0; gq < nG * p.nq; ++gq) {
      const int g = gq / p.nq, q = gq - g * p.nq;
      if (lane == 0) {
        double xq[3];
        pointGeometry(p, terms, g, q, S.X, S.J0, S.det0, S.J, S.det, S.Jinv, xq);
        double2 lam = make_double2(0.0, 0.0), mu = make_double2(0.0, 0.0), cm = make_double2(0.0, 0.0);
        const double *phq = p.bval + ((size_t)o * p.nq + q) * p.nb;  // scalar basis values (field nodes)
        for (int t = 0; t < terms->n; ++t) {
          const DevTerm &T = terms->t[t];
          if (T.mod != g) continue;
          if (T.kind == FG_TERM_ELASTIC) {
            lam = cadd(lam, cmul(T.factor, evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq)));
            mu = cadd(mu, cmul(T.factor, evalExpr(T.coef2, e, xq, phq, p.nb, q, p.nq)));
          } else if (T.kind == FG_TERM_MASS) {
            cm = cadd(cm, cmul(T.factor, evalExpr(T.coef, e, xq, phq, p.nb, q, p.nq)));
          }
        }
        const double wd = p.w[q] * S.det;
        S.lam = make_double2(wd * lam.x, wd * lam.y);
        S.mu = make_double2(wd * mu.x, wd * mu.y);
        S.cm = make_double2(wd * cm.x, wd * cm.y);
      }
      __syncwarp();
      const size_t base = ((size_t)o * p.nq + q) * p.nb;
      for (int i = lane; i < ns; i += 32) {
        const double g0 = p.bgrad[3 * (base + i)], g1 = p.bgrad[3 * (base + i) + 1], g2 = p.bgrad[3 * (base + i) + 2];
#pragma unroll
        for (int r = 0; r < 3; ++r) S.G[r][i] = S.Jinv[r] * g0 + S.Jinv[3 + r] * g1 + S.Jinv[6 + r] * g2;
        S.phi[i] = p.bval[base + i];
      }
      __syncwarp();
#pragma unroll
      for (int m = 0; m < MAXP; ++m) {
        const int k = lane + 32 * m;
        if (k < nPairs) {
          const int i = pairI[k], j = pairJ[k];
          const double gi[3] = {S.G[0][i], S.G[1][i], S.G[2][i]};
          const double gj[3] = {S.G[0][j], S.G[1][j], S.G[2][j]};
          const double dot = gi[0] * gj[0] + gi[1] * gj[1] + gi[2] * gj[2];
          const double pp = S.phi[i] * S.phi[j];
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
              const double tl = gj[b] * gi[a];
              const double tm = gj[a] * gi[b] + (a == b ? dot : 0.0);
              const double tc = a == b ? pp : 0.0;
              accR[m][3 * a + b] += S.lam.x * tl + S.mu.x * tm + S.cm.x * tc;
              if (CPLX) accI[m][3 * a + b] += S.lam.y * tl + S.mu.y * tm + S.cm.y * tc;
            }
        }
      }
      __syncwarp();
    }
    const int ncomp = CPLX ? 2 : 1;
    double *K = ke + (size_t)e * ncomp * n * n;
#pragma unroll
    for (int m = 0; m < MAXP; ++m) {
      const int k = lane + 32 * m;
      if (k < nPairs) {
        const int i = pairI[k], j = pairJ[k];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            const int ii = 3 * i + a, jj = 3 * j + b;  // test (i, a), unknown (j, b)
            K[ii * n + jj] = accR[m][3 * a + b];
            K[jj * n + ii] = accR[m][3 * a + b];
            if (CPLX) {
              K[n * n + ii * n + jj] = accI[m][3 * a + b];
              K[n * n + jj * n + ii] = accI[m][3 * a + b];
            }
          }
      }
    }
    if (be)
      for (int i = lane; i < n; i += 32) be[(size_t)e * n + i] = make_double2(0.0, 0.0);
    __syncwarp();
  }
}

// Lowest-order-and-up HCurl field (FG_FORM_1): with the Form1 values
// P = J^-T v and the Form2 curls C = J c / det (FieldEvaluator<Form1/Form2>,
// src/term/evaluator/FieldEvaluator.h:59-105),
//   Ke[i][j] = sum_q w det (c_curl C_j . C_i + c_m P_j . P_i),
// or, with tensor terms (TensorFunction * curl, TensorFunction * dof: the
// Maxwell PML), sum_q w det (C_i . A C_j + P_i . B P_j) with A = c_curl I + c D.
// Warp per element, lanes over the pairs i <= j (the matrix is symmetric),
// 256 pairs at a time: the points are visited once per 256 pairs.
struct HcurlWarpSmem {
  double X[kMaxNodes * 3];
  double J0[9], J[9], Jinv[9];
  double det0, det;
  double2 a, b;  // w det c_curl, w det c_m
  double2 Aw[6], Bw[6];  // w det times the curl and mass coefficient tensors (tensor terms)
  double C[3][kMaxDofs], P[3][kMaxDofs];
  double Cs[2][3][kMaxDofs], Ps[2][3][kMaxDofs];  // tensor terms: (w det A) C, (w det B) P (real, imaginary)
};

template <int MAXENT, bool CPLX>
__global__ void __launch_bounds__(32 * kWarpsPerBlockElem)
    k_element_hcurl_fp64(const PlanDev p, const DevTerms *__restrict__ terms, double *__restrict__ ke) {
  __shared__ HcurlWarpSmem smem[kWarpsPerBlockElem];
  __shared__ uint8_t pairI[kMaxDofs * (kMaxDofs + 1) / 2], pairJ[kMaxDofs * (kMaxDofs + 1) / 2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = p.nb;
  const int nEnt = n * (n + 1) / 2;
  for (int k = threadIdx.x; k < nEnt; k += blockDim.x) {
    int i = 0, rem = k;
    while (rem >= n - i) {
      rem -= n - i;
      ++i;
    }
    pairI[k] = (uint8_t)i;
    pairJ[k] = (uint8_t)(i + rem);
  }
  __syncthreads();
  HcurlWarpSmem &S = smem[warp];
  const bool tensor = terms->tensorTerm >= 0 || terms->tensorMassTerm >= 0;
  const int64_t stride = (int64_t)gridDim.x * kWarpsPerBlockElem;
  for (int64_t e = (int64_t)blockIdx.x * kWarpsPerBlockElem + warp; e < p.E; e += stride) {
    const int o = p.orient ? p.orient[e] : 0;
    for (int t = lane; t < p.nn * 3; t += 32) S.X[t] = p.xyz[3 * (int64_t)p.enodes[e * p.nn + t / 3] + t % 3];
    __syncwarp();
    // the pairs in chunks of 32 MAXENT, the points once per chunk
    for (int c0 = 0; c0 < nEnt; c0 += 32 * MAXENT) {
    double accR[MAXENT], accI[MAXENT];
#pragma unroll
    for (int m = 0; m < MAXENT; ++m) accR[m] = accI[m] = 0.0;
    const int nG = terms->nMod > 1 ? terms->nMod : 1;
    for (int gq = 0; gq < nG * p.nq; ++gq) {
      const int g = gq / p.nq, q = gq - g * p.nq;
      if (lane == 0) {
        double xq[3];
        pointGeometry(p, terms, g, q, S.X, S.J0, S.det0, S.J, S.det, S.Jinv, xq);
        double2 cc = make_double2(0.0, 0.0), cm = make_double2(0.0, 0.0);
        for (int t = 0; t < terms->n; ++t) {
          const DevTerm &T = terms->t[t];
          if (T.mod != g) continue;
          const double2 v = evalExpr(T.coef, e, xq, nullptr, 0, q, p.nq);
          if (T.kind == FG_TERM_GRAD_GRAD) cc = cadd(cc, cmul(T.factor, v));
          else if (T.kind == FG_TERM_MASS) cm = cadd(cm, cmul(T.factor, v));
        }
        const double wd = p.w[q] * S.det;
        S.a = make_double2(wd * cc.x, wd * cc.y);
        S.b = make_double2(wd * cm.x, wd * cm.y);
        if (tensor) {
          double2 A[6], B[6];
          coefTensor(terms, terms->tensorTerm, terms->tensor, g, e, xq, cc, A, nullptr, 0, q, p.nq);
          coefTensor(terms, terms->tensorMassTerm, terms->tensorMass, g, e, xq, cm, B, nullptr, 0, q, p.nq);
          for (int k = 0; k < 6; ++k) {
            S.Aw[k] = make_double2(wd * A[k].x, wd * A[k].y);
            S.Bw[k] = make_double2(wd * B[k].x, wd * B[k].y);
          }
        }
      }
      __syncwarp();
      const size_t base = ((size_t)o * p.nq + q) * p.nb;
      for (int i = lane; i < n; i += 32) {
        const double *cr = p.bgrad + 3 * (base + i), *vr = p.bval + 3 * (base + i);
        double Ci[3], Pi[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          Ci[r] = (S.J[r] * cr[0] + S.J[3 + r] * cr[1] + S.J[6 + r] * cr[2]) / S.det;
          Pi[r] = S.Jinv[r] * vr[0] + S.Jinv[3 + r] * vr[1] + S.Jinv[6 + r] * vr[2];
          S.C[r][i] = Ci[r];
          S.P[r][i] = Pi[r];
        }
        if (tensor) {
          const int row[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            S.Cs[0][r][i] = S.Aw[row[r][0]].x * Ci[0] + S.Aw[row[r][1]].x * Ci[1] + S.Aw[row[r][2]].x * Ci[2];
            S.Ps[0][r][i] = S.Bw[row[r][0]].x * Pi[0] + S.Bw[row[r][1]].x * Pi[1] + S.Bw[row[r][2]].x * Pi[2];
            if (CPLX) {
              S.Cs[1][r][i] = S.Aw[row[r][0]].y * Ci[0] + S.Aw[row[r][1]].y * Ci[1] + S.Aw[row[r][2]].y * Ci[2];
              S.Ps[1][r][i] = S.Bw[row[r][0]].y * Pi[0] + S.Bw[row[r][1]].y * Pi[1] + S.Bw[row[r][2]].y * Pi[2];
            }
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int m = 0; m < MAXENT; ++m) {
        const int k = c0 + lane + 32 * m;
        if (k < nEnt) {
          const int i = pairI[k], j = pairJ[k];
          if (tensor) {
            accR[m] += S.C[0][i] * S.Cs[0][0][j] + S.C[1][i] * S.Cs[0][1][j] + S.C[2][i] * S.Cs[0][2][j] +
                       S.P[0][i] * S.Ps[0][0][j] + S.P[1][i] * S.Ps[0][1][j] + S.P[2][i] * S.Ps[0][2][j];
            if (CPLX)
              accI[m] += S.C[0][i] * S.Cs[1][0][j] + S.C[1][i] * S.Cs[1][1][j] + S.C[2][i] * S.Cs[1][2][j] +
                         S.P[0][i] * S.Ps[1][0][j] + S.P[1][i] * S.Ps[1][1][j] + S.P[2][i] * S.Ps[1][2][j];
          } else {
            const double cc = S.C[0][i] * S.C[0][j] + S.C[1][i] * S.C[1][j] + S.C[2][i] * S.C[2][j];
            const double pp = S.P[0][i] * S.P[0][j] + S.P[1][i] * S.P[1][j] + S.P[2][i] * S.P[2][j];
            accR[m] += S.a.x * cc + S.b.x * pp;
            if (CPLX) accI[m] += S.a.y * cc + S.b.y * pp;
          }
        }
      }
      __syncwarp();
    }
    const int ncomp = CPLX ? 2 : 1;
    double *K = ke + (size_t)e * ncomp * n * n;
#pragma unroll
    for (int m = 0; m < MAXENT; ++m) {
      const int k = c0 + lane + 32 * m;
      if (k < nEnt) {
        const int i = pairI[k], j = pairJ[k];
        K[i * n + j] = K[j * n + i] = accR[m];
        if (CPLX) K[n * n + i * n + j] = K[n * n + j * n + i] = accI[m];
      }
    }
    __syncwarp();
    }
  }
}

static int launchElementKernels(fg_plan *plan, const DevTerms &terms, const DevTerms *dterms, double *ke, double *be, cudaStream_t s) {
  const PlanDev &p = plan->d;
  if (terms.nonSym) {
    const int perLane = (p.nb * p.nbU + 31) / 32;
    int64_t blocks = std::min<int64_t>((p.E + kWarpsPerBlockElem - 1) / kWarpsPerBlockElem, (int64_t)smCount() * 64);
    if (blocks < 1) blocks = 1;
    const bool cplx = terms.complexKe != 0;
    double2 *be2 = (double2 *)be;
    ProfScope prof("k_element_full_fp64", s);
#define FG_LAUNCH_FULL(M)                                                                                             \
  do {                                                                                                                \
    if (cplx) k_element_full_fp64<M, true><<<(unsigned)blocks, 32 * kWarpsPerBlockElem, 0, s>>>(p, dterms, ke, be2);  \
    else k_element_full_fp64<M, false><<<(unsigned)blocks, 32 * kWarpsPerBlockElem, 0, s>>>(p, dterms, ke, be2);     \
  } while (0)
    if (perLane <= 2) FG_LAUNCH_FULL(2);
    else if (perLane <= 8) FG_LAUNCH_FULL(8);
    else if (perLane <= 13) FG_LAUNCH_FULL(13);
    else if (perLane <= 39) FG_LAUNCH_FULL(39);
    else {
      setLastError("FP64 full element kernel: more than 35 basis functions per element");
      return FG_ERR_UNSUPPORTED;
    }
#undef FG_LAUNCH_FULL
    countLaunch();
    FG_CUDA(cudaGetLastError());
    return FG_OK;
  }
  if (p.E > 0 && factoredFp64Applies(plan, terms)) {
    int st = launchFactoredFp64(plan, terms, dterms, ke, s);
    if (st) return st;
    if (be) {
      if (p.form == FG_FORM_1) {
        setLastError("HCurl fields take no source terms");
        return FG_ERR_UNSUPPORTED;
      }
      return launchRhsFp64(plan, dterms, be, s);
    }
    return FG_OK;
  }
  if (p.form == FG_FORM_1) {
    const int nEnt = p.nb * (p.nb + 1) / 2;
    const int perLane = (nEnt + 31) / 32;
    int64_t blocks = std::min<int64_t>((p.E + kWarpsPerBlockElem - 1) / kWarpsPerBlockElem, (int64_t)smCount() * 64);
    if (blocks < 1) blocks = 1;
    const bool cplx = terms.complexKe != 0;
    ProfScope prof("k_element_hcurl_fp64", s);
#define FG_LAUNCH_HC(M)                                                                                              \
  do {                                                                                                               \
    if (cplx) k_element_hcurl_fp64<M, true><<<(unsigned)blocks, 32 * kWarpsPerBlockElem, 0, s>>>(p, dterms, ke);     \
    else k_element_hcurl_fp64<M, false><<<(unsigned)blocks, 32 * kWarpsPerBlockElem, 0, s>>>(p, dterms, ke);        \
  } while (0)
    if (perLane <= 1) FG_LAUNCH_HC(1);
    else FG_LAUNCH_HC(8);  // 256 pairs per chunk: one chunk up to 22 functions, more chunks beyond
#undef FG_LAUNCH_HC
    (void)be;
    countLaunch();
    FG_CUDA(cudaGetLastError());
    return FG_OK;
  }
  if (p.mult != 1 || terms.hasElastic) {
    if (p.mult != 3 || terms.hasSource) {
      setLastError("FP64 element kernel: compound fields take the elastic and mass terms only");
      return FG_ERR_UNSUPPORTED;
    }
    const int nPairs = p.nb * (p.nb + 1) / 2;
    const int perLane = (nPairs + 31) / 32;
    int64_t blocks = std::min<int64_t>((p.E + kWarpsPerBlockElem - 1) / kWarpsPerBlockElem, (int64_t)smCount() * 64);
    if (blocks < 1) blocks = 1;
    const bool cplx = terms.complexKe != 0;
    ProfScope prof("k_element_elastic_fp64", s);
#define FG_LAUNCH_EL(M)                                                                                                    \
  do {                                                                                                                     \
    if (cplx) k_element_elastic_fp64<M, true><<<(unsigned)blocks, 32 * kWarpsPerBlockElem, 0, s>>>(p, dterms, ke, (double2 *)be); \
    else k_element_elastic_fp64<M, false><<<(unsigned)blocks, 32 * kWarpsPerBlockElem, 0, s>>>(p, dterms, ke, (double2 *)be); \
  } while (0)
    if (perLane <= 2) FG_LAUNCH_EL(2);
    else if (perLane <= 4) FG_LAUNCH_EL(4);
    else if (perLane <= 8) FG_LAUNCH_EL(8);
    else {
      setLastError("FP64 elastic kernel: more than 21 scalar basis functions per element");
      return FG_ERR_UNSUPPORTED;
    }
#undef FG_LAUNCH_EL
    countLaunch();
    FG_CUDA(cudaGetLastError());
    return FG_OK;
  }
  const int nEnt = p.nb * (p.nb + 1) / 2;
  const int perLane = (nEnt + 31) / 32;
  const int sms = smCount();
  int64_t blocks = (p.E + kWarpsPerBlockElem - 1) / kWarpsPerBlockElem;
  blocks = std::min<int64_t>(blocks, (int64_t)sms * 64);
  if (blocks < 1) blocks = 1;
  const bool cplx = terms.complexKe != 0;
  double2 *be2 = (double2 *)be;
#define FG_LAUNCH_ELEM(M)                                                                                   \
  do {                                                                                                      \
    if (cplx) k_element_fp64<M, true><<<(unsigned)blocks, 32 * kWarpsPerBlockElem, 0, s>>>(p, dterms, ke, be2); \
    else k_element_fp64<M, false><<<(unsigned)blocks, 32 * kWarpsPerBlockElem, 0, s>>>(p, dterms, ke, be2);  \
  } while (0)
  ProfScope prof("k_element_fp64", s);
  if (perLane <= 1) FG_LAUNCH_ELEM(1);
  else if (perLane <= 8) FG_LAUNCH_ELEM(8);
  else if (perLane <= 20) FG_LAUNCH_ELEM(20);
  else {
    setLastError("FP64 element kernel: more than 35 basis functions per element");
    return FG_ERR_UNSUPPORTED;
  }
#undef FG_LAUNCH_ELEM
  countLaunch();
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

// With Jacobian modificators the kernels flag integration points outside a
// shell; the flag is read back here (the reference throws from apply()).
int launchElementFp64(fg_plan *plan, const DevTerms &terms, const DevTerms *dterms, double *ke, double *be, cudaStream_t s) {
  const PlanDev &p = plan->d;
  if (!terms.hasJacMod || p.E == 0) return launchElementKernels(plan, terms, dterms, ke, be, s);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  FG_CUDA(cudaStreamIsCapturing(s, &cs));
  if (cs != cudaStreamCaptureStatusNone) {
    setLastError("Jacobian modificators: the shell-radius check reads a device word back, which a stream capture cannot");
    return FG_ERR_UNSUPPORTED;
  }
  FG_CUDA(cudaMemsetAsync(p.jmErr, 0, sizeof(int), s));
  int st = launchElementKernels(plan, terms, dterms, ke, be, s);
  if (st) return st;
  FG_CUDA(cudaMemcpyAsync(plan->jmErrHost, p.jmErr, sizeof(int), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  if (*plan->jmErrHost) {
    setLastError("Jacobian modificator: an integration point lies outside the shell [r_min, r_max]");
    return FG_ERR_ARG;
  }
  return FG_OK;
}

int prepareOutputs(fg_plan *plan, double *csr_values, double *rhs, Outputs *o) {
  if (!csr_values) {
    setLastError("csr_values must not be NULL");
    return FG_ERR_ARG;
  }
  o->hostValues = !isDevicePointer(csr_values);
  if (plan->accumulate && (o->hostValues || (rhs && !isDevicePointer(rhs)))) {
    setLastError("accumulating assembly adds into device outputs: csr_values and rhs must be device memory");
    return FG_ERR_ARG;
  }
  o->values = csr_values;
  if (o->hostValues) {
    int st = ensureDevice((void **)&plan->values, &plan->valuesBytes, plan->d.nnz * 16);
    if (st) return st;
    o->values = plan->values;
  }
  o->rhs = rhs;
  if (rhs) {
    o->hostRhs = !isDevicePointer(rhs);
    if (o->hostRhs) {
      int st = ensureDevice((void **)&plan->rhs, &plan->rhsBytes, plan->d.nRows * 16);
      if (st) return st;
      o->rhs = plan->rhs;
    }
  }
  return FG_OK;
}

int finishOutputs(fg_plan *plan, const Outputs &o, double *csr_values, double *rhs, cudaStream_t s) {
  if (o.hostValues && !o.valuesCopied) FG_CUDA(cudaMemcpyAsync(csr_values, o.values, plan->d.nnz * 16, cudaMemcpyDeviceToHost, s));
  if (o.valuesCopied) FG_CUDA(cudaStreamSynchronize(plan->copyStream));
  if (rhs && o.hostRhs) FG_CUDA(cudaMemcpyAsync(rhs, o.rhs, plan->d.nRows * 16, cudaMemcpyDeviceToHost, s));
  if (o.hostValues || (rhs && o.hostRhs)) FG_CUDA(cudaStreamSynchronize(s));
  return FG_OK;
}

}  // namespace femg

using namespace femg;

extern "C" int fg_assemble_fp64(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, double frequency, const double *dirichlet,
                                double *csr_values, double *rhs, void *stream) {
  if (!plan) return FG_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  DevTerms dt;
  const DevTerms *dterms = nullptr;
  int st = resolveTerms(plan, terms, n_terms, frequency, &dt, &dterms, s);
  if (st) return st;
  if ((st = coupledLiftCheck(plan, rhs))) return st;
  const double *uD = nullptr;
  if ((st = uploadDirichlet(plan, dirichlet, &uD, s))) return st;
  Outputs o;
  if ((st = prepareOutputs(plan, csr_values, rhs, &o))) return st;
  const PlanDev &p = plan->d;
  const int ncomp = dt.complexKe ? 2 : 1;
  if ((st = ensureDevice((void **)&plan->ke, &plan->keBytes, (size_t)p.E * ncomp * p.n * p.nc * sizeof(double)))) return st;
  double *be = nullptr;
  if (dt.hasSource && rhs) {
    if ((st = ensureDevice((void **)&plan->be, &plan->beBytes, (size_t)p.E * p.n * 16))) return st;
    be = plan->be;
  }
  if (p.E > 0) {
    if ((st = launchElementFp64(plan, dt, dterms, plan->ke, be, s))) return st;
  }
  if ((st = gatherToOutputs(plan, plan->ke, dt.complexKe, 0, keRect(p.n, p.nc), be, uD, o, csr_values, s))) return st;
  return finishOutputs(plan, o, csr_values, rhs, s);
}
