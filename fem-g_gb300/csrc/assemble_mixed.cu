// Mixed-precision assembly: FP64 geometry, 3xTF32 tensor-core contraction
// (tcgen05, accumulators in TMEM), FP32 element matrices, FP64 CSR.
//
// The element contraction of BilinearTerm::evaluate (src/term/BilinearTerm.cpp:304-343)
//     Ke[i][j] = sum_q w_q det_q c (J_q^-T grad phi_j) . (J_q^-T grad phi_i) + c_m phi_j phi_i
// is refactored for affine elements with per-element coefficients into a
// product of a per-element factor row and a constant per-orientation tensor:
//     Ke[i][j] = sum_k D_e[k] T^o[k][i*n + j],
//     D_e = c det (K_00, K_11, K_22, K_01, K_02, K_12, c_m/c, 0),  K = J^-1 J^-T,
//     T^o[ab][ij] = sum_q w_q (d_a phi_j d_b phi_i + [a != b] d_b phi_j d_a phi_i),
//     T^o[6][ij]  = sum_q w_q phi_i phi_j       (orientation o's reference basis).
// Over all elements that is one GEMM C[M = elements, N = n^2] = A[M, K] B[K, N]
// with B shared by every element of an orientation: the tensor-core shape.
// 3xTF32: A = A_hi + A_lo, B = B_hi + B_lo (each part exactly representable
// in TF32), C = A_hi B_hi + A_lo B_hi + A_hi B_lo, realised as one MMA chain
// over K' = 3K with A' = [A_hi | A_lo | A_hi] and B' = [B_hi ; B_hi ; B_lo].
// Geometry (J, det, J^-1) and the factors are computed in FP64; the element
// matrices leave TMEM as FP32 and are reduced into the FP64 CSR by the same
// deterministic gather as the FP64 path.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <numeric>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"

namespace femg {

constexpr int kBM = 128;       // rows (element components) per tile = TMEM lanes
constexpr int kKp = 8;         // factor columns (7 used)
constexpr int kK3 = 3 * kKp;   // K' of the 3xTF32 chain
constexpr int kThreadsGemm = 256;

struct MixedState {
  int built = 0;
  int ncomp = 0, groups = 0;  // layout of the current tiles and buffers
  int n = 0, nn2 = 0, Npad = 0;
  // row stride of the FP32 element matrices: nn2, except for one-block fields
  // whose nn2 is not a multiple of 4 (order-4 tets: 1,225), padded to a
  // multiple of 8 floats so that every row starts on a 32-byte sector and the
  // contraction stores whole 16-byte vectors (the padding holds the zero
  // columns of the reference tensors)
  int ld = 0;
  int nOrient = 0;
  int blocks = 1;            // 9 component blocks per element for a compound field
  int kp = 0, k3 = 0;        // factor columns and K' of the 3xTF32 chain
  int rowsPerElem = 1;       // GEMM rows per element = groups * ncomp * blocks
  std::vector<int64_t> orientCount;
  int64_t rows = 0;          // GEMM rows = E * rowsPerElem
  float *A = nullptr;        // [rows][kK3] row-major split factors
  size_t Abytes = 0;
  float *B = nullptr;        // [nOrient] smem images of B' (core-matrix layout)
  int32_t *perm = nullptr;   // sorted rank -> element
  int4 *tiles = nullptr;     // [nTiles]: problem 0, orientation, first row, row count
  int nTiles = 0;
  int32_t *ctaStart = nullptr;  // contiguous tile ranges of the persistent CTAs
  int nCta = 0;
  int ctasPerSm = 1;            // contraction CTAs per SM (TMEM columns 512 / ctasPerSm each)
  alignas(64) CUtensorMap aMap;  // TMA view of A: [rows][k3] floats, box 4 x 128
  int mmaN = 256;               // N of one MMA instruction
  void *probDev = nullptr;      // this plan's GemmProblem on the device
  float *ke = nullptr;       // [E][groups][ncomp][ld] fp32 (layout: mixedLayout)
  size_t keBytes = 0;
  int *err = nullptr;        // device error word (wait timeouts)
  int *errHost = nullptr;    // pinned copy of err
  cudaEvent_t errEvent = nullptr;
  bool errPending = false;
};

// The layout of m->ke for the reduction
static KeLayout mixedLayout(const MixedState *m) {
  return KeLayout{m->blocks == 9 ? kKeBlocks3 : kKeFull, m->blocks == 9 ? m->n * m->n : m->ld};
}

// Reports (once) a device wait timeout recorded by an earlier launch: when
// wait is false only an already completed copy of the error word is read.
static int checkTimeout(MixedState *m, bool wait) {
  if (!m->errPending) return FG_OK;
  if (wait) {
    if (cudaEventSynchronize(m->errEvent) != cudaSuccess) return FG_ERR_CUDA;
  } else if (cudaEventQuery(m->errEvent) != cudaSuccess) {
    cudaGetLastError();  // not ready yet: check on a later call
    return FG_OK;
  }
  m->errPending = false;
  if (*m->errHost) {
    *m->errHost = 0;
    cudaMemset(m->err, 0, sizeof(int));
    setLastError("mixed path: a bounded device wait timed out");
    return FG_ERR_TIMEOUT;
  }
  return FG_OK;
}

#include "tc_ptx.cuh"

// ------------------------------------------------- geometry: factor rows

// One thread per element: J, det, J^-1 in FP64 from the element nodes at the
// first quadrature point (affine elements: the geometric Jacobian is constant), per-element coefficients,
// factors D_e split into TF32 hi/lo, written as row [hi | lo | hi] at the
// element's rank in the orientation-sorted order.
// ROWF: floats per factor row, 24 ([hi | lo | hi], the split contraction) or
// 16 ([hi | lo], the fused kernel, which reuses hi for the third product);
// rankOf null: rows in element order.
template <bool TENSOR, int ROWF = kK3>
__device__ __forceinline__ void factorsScalar(const PlanDev &p, const DevTerms *__restrict__ terms, const int32_t *__restrict__ rankOf,
                                              float *__restrict__ A, int ncomp, int rowsPerElem, int rowOff, int64_t e) {
  double X[kMaxNodes * 3];
  const int nx = p.p1geom ? p.dim + 1 : p.nn;
  for (int k = 0; k < nx; ++k)
    for (int c = 0; c < 3; ++c) X[3 * k + c] = p.xyz[3 * (int64_t)p.enodes[e * p.nn + k] + c];
  double J[9];
  if (p.p1geom) jacobianP1(p.dim, X, J);
  else jacobian(p.dim, p.nn, X, p.geoGrad, J);  // q = 0: affine
  // FP64 geometry without the explicit inverse (the FP64 pipe is GB300's
  // narrowest): with the cofactors C, J^-1 = C^T / det, so
  // det K = det J^-1 J^-T = (C^T C) / det, and det = J column 0 . C column 0.
  auto Jm = [&](int r, int c) { return J[3 * c + r]; };
  double C[9];  // C[3a + r] = (adj J)(a, r)
  C[0] = Jm(1, 1) * Jm(2, 2) - Jm(1, 2) * Jm(2, 1);
  C[1] = Jm(0, 2) * Jm(2, 1) - Jm(0, 1) * Jm(2, 2);
  C[2] = Jm(0, 1) * Jm(1, 2) - Jm(0, 2) * Jm(1, 1);
  C[3] = Jm(1, 2) * Jm(2, 0) - Jm(1, 0) * Jm(2, 2);
  C[4] = Jm(0, 0) * Jm(2, 2) - Jm(0, 2) * Jm(2, 0);
  C[5] = Jm(0, 2) * Jm(1, 0) - Jm(0, 0) * Jm(1, 2);
  C[6] = Jm(1, 0) * Jm(2, 1) - Jm(1, 1) * Jm(2, 0);
  C[7] = Jm(0, 1) * Jm(2, 0) - Jm(0, 0) * Jm(2, 1);
  C[8] = Jm(0, 0) * Jm(1, 1) - Jm(0, 1) * Jm(1, 0);
  const double det = C[0] * Jm(0, 0) + C[1] * Jm(1, 0) + C[2] * Jm(2, 0);
  double CC[6];  // (C C^T)(a, b) = det^2 K(a, b)
  const int ab[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  for (int k = 0; k < 6; ++k) {
    const int a = ab[k][0], b = ab[k][1];
    CC[k] = C[3 * a] * C[3 * b] + C[3 * a + 1] * C[3 * b + 1] + C[3 * a + 2] * C[3 * b + 2];
  }
  double xc[3] = {0.0, 0.0, 0.0};  // coefficients are per element here: any point of it
  double2 cgg = make_double2(0.0, 0.0), cm = make_double2(0.0, 0.0);
  for (int t = 0; t < terms->n; ++t) {
    const DevTerm &T = terms->t[t];
    const double2 v = evalExpr(T.coef, e, xc);
    // real factor times real coefficient: one multiply instead of a complex product
    const double2 fv = (T.factor.y == 0.0 && v.y == 0.0) ? make_double2(T.factor.x * v.x, 0.0) : cmul(T.factor, v);
    if (T.kind == FG_TERM_GRAD_GRAD) cgg = cadd(cgg, fv);
    else if (T.kind == FG_TERM_MASS) cm = cadd(cm, fv);
  }
  const double idet = 1.0 / det;
  const int64_t r0 = (rankOf ? (int64_t)rankOf[e] : e) * rowsPerElem + rowOff;
  // tensor grad-grad term (TENSOR: the terms have one; a separate
  // instantiation keeps the scalar kernel's registers):
  // det J^-1 A J^-T = C^T A C / det in place of c det K
  double2 A6[6];
  if (TENSOR) diffusionTensor(terms, 0, e, xc, cgg, A6);
  for (int comp = 0; comp < ncomp; ++comp) {
    const double g = (comp == 0 ? cgg.x : cgg.y) * idet;
    const double m = (comp == 0 ? cm.x : cm.y) * det;
    float hi[kKp], lo[kKp];
    if (TENSOR) {
      const int sym[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
      double CA[9];  // CA[3a + s] = sum_r C[3a + r] A(r, s)
      for (int a = 0; a < 3; ++a)
        for (int s2 = 0; s2 < 3; ++s2) {
          double v = 0.0;
          for (int r = 0; r < 3; ++r) v += C[3 * a + r] * (comp == 0 ? A6[sym[r][s2]].x : A6[sym[r][s2]].y);
          CA[3 * a + s2] = v;
        }
      for (int k = 0; k < 6; ++k) {
        const int a = ab[k][0], b = ab[k][1];
        const double f = (CA[3 * a] * C[3 * b] + CA[3 * a + 1] * C[3 * b + 1] + CA[3 * a + 2] * C[3 * b + 2]) * idet;
        splitTf32Dev(f, hi[k], lo[k]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 6; ++k) splitTf32Dev(g * CC[k], hi[k], lo[k]);
    }
    splitTf32Dev(m, hi[6], lo[6]);
    hi[7] = lo[7] = 0.0f;
    // [hi | lo | hi] (or [hi | lo]) as 16-byte stores (rows are 96 or 64 bytes)
    float4 *row = reinterpret_cast<float4 *>(A + (r0 + comp) * ROWF);
    row[0] = make_float4(hi[0], hi[1], hi[2], hi[3]);
    row[1] = make_float4(hi[4], hi[5], hi[6], hi[7]);
    row[2] = make_float4(lo[0], lo[1], lo[2], lo[3]);
    row[3] = make_float4(lo[4], lo[5], lo[6], lo[7]);
    if (ROWF == kK3) {
      row[4] = row[0];
      row[5] = row[1];
    }
  }
}

template <bool TENSOR>
__global__ void k_factors(const PlanDev p, const DevTerms *__restrict__ terms, const int32_t *__restrict__ rankOf, float *__restrict__ A,
                          int ncomp, int rowsPerElem, int rowOff) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < p.E) factorsScalar<TENSOR>(p, terms, rankOf, A, ncomp, rowsPerElem, rowOff, e);
}

// Factor rows [hi | lo] in element order for the fused kernel (one
// component: real element matrices)
template <bool TENSOR>
__global__ void k_factors_compact(const PlanDev p, const DevTerms *__restrict__ terms, float *__restrict__ A) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < p.E) factorsScalar<TENSOR, 16>(p, terms, nullptr, A, 1, 1, 0, e);
}

int launchFactorsCompact(const PlanDev &p, const DevTerms *dterms, bool tensor, float *A16, cudaStream_t s) {
  if (p.E == 0) return FG_OK;
  ProfScope prof("k_factors_compact", s);
  if (tensor) k_factors_compact<true><<<(unsigned)((p.E + 127) / 128), 128, 0, s>>>(p, dterms, A16);
  else k_factors_compact<false><<<(unsigned)((p.E + 127) / 128), 128, 0, s>>>(p, dterms, A16);
  countLaunch();
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

// Compound field with the isotropic Tensor4 term: for every component pair
// (a, b) (test component a, unknown component b) the block of the element
// matrix is  Ke_ab[i][j] = sum_{p,p'} D_ab[p p'] S_{p p'}[i][j] + D_ab[9] M[i][j]
// with S_{pp'}[i][j] = sum_q w d_p phi_j d_p' phi_i (reference gradients),
// M = sum_q w phi_i phi_j and, with J^-1 = Ji (affine element),
//   D_ab[p p'] = det (lambda Ji[p][b] Ji[p'][a] + mu Ji[p][a] Ji[p'][b] + mu d_ab K[p][p']),
//   D_ab[9]   = det c_m d_ab,   K = Ji Ji^T.
// 16 factor columns (10 used); rows (element, component of the coefficient,
// block a*3+b) in the orientation-sorted element order.
constexpr int kKpE = 16;
constexpr int kK3E = 3 * kKpE;
__device__ __forceinline__ void factorsElastic(const PlanDev &p, const DevTerms *__restrict__ terms, const int32_t *__restrict__ rankOf,
                                               float *__restrict__ A, int ncomp, int rowsPerElem, int rowOff, int64_t e) {
  double X[kMaxNodes * 3];
  const int nx = p.p1geom ? p.dim + 1 : p.nn;
  for (int k = 0; k < nx; ++k)
    for (int c = 0; c < 3; ++c) X[3 * k + c] = p.xyz[3 * (int64_t)p.enodes[e * p.nn + k] + c];
  double J[9], Ji[9];
  const double det = p.p1geom ? jacobianP1(p.dim, X, J) : jacobian(p.dim, p.nn, X, p.geoGrad, J);
  jacobianInverse(J, det, Ji);  // Ji[3p + a] = (J^-1)(p, a)
  double K[9];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) K[3 * a + b] = Ji[3 * a] * Ji[3 * b] + Ji[3 * a + 1] * Ji[3 * b + 1] + Ji[3 * a + 2] * Ji[3 * b + 2];
  double xc[3] = {0.0, 0.0, 0.0};
  double2 lam = make_double2(0.0, 0.0), mu = make_double2(0.0, 0.0), cm = make_double2(0.0, 0.0);
  for (int t = 0; t < terms->n; ++t) {
    const DevTerm &T = terms->t[t];
    if (T.kind == FG_TERM_ELASTIC) {
      lam = cadd(lam, cmul(T.factor, evalExpr(T.coef, e, xc)));
      mu = cadd(mu, cmul(T.factor, evalExpr(T.coef2, e, xc)));
    } else if (T.kind == FG_TERM_MASS) {
      cm = cadd(cm, cmul(T.factor, evalExpr(T.coef, e, xc)));
    }
  }
  const int64_t r0 = (int64_t)rankOf[e] * rowsPerElem + rowOff;
  for (int comp = 0; comp < ncomp; ++comp) {
    const double l = (comp == 0 ? lam.x : lam.y) * det, m = (comp == 0 ? mu.x : mu.y) * det;
    const double c = (comp == 0 ? cm.x : cm.y) * det;
    double lJ[9], mJ[9];  // l Ji, m Ji
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      lJ[k] = l * Ji[k];
      mJ[k] = m * Ji[k];
    }
    const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        float hi[12], lo[12];
#pragma unroll
        for (int pp = 0; pp < 3; ++pp)
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            double d = fma(lJ[3 * pp + b], Ji[3 * q + a], mJ[3 * pp + a] * Ji[3 * q + b]);
            if (a == b) d = fma(m, K[3 * pp + q], d);
            splitTf32Dev(d, hi[3 * pp + q], lo[3 * pp + q]);
          }
        if (a == b) splitTf32Dev(c, hi[9], lo[9]);
        else hi[9] = lo[9] = 0.0f;
        hi[10] = hi[11] = lo[10] = lo[11] = 0.0f;
        // [hi | lo | hi] of 16 columns (10 used) as 16-byte stores (rows are 192 bytes)
        float4 *row = reinterpret_cast<float4 *>(A + (r0 + comp * 9 + 3 * a + b) * kK3E);
        const float4 h0 = make_float4(hi[0], hi[1], hi[2], hi[3]), h1 = make_float4(hi[4], hi[5], hi[6], hi[7]),
                     h2 = make_float4(hi[8], hi[9], 0.0f, 0.0f);
        row[0] = h0;
        row[1] = h1;
        row[2] = h2;
        row[3] = zero;
        row[4] = make_float4(lo[0], lo[1], lo[2], lo[3]);
        row[5] = make_float4(lo[4], lo[5], lo[6], lo[7]);
        row[6] = make_float4(lo[8], lo[9], 0.0f, 0.0f);
        row[7] = zero;
        row[8] = h0;
        row[9] = h1;
        row[10] = h2;
        row[11] = zero;
      }
  }
}

__global__ void k_factors_elastic(const PlanDev p, const DevTerms *__restrict__ terms, const int32_t *__restrict__ rankOf,
                                  float *__restrict__ A, int ncomp, int rowsPerElem, int rowOff) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < p.E) factorsElastic(p, terms, rankOf, A, ncomp, rowsPerElem, rowOff, e);
}

// HCurl field (lowest order and up), affine elements, per-element coefficients:
//   curl-curl: sum_q w det c (J c_j / det) . (J c_i / det) = (c / det) sum_ab (J^T J)_ab T_ab[i][j]
//   mass:      sum_q w det c (J^-T v_j) . (J^-T v_i)       = c det sum_ab (J^-1 J^-T)_ab T_6+ab[i][j]
// 12 factors in 16 columns, rows [hi | lo | hi] as for the scalar field.
__device__ __forceinline__ void factorsHcurl(const PlanDev &p, const DevTerms *__restrict__ terms, const int32_t *__restrict__ rankOf,
                                             float *__restrict__ A, int ncomp, int rowsPerElem, int rowOff, int64_t e) {
  double X[kMaxNodes * 3];
  const int nx = p.p1geom ? p.dim + 1 : p.nn;
  for (int k = 0; k < nx; ++k)
    for (int c = 0; c < 3; ++c) X[3 * k + c] = p.xyz[3 * (int64_t)p.enodes[e * p.nn + k] + c];
  double J[9], Ji[9];
  const double det = p.p1geom ? jacobianP1(p.dim, X, J) : jacobian(p.dim, p.nn, X, p.geoGrad, J);
  jacobianInverse(J, det, Ji);
  const int ab[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  double K[6], M[6];
  for (int k = 0; k < 6; ++k) {
    const int a = ab[k][0], b = ab[k][1];
    K[k] = Ji[3 * a] * Ji[3 * b] + Ji[3 * a + 1] * Ji[3 * b + 1] + Ji[3 * a + 2] * Ji[3 * b + 2];
    M[k] = J[3 * a] * J[3 * b] + J[3 * a + 1] * J[3 * b + 1] + J[3 * a + 2] * J[3 * b + 2];  // columns of J
  }
  double xc[3] = {0.0, 0.0, 0.0};
  double2 cc = make_double2(0.0, 0.0), cm = make_double2(0.0, 0.0);
  for (int t = 0; t < terms->n; ++t) {
    const DevTerm &T = terms->t[t];
    if (T.kind == FG_TERM_GRAD_GRAD) cc = cadd(cc, cmul(T.factor, evalExpr(T.coef, e, xc)));
    else if (T.kind == FG_TERM_MASS) cm = cadd(cm, cmul(T.factor, evalExpr(T.coef, e, xc)));
  }
  const int64_t r0 = (int64_t)rankOf[e] * rowsPerElem + rowOff;
  // tensor terms (Maxwell PML): (J^T A J)(a, b) / det for the curls and
  // det (J^-1 B J^-T)(a, b) for the values, in place of c M / det and c det K
  const bool tensor = terms->tensorTerm >= 0 || terms->tensorMassTerm >= 0;
  double2 A6[6], B6[6];
  if (tensor) {
    coefTensor(terms, terms->tensorTerm, terms->tensor, 0, e, xc, cc, A6);
    coefTensor(terms, terms->tensorMassTerm, terms->tensorMass, 0, e, xc, cm, B6);
  }
  for (int comp = 0; comp < ncomp; ++comp) {
    const double gc = (comp == 0 ? cc.x : cc.y) / det, gm = (comp == 0 ? cm.x : cm.y) * det;
    float hi[kKpE], lo[kKpE];
    if (tensor) {
      double FA[6], FB[6];
      congruence6(J, A6, comp, FA);
      congruence6(Ji, B6, comp, FB);
      for (int k = 0; k < 6; ++k) {
        splitTf32Dev(FA[k] / det, hi[k], lo[k]);
        splitTf32Dev(FB[k] * det, hi[6 + k], lo[6 + k]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        splitTf32Dev(gc * M[k], hi[k], lo[k]);
        splitTf32Dev(gm * K[k], hi[6 + k], lo[6 + k]);
      }
    }
#pragma unroll
    for (int k = 12; k < kKpE; ++k) hi[k] = lo[k] = 0.0f;
    float4 *row = reinterpret_cast<float4 *>(A + (r0 + comp) * kK3E);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      row[q] = make_float4(hi[4 * q], hi[4 * q + 1], hi[4 * q + 2], hi[4 * q + 3]);
      row[4 + q] = make_float4(lo[4 * q], lo[4 * q + 1], lo[4 * q + 2], lo[4 * q + 3]);
      row[8 + q] = row[q];
    }
  }
}

__global__ void k_factors_hcurl(const PlanDev p, const DevTerms *__restrict__ terms, const int32_t *__restrict__ rankOf,
                                float *__restrict__ A, int ncomp, int rowsPerElem, int rowOff) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < p.E) factorsHcurl(p, terms, rankOf, A, ncomp, rowsPerElem, rowOff, e);
}

// Factor rows of many plans in one launch: thread -> (job, element) through
// the jobs' element offsets
__global__ void k_factors_batch(const FactorJob *__restrict__ jobs, int nJobs, int64_t total) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  int lo = 0, hi = nJobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].elemStart <= g) lo = mid;
    else hi = mid - 1;
  }
  const FactorJob &J = jobs[lo];
  const int64_t e = g - J.elemStart;
  if (J.kind == 1) factorsElastic(J.p, J.terms, J.rankOf, J.A, J.ncomp, J.rowsPerElem, J.rowOff, e);
  else if (J.kind == 2) factorsHcurl(J.p, J.terms, J.rankOf, J.A, J.ncomp, J.rowsPerElem, J.rowOff, e);
  else if (J.kind == 3) factorsScalar<true>(J.p, J.terms, J.rankOf, J.A, J.ncomp, J.rowsPerElem, J.rowOff, e);
  else factorsScalar<false>(J.p, J.terms, J.rankOf, J.A, J.ncomp, J.rowsPerElem, J.rowOff, e);
}

// --------------------------------------------------- tcgen05 contraction

// Tiles of one launch: tile t = (problem, orientation, first row, rows);
// CTA b takes the contiguous tiles [ctaStart[b], ctaStart[b + 1]).
struct GemmSched {
  CUtensorMap aMap;  // one problem: its factor rows [rows][K3] as a TMA tensor (box 4 x 128)
  const GemmProblem *probs;
  const int4 *tiles;
  const int32_t *ctaStart;
  int *err;
  int tma;           // A tiles by TMA through aMap (one problem), else by cp.async
  long long mmaWaitCycles;  // bound of the wait for an MMA chain (fg_set_wait_limit)
  // dynamic schedule (batches): CTAs take `chunk` consecutive tiles at a time
  // from the counter `next` (zeroed before the launch) until nTiles; null:
  // the static ranges of ctaStart
  int *next;
  int nTiles, chunk;
};


// A tile of rows [row0, row0 + nrows) into the core-matrix image at As:
// row r, 16-byte chunk kc -> core matrix (r/8, kc), K-direction stride 2048 B;
// rows past nrows are zero-filled
__device__ inline void loadATile(const GemmProblem &g, uint32_t As, int row0, int nrows, int tid) {
  const int chunks = g.K3 / 4;
  for (int c = tid; c < kBM * chunks; c += kThreadsGemm) {
    const int r = c / chunks, kc = c % chunks;
    const bool live = r < nrows;
    const float *src = g.A + (size_t)(row0 + (live ? r : 0)) * g.K3 + kc * 4;
    cpAsync16(As + kc * 2048 + (r >> 3) * 128 + (r & 7) * 16, src, live ? 16u : 0u);
  }
  cpAsyncCommit();
}

// The A tile of rows [row0, row0 + nrows) into As: by TMA (one thread; the
// whole 128-row box, rows past the array read as zero) completing on `bar`,
// or by cp.async from every thread.
__device__ inline void issueATile(const GemmSched &sc, const GemmProblem &g, float *As, int row0, int nrows, int tid, uint64_t *bar) {
  if (sc.tma) {
    if (tid == 0) {
      mbarExpectTx(bar, (uint32_t)(kBM * g.K3 * 4));
      for (int kc = 0; kc < g.K3 / 4; ++kc) tmaLoad2d(smemAddr(As) + kc * 2048, &sc.aMap, 4 * kc, row0, bar);
    }
  } else {
    loadATile(g, smemAddr(As), row0, nrows, tid);
  }
}

// The B image of orientation o (Npad x K3 floats, core-matrix layout) by
// one TMA bulk copy completing on `bar`.
__device__ inline void loadB(const GemmProblem &g, float *Bs, int o, int tid, uint64_t *bar) {
  if (tid == 0) {
    const uint32_t bytes = (uint32_t)g.Npad * (uint32_t)g.K3 * 4u;
    mbarExpectTx(bar, bytes);
    bulkLoad(smemAddr(Bs), g.B + (size_t)o * g.Npad * g.K3, bytes, bar);
  }
}

// drain TMEM columns [c0, c1) of this warp's 32 lanes into the element rows
// (element-matrix column = colOff + TMEM column). Full 32-column chunks go
// through a padded per-warp stage (32 rows x 36 floats) so that each float4
// store instruction writes 4 rows x 128 contiguous bytes instead of 32
// scattered 16-byte pieces.
__device__ inline void drainColumns(const GemmProblem &g, uint32_t tmemRow, float *out, bool live, int c0, int c1, float *stage,
                                    int colOff) {
  const int lane = threadIdx.x & 31;
  const bool vec = (g.ld & 3) == 0;
  out += colOff;
  // columns left in the element row, its padding included (the reference
  // tensors' zero columns land there)
  const int nn2 = g.ld - colOff;
  int c = c0;
  for (; c + 32 <= c1; c += 32) {
    float v[32];
    tmemLoad32(tmemRow + (uint32_t)c, v);
    if (vec && c + 32 <= nn2) {
#pragma unroll
      for (int k = 0; k < 32; k += 4) *reinterpret_cast<float4 *>(stage + lane * 36 + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
      __syncwarp();
      const int sub = lane >> 3, part = lane & 7;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int src = 4 * q + sub;
        float *dst = reinterpret_cast<float *>(__shfl_sync(0xffffffffu, reinterpret_cast<uintptr_t>(out), src));
        const bool dlive = __shfl_sync(0xffffffffu, live ? 1 : 0, src) != 0;
        const float4 val = *reinterpret_cast<const float4 *>(stage + src * 36 + 4 * part);
        if (dlive) *reinterpret_cast<float4 *>(dst + c + 4 * part) = val;
      }
      __syncwarp();
    } else {
      // rows not 16-byte aligned (n^2 not a multiple of 4): transpose through
      // the stage and write one row per instruction, 32 consecutive floats
#pragma unroll
      for (int k = 0; k < 32; ++k) stage[lane * 33 + k] = v[k];
      __syncwarp();
      for (int rr = 0; rr < 32; ++rr) {
        float *dst = reinterpret_cast<float *>(__shfl_sync(0xffffffffu, reinterpret_cast<uintptr_t>(out), rr));
        const bool dlive = __shfl_sync(0xffffffffu, live ? 1 : 0, rr) != 0;
        if (dlive && c + lane < nn2) dst[c + lane] = stage[rr * 33 + lane];
      }
      __syncwarp();
    }
  }
  if (c < c1) {
    float v[16];
    tmemLoad16(tmemRow + (uint32_t)c, v);
    if (vec && c + 16 <= nn2) {
      if (live) {
#pragma unroll
        for (int k = 0; k < 16; k += 4) *reinterpret_cast<float4 *>(out + c + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
      }
    } else {
      // two rows per instruction, 16 consecutive floats each
#pragma unroll
      for (int k = 0; k < 16; ++k) stage[lane * 33 + k] = v[k];
      __syncwarp();
      const int col = lane & 15;
      for (int rr = 0; rr < 32; rr += 2) {
        const int row = rr + (lane >> 4);
        float *dst = reinterpret_cast<float *>(__shfl_sync(0xffffffffu, reinterpret_cast<uintptr_t>(out), row));
        const bool dlive = __shfl_sync(0xffffffffu, live ? 1 : 0, row) != 0;
        if (dlive && c + col < nn2) dst[c + col] = stage[row * 33 + col];
      }
      __syncwarp();
    }
  }
}

// Persistent: one CTA per SM, 8 warps, over a contiguous range of tiles of
// one or many problems. Warp 0 owns the TMEM allocation, thread 0 issues the
// MMAs, all warps drain TMEM (warp w: lanes of quadrant w % 4, half w / 4 of
// the columns). Element matrices wider than the 512 TMEM columns are done in
// column chunks of 512. The next tile's A is fetched with cp.async while the
// current tile computes and drains when both share the B image in shared
// memory; B is reloaded when the (problem, orientation) changes.
__global__ void __launch_bounds__(kThreadsGemm, 2)
    k_contract_tf32x3(const __grid_constant__ GemmSched sc, int maxK3, int tmemCols) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ GemmProblem gs;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem);      // MMA completion
  uint64_t *aBar = reinterpret_cast<uint64_t *>(smem + 8);  // [2] TMA loads of the A buffers
  uint64_t *bBar = reinterpret_cast<uint64_t *>(smem + 24); // TMA load of the B image
  uint32_t *tmemBase = reinterpret_cast<uint32_t *>(smem + 32);
  float *Stage = reinterpret_cast<float *>(smem + 128);     // 8 warps x 32 x 36 floats
  float *As0 = Stage + 8 * 32 * 36;                         // 2 x kBM * maxK3, 128-byte aligned (TMA)
  float *Bs = As0 + 2 * kBM * maxK3;                        // Npad * K3
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, half = warp >> 2;

  if (warp == 0) {
    tmemAlloc(tmemBase, (uint32_t)tmemCols);
    tmemRelinquish();
  }
  if (tid == 0) {
    mbarInit(mbar, 1);
    mbarInit(&aBar[0], 1);
    mbarInit(&aBar[1], 1);
    mbarInit(bBar, 1);
    fenceMbarInit();
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = *tmemBase;
  const uint32_t bBase = smemAddr(Bs);
  uint32_t phase = 0;
  uint32_t aParity = 0, aPending = 0;  // per A buffer: completion parity, load in flight
  uint32_t bParity = 0, bPending = 0;  // the B image: completion parity, load in flight
  bool failed = false;
  // the tiles of this CTA: [t, ce) is the current chunk. Static: one chunk,
  // the CTA's range. Dynamic: chunks taken from the counter; the next one is
  // taken while the current chunk's last tile runs (sGrab, written by thread
  // 0 and read by all after the barrier that follows in the same tile).
  __shared__ int sGrab;
  int t, ce;
  if (sc.next) {
    if (tid == 0) sGrab = atomicAdd(sc.next, sc.chunk);
    __syncthreads();
    t = sGrab;
    ce = min(t + sc.chunk, sc.nTiles);
  } else {
    t = sc.ctaStart[blockIdx.x];
    ce = sc.ctaStart[blockIdx.x + 1];
  }
  if (t < ce) {
    const int4 T = sc.tiles[t];
    if (tid == 0) gs = sc.probs[T.x];
    __syncthreads();
    loadB(gs, Bs, T.y, tid, bBar);
    bPending = 1;
    issueATile(sc, gs, As0, T.z, T.w, tid, &aBar[0]);
    aPending |= 1u;
  }
  for (int it = 0; t < ce && !failed; ++it) {
    const int buf = it & 1;
    const int4 T = sc.tiles[t];
    if (sc.next && t + 1 == ce && tid == 0) sGrab = atomicAdd(sc.next, sc.chunk);
    const int o = T.y, row0 = T.z, nrows = T.w;
    const uint32_t aAddr = smemAddr(As0 + buf * kBM * gs.K3);
    const uint32_t bLbo = (uint32_t)gs.Npad * 16u;  // K-adjacent core matrices of B
    if (sc.tma) {
      const bool okA = mbarWait(&aBar[buf], (aParity >> buf) & 1u);
      if (__syncthreads_or(okA ? 0 : 1)) {
        if (tid == 0) atomicExch(sc.err, 1);
        failed = true;
        break;
      }
      aParity ^= 1u << buf;
      aPending &= ~(1u << buf);
    } else {
      cpAsyncWaitAll();
    }
    if (bPending) {
      const bool okB = mbarWait(bBar, bParity);
      if (__syncthreads_or(okB ? 0 : 1)) {
        if (tid == 0) atomicExch(sc.err, 1);
        failed = true;
        break;
      }
      bParity ^= 1u;
      bPending = 0;
    }
    fenceProxyAsync();  // cp.async A tiles (generic proxy) before the MMAs read them
    __syncthreads();
    // the next tile (in this chunk, or the first of the next one taken), and
    // the prefetch of its A when it shares this B image
    int tn, ceN;
    if (t + 1 < ce) {
      tn = t + 1;
      ceN = ce;
    } else if (sc.next) {
      tn = sGrab;
      ceN = min(tn + sc.chunk, sc.nTiles);
    } else {
      tn = ceN = 0;
    }
    const bool hasNext = tn < ceN;
    int4 Tn = make_int4(-1, -1, 0, 0);
    if (hasNext) Tn = sc.tiles[tn];
    const bool nextSameB = hasNext && Tn.x == T.x && Tn.y == o;
    const int r = quad * 32 + lane;
    const bool live = r < nrows;
    const int grow = row0 + r;
    const int64_t e = live ? gs.perm[grow / gs.rowsPerElem] : 0;
    float *out = gs.ke + ((size_t)e * gs.rowsPerElem + (grow % gs.rowsPerElem)) * gs.ld;
    const uint32_t tmemRow = tmem + ((uint32_t)(quad * 32) << 16);
    float *stage = Stage + warp * (32 * 36);
    for (int n0 = 0; n0 < gs.Npad && !failed; n0 += tmemCols) {
      const int ncols = min(tmemCols, gs.Npad - n0);
      if (tid == 0) {
        tcFenceAfter();
        for (int c0 = 0; c0 < ncols; c0 += gs.mmaN) {
          const int nc = min(gs.mmaN, ncols - c0);
          const uint32_t idesc = idescTf32(kBM, nc);
          for (int ks = 0; ks < gs.K3 / 8; ++ks) {
            const uint64_t ad = smemDesc(aAddr + ks * 2 * 2048, 2048, 128);
            const uint64_t bd = smemDesc(bBase + ks * 2 * bLbo + ((n0 + c0) >> 3) * 128, bLbo, 128);
            mmaTf32(tmem + (uint32_t)c0, ad, bd, idesc, ks > 0 ? 1u : 0u);
          }
        }
        mmaCommit(mbar);
      }
      if (n0 == 0 && nextSameB) {
        issueATile(sc, gs, As0 + (buf ^ 1) * kBM * gs.K3, Tn.z, Tn.w, tid, &aBar[buf ^ 1]);
        aPending |= 1u << (buf ^ 1);
      }
      __syncwarp();
      const bool ok = mbarWaitFor(mbar, phase, sc.mmaWaitCycles);
      failed = __syncthreads_or(ok ? 0 : 1) != 0;  // block-uniform
      if (failed) {
        if (tid == 0) atomicExch(sc.err, 1);
      } else {
        phase ^= 1u;
      }
      tcFenceAfter();
      if (!failed) {
        const int colSplit = ((ncols / 2 + 15) / 16) * 16;
        if (half == 0) drainColumns(gs, tmemRow, out, live, 0, min(colSplit, ncols), stage, n0);
        else drainColumns(gs, tmemRow, out, live, min(colSplit, ncols), ncols, stage, n0);
      }
      tcFenceBefore();
      __syncthreads();
    }
    if (!failed && hasNext && !nextSameB) {
      // problem or orientation change: the MMAs are done with Bs, reload it and the next A
      if (tid == 0 && Tn.x != T.x) gs = sc.probs[Tn.x];
      __syncthreads();
      loadB(gs, Bs, Tn.y, tid, bBar);
      bPending = 1;
      issueATile(sc, gs, As0 + (buf ^ 1) * kBM * gs.K3, Tn.z, Tn.w, tid, &aBar[buf ^ 1]);
      aPending |= 1u << (buf ^ 1);
    }
    t = tn;
    ce = ceN;
  }
  cpAsyncWaitAll();
  if (failed) {
    // give the in-flight MMA chain a second bounded chance to retire (same
    // completion parity) before the TMEM is freed, and the TMA loads in
    // flight one before the shared memory is released
    mbarWait(mbar, phase);
    for (int b = 0; b < 2; ++b)
      if (aPending & (1u << b)) mbarWait(&aBar[b], (aParity >> b) & 1u);
    if (bPending) mbarWait(bBar, bParity);
  }
  __syncthreads();
  tcFenceAfter();
  if (warp == 0) tmemDealloc(tmem, (uint32_t)tmemCols);
}

// ---------------------------------------------------- FP64 RHS (mixed)

// b_e[i] = sum_q w det conj(phi_i) f(x_q)  (LinearTerm::evaluate), warp per element
__global__ void k_rhs_fp64(const PlanDev p, const DevTerms *__restrict__ terms, double2 *__restrict__ be) {
  const int lane = threadIdx.x & 31;
  const int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (e >= p.E) return;
  const int o = p.orient ? p.orient[e] : 0;
  double X[kMaxNodes * 3];
  for (int k = 0; k < p.nn; ++k)
    for (int c = 0; c < 3; ++c) X[3 * k + c] = p.xyz[3 * (int64_t)p.enodes[e * p.nn + k] + c];
  double2 acc[2] = {make_double2(0, 0), make_double2(0, 0)};
  for (int q = 0; q < p.nq; ++q) {
    double2 s = make_double2(0.0, 0.0);
    if (lane == 0) {
      double J[9];
      const double det = jacobian(p.dim, p.nn, X, p.geoGrad + (size_t)q * p.nn * 3, J);
      double xq[3] = {0, 0, 0};
      for (int k = 0; k < p.nn; ++k)
        for (int c = 0; c < 3; ++c) xq[c] += p.geoVal[q * p.nn + k] * X[3 * k + c];
      double2 f = make_double2(0.0, 0.0);
      for (int t = 0; t < terms->n; ++t)
        if (terms->t[t].kind == FG_TERM_SOURCE)
          f = cadd(f, evalExpr(terms->t[t].coef, e, xq, p.bval + ((size_t)o * p.nq + q) * p.nb, p.nb, q, p.nq));
      s = make_double2(p.w[q] * det * f.x, p.w[q] * det * f.y);
    }
    s.x = __shfl_sync(0xffffffffu, s.x, 0);
    s.y = __shfl_sync(0xffffffffu, s.y, 0);
    const size_t base = ((size_t)o * p.nq + q) * p.nb;
    for (int i = lane; i < p.nb; i += 32) {
      const double ph = p.bval[base + i];
      acc[i >> 5].x += s.x * ph;
      acc[i >> 5].y += s.y * ph;
    }
  }
  for (int i = lane; i < p.nb; i += 32) be[(size_t)e * p.nb + i] = acc[i >> 5];
}

// -------------------------------------------- error report (device side)

// per element ||Ke32 - Ke64||_F^2 and ||Ke64||_F^2; the FP64 matrices are
// row-major [ncomp][n][n], the FP32 ones [ncomp][lay.ld] in the layout lay
__global__ void k_elem_err(const float *__restrict__ k32, const double *__restrict__ k64, int64_t E, int ncomp, int n, KeLayout lay,
                           double *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= E) return;
  const int nn = n * n, len = ncomp * nn;
  double d2 = 0.0, r2 = 0.0;
  for (int k = lane; k < len; k += 32) {
    const int comp = k / nn, r = k - comp * nn, ii = r / n, jj = r - ii * n;
    const int o32 = comp * lay.ld + keOffset(lay, n, ii, jj);
    const double a = k64[(size_t)e * len + k];
    const double d = (double)k32[(size_t)e * ncomp * lay.ld + o32] - a;
    d2 += d * d;
    r2 += a * a;
  }
  for (int off = 16; off > 0; off >>= 1) {
    d2 += __shfl_down_sync(0xffffffffu, d2, off);
    r2 += __shfl_down_sync(0xffffffffu, r2, off);
  }
  if (lane == 0) {
    out[2 * e] = d2;
    out[2 * e + 1] = r2;
  }
}

__global__ void k_diff_norms(const double *__restrict__ a, const double *__restrict__ b, int64_t n, double *__restrict__ out) {
  double d2 = 0.0, r2 = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = a[i] - b[i];
    d2 += d * d;
    r2 += b[i] * b[i];
  }
  __shared__ double s[2][32];
  for (int off = 16; off > 0; off >>= 1) {
    d2 += __shfl_down_sync(0xffffffffu, d2, off);
    r2 += __shfl_down_sync(0xffffffffu, r2, off);
  }
  if ((threadIdx.x & 31) == 0) {
    s[0][threadIdx.x >> 5] = d2;
    s[1][threadIdx.x >> 5] = r2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0, y = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      x += s[0][w];
      y += s[1][w];
    }
    out[2 * blockIdx.x] = x;
    out[2 * blockIdx.x + 1] = y;
  }
}

// --------------------------------------------------------------- host

static MixedState *state(fg_plan *plan) {
  if (!plan->mixed) plan->mixed = new MixedState();
  return (MixedState *)plan->mixed;
}

// reference tensors T^o (FP64 on the host from the plan's basis tables), split
// and laid out as the B' shared-memory image: row r (= i*nb + j) of B' holds
// its K' = 3*kp values; core matrix (r/8, kc) at kc * (Npad*16) + (r/8)*128,
// row r%8 at +16*(r%8).
//  scalar field (kp = 8):  T[ab] = sum_q w (d_a phi_j d_b phi_i + [a != b] d_b phi_j d_a phi_i)
//                          for ab = 00,11,22,01,02,12, T[6] = sum_q w phi_i phi_j
//  compound field (kp = 16): T[3p+p'] = sum_q w d_p phi_j d_p' phi_i, T[9] = sum_q w phi_i phi_j
//  HCurl field (kp = 16):    T[ab] as the scalar field's with the reference curls c,
//                            T[6 + ab] the same with the reference vector values v
// compact: K' = 2 kp, [B_hi ; B_lo] (the fused kernel's image; its third
// product reads B_hi again)
void buildB(const PlanDev &p, const std::vector<double> &w, const std::vector<double> &bval, const std::vector<double> &bgrad,
            int o, int Npad, int kp, std::vector<float> &img, bool compact) {
  const int nb = p.nb, nq = p.nq, k3 = (compact ? 2 : 3) * kp;
  img.assign((size_t)Npad * k3, 0.0f);
  const int ab[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  std::vector<double> T(kp);
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j < nb; ++j) {
      std::fill(T.begin(), T.end(), 0.0);
      for (int q = 0; q < nq; ++q) {
        const double *gi = &bgrad[(((size_t)o * nq + q) * nb + i) * 3];
        const double *gj = &bgrad[(((size_t)o * nq + q) * nb + j) * 3];
        if (p.form == FG_FORM_1) {
          const double *vi = &bval[(((size_t)o * nq + q) * nb + i) * 3];
          const double *vj = &bval[(((size_t)o * nq + q) * nb + j) * 3];
          for (int k = 0; k < 6; ++k) {
            const int a = ab[k][0], b = ab[k][1];
            T[k] += w[q] * (gj[a] * gi[b] + (a != b ? gj[b] * gi[a] : 0.0));
            T[6 + k] += w[q] * (vj[a] * vi[b] + (a != b ? vj[b] * vi[a] : 0.0));
          }
          continue;
        }
        const double mass = w[q] * bval[((size_t)o * nq + q) * nb + i] * bval[((size_t)o * nq + q) * nb + j];
        if (kp == kKp) {
          for (int k = 0; k < 6; ++k) {
            const int a = ab[k][0], b = ab[k][1];
            T[k] += w[q] * (gj[a] * gi[b] + (a != b ? gj[b] * gi[a] : 0.0));
          }
          T[6] += mass;
        } else {
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) T[3 * a + b] += w[q] * gj[a] * gi[b];
          T[9] += mass;
        }
      }
      const int row = i * nb + j;
      for (int k = 0; k < kp; ++k) {
        float hi, lo;
        splitTf32(T[k], hi, lo);
        const float vals[3] = {hi, compact ? lo : hi, lo};  // K' blocks: [B_hi ; B_hi ; B_lo] or [B_hi ; B_lo]
        for (int blk = 0; blk < (compact ? 2 : 3); ++blk) {
          const int kk = blk * kp + k;
          const int kc = kk >> 2, within = kk & 3;
          const size_t off = (size_t)kc * (Npad * 4) + (size_t)(row >> 3) * 32 + (row & 7) * 4 + within;  // in floats
          img[off] = vals[blk];
        }
      }
    }
}

static size_t gemmSmemNeed(int Npad, int k3) { return 128 + 8 * 32 * 36 * 4 + 2 * (size_t)kBM * k3 * 4 + (size_t)Npad * k3 * 4; }
// TMA tensor map of the factor rows A [rows][k3] (floats, 16-byte rows
// pieces): box {4 floats, 128 rows}, no swizzle, zero fill past the rows,
// so one box lands at As + kc * 2048 with row r at 16 r, the K-major
// core-matrix layout of the MMA descriptors.
static int encodeRowsMap(CUtensorMap *map, const float *A, int k3, int64_t rows) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      cudaGetLastError();
      setLastError("mixed path: cuTensorMapEncodeTiled not available");
      return FG_ERR_CUDA;
    }
    encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)k3, (cuuint64_t)std::max<int64_t>(rows, 1)};
  const cuuint64_t strides[1] = {(cuuint64_t)k3 * 4};
  const cuuint32_t box[2] = {4, (cuuint32_t)kBM};
  const cuuint32_t elemStrides[2] = {1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(A), dims, strides, box, elemStrides,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    setLastError("mixed path: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return FG_ERR_CUDA;
  }
  return FG_OK;
}

int gemmCtasPerSm(int Npad, int k3) { return gemmSmemNeed(Npad, k3) <= 110 * 1024 ? 2 : 1; }
size_t gemmSmem(int Npad, int k3, int ctasPerSm) {
  // one CTA per SM takes at least half the SM's shared memory and all 512
  // TMEM columns; two take at least a third each and 256 columns each. No
  // CTA ever waits in tcgen05.alloc for another one's columns.
  return std::max<size_t>(gemmSmemNeed(Npad, k3), ctasPerSm == 2 ? 80 * 1024 : 116 * 1024);
}

// Contiguous tile ranges for nCta persistent CTAs with about equal summed cost
std::vector<int32_t> partitionTiles(const std::vector<double> &cost, int nCta) {
  std::vector<int32_t> start((size_t)nCta + 1, (int32_t)cost.size());
  double total = 0.0;
  for (double c : cost) total += c;
  double acc = 0.0;
  int b = 0;
  start[0] = 0;
  for (size_t t = 0; t < cost.size() && b + 1 < nCta; ++t) {
    acc += cost[t];
    while (b + 1 < nCta && acc >= total * (b + 1) / nCta) start[++b] = (int32_t)(t + 1);
  }
  for (int k = b + 1; k <= nCta; ++k) start[k] = (int32_t)cost.size();
  return start;
}

// Bound of the contraction's wait for each MMA chain, in SM cycles
// (fg_set_wait_limit). After it runs out the kernel records a timeout, waits
// once more with the fixed bound for the chain it issued, frees its TMEM and
// returns.
static std::atomic<long long> g_mmaWaitCycles{kWaitCycles};

// One contraction launch over the tiles of one or many problems
int launchContract(const void *probsDev, const int4 *tilesDev, const int32_t *ctaStartDev, int nCta, int *err, int maxK3,
                   size_t smem, cudaStream_t s, int tmemCols, const void *aMap, int *next, int nTiles, int chunk) {
  static SmemAllowance allowed;
  FG_CUDA(allowSmem(k_contract_tf32x3, smem, allowed));
  GemmSched sc;
  std::memset(&sc, 0, sizeof(sc));
  if (aMap) {
    std::memcpy(&sc.aMap, aMap, sizeof(CUtensorMap));
    sc.tma = 1;
  }
  sc.probs = (const GemmProblem *)probsDev;
  sc.tiles = tilesDev;
  sc.ctaStart = ctaStartDev;
  sc.err = err;
  sc.mmaWaitCycles = g_mmaWaitCycles.load();
  if (next) {
    FG_CUDA(cudaMemsetAsync(next, 0, sizeof(int), s));
    sc.next = next;
    sc.nTiles = nTiles;
    sc.chunk = std::max(1, chunk);
  }
  ProfScope prof("k_contract_tf32x3", s);
  k_contract_tf32x3<<<std::max(1, nCta), kThreadsGemm, smem, s>>>(sc, maxK3, tmemCols);
  countLaunch();
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

// GEMM tiles of a plan (problem index `prob` of a launch): 128 rows of one
// orientation each, rows = element rank * rowsPerElem + row within element
std::vector<int4> mixedTiles(fg_plan *plan, int prob, int rowsPerElem) {
  MixedState *m = state(plan);
  std::vector<int4> tiles;
  int64_t start = 0;
  for (int o = 0; o < plan->d.nOrient; ++o) {
    const int64_t r0 = start * rowsPerElem, r1 = (start + m->orientCount[o]) * rowsPerElem;
    for (int64_t r = r0; r < r1; r += kBM) tiles.push_back(make_int4(prob, o, (int)r, (int)std::min<int64_t>(kBM, r1 - r)));
    start += m->orientCount[o];
  }
  return tiles;
}

GemmProblem mixedGemmProblem(fg_plan *plan) {
  MixedState *m = state(plan);
  GemmProblem g;
  std::memset(&g, 0, sizeof(g));
  g.A = m->A;
  g.B = m->B;
  g.perm = m->perm;
  g.ke = m->ke;
  g.Npad = m->Npad;
  g.nn2 = m->nn2;
  g.ld = m->ld;
  g.rowsPerElem = m->rowsPerElem;
  g.K3 = m->k3;
  g.mmaN = std::min(m->mmaN, std::min(m->Npad, 256));
  return g;
}

// Tables, tiles and buffers for element matrices of `groups` term groups
// (one per frequency factor of the multi-frequency path; 1 otherwise), each
// with ncomp (1 real, 2 complex) parts.
int prepareMixed(fg_plan *plan, int ncomp, int groups) {
  MixedState *m = state(plan);
  const PlanDev &p = plan->d;
  if (m->built && m->ncomp == ncomp && m->groups == groups) return FG_OK;
  if (!m->built) {
    if (p.mult != 1 && p.mult != 3) {
      setLastError("mixed path: fields of 1 or 3 components only");
      return FG_ERR_UNSUPPORTED;
    }
    if (!p.affine) {
      setLastError("mixed path: needs geometrically affine (straight-sided) elements");
      return FG_ERR_UNSUPPORTED;
    }
    m->blocks = p.mult == 3 ? 9 : 1;
    m->kp = (p.mult == 3 || p.form == FG_FORM_1) ? kKpE : kKp;
    m->k3 = 3 * m->kp;
    m->n = p.n;
    m->nn2 = p.nb * p.nb;  // one (block of the) element matrix per GEMM row
    m->Npad = (m->nn2 + 15) / 16 * 16;
    m->ld = (m->blocks == 1 && m->nn2 % 4 != 0) ? (m->nn2 + 7) / 8 * 8 : m->nn2;
    m->nOrient = p.nOrient;
    if (gemmSmem(m->Npad, m->k3) > 220 * 1024) {
      setLastError("mixed path: element matrix too large for the shared-memory B tile");
      return FG_ERR_UNSUPPORTED;
    }
    // tables back to the host
    std::vector<double> w(p.nq), bval((size_t)p.nOrient * p.nq * p.nb * (p.form == FG_FORM_1 ? 3 : 1)),
        bgrad((size_t)p.nOrient * p.nq * p.nb * 3);
    FG_CUDA(cudaMemcpy(w.data(), p.w, w.size() * 8, cudaMemcpyDeviceToHost));
    FG_CUDA(cudaMemcpy(bval.data(), p.bval, bval.size() * 8, cudaMemcpyDeviceToHost));
    FG_CUDA(cudaMemcpy(bgrad.data(), p.bgrad, bgrad.size() * 8, cudaMemcpyDeviceToHost));
    std::vector<float> all((size_t)p.nOrient * m->Npad * m->k3), img;
    for (int o = 0; o < p.nOrient; ++o) {
      buildB(p, w, bval, bgrad, o, m->Npad, m->kp, img, false);
      std::copy(img.begin(), img.end(), all.begin() + (size_t)o * m->Npad * m->k3);
    }
    FG_CUDA(cudaMalloc(&m->B, all.size() * 4));
    FG_CUDA(cudaMemcpy(m->B, all.data(), all.size() * 4, cudaMemcpyHostToDevice));
    // elements sorted by orientation (stable)
    std::vector<int32_t> orient((size_t)p.E, 0);
    if (p.orient) FG_CUDA(cudaMemcpy(orient.data(), p.orient, (size_t)p.E * 4, cudaMemcpyDeviceToHost));
    std::vector<int32_t> perm((size_t)p.E);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int32_t a, int32_t b) { return orient[a] < orient[b]; });
    std::vector<int32_t> rank((size_t)p.E);
    for (int64_t r = 0; r < p.E; ++r) rank[perm[r]] = (int32_t)r;
    m->orientCount.assign(p.nOrient, 0);
    for (int64_t e = 0; e < p.E; ++e) m->orientCount[orient[e]]++;
    FG_CUDA(cudaMalloc(&m->perm, (size_t)p.E * 4 * 2));
    FG_CUDA(cudaMemcpy(m->perm, perm.data(), (size_t)p.E * 4, cudaMemcpyHostToDevice));
    FG_CUDA(cudaMemcpy(m->perm + p.E, rank.data(), (size_t)p.E * 4, cudaMemcpyHostToDevice));
    FG_CUDA(cudaMalloc(&m->err, sizeof(int)));
    FG_CUDA(cudaMallocHost(&m->errHost, sizeof(int)));
    *m->errHost = 0;
    FG_CUDA(cudaEventCreateWithFlags(&m->errEvent, cudaEventDisableTiming));
    FG_CUDA(cudaMemset(m->err, 0, sizeof(int)));
    m->built = 1;
  }
  // tiles: rows of one orientation never share a tile
  const int rowsPerElem = groups * ncomp * m->blocks;
  if ((int64_t)p.E * rowsPerElem >= (int64_t(1) << 31)) {
    setLastError("mixed path: more than 2^31 GEMM rows in one plan");
    return FG_ERR_UNSUPPORTED;
  }
  std::vector<int4> tiles = mixedTiles(plan, 0, rowsPerElem);
  m->nTiles = (int)tiles.size();
  m->ctasPerSm = gemmCtasPerSm(m->Npad, m->k3);
  m->nCta = std::max(1, std::min(m->ctasPerSm * smCount(), m->nTiles));
  std::vector<int32_t> start = partitionTiles(std::vector<double>(tiles.size(), 1.0), m->nCta);
  if (m->tiles) cudaFree(m->tiles);
  if (m->ctaStart) cudaFree(m->ctaStart);
  m->tiles = nullptr;
  m->ctaStart = nullptr;
  FG_CUDA(cudaMalloc(&m->tiles, std::max<size_t>(tiles.size(), 1) * sizeof(int4)));
  if (!tiles.empty()) FG_CUDA(cudaMemcpy(m->tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMalloc(&m->ctaStart, start.size() * 4));
  FG_CUDA(cudaMemcpy(m->ctaStart, start.data(), start.size() * 4, cudaMemcpyHostToDevice));
  m->rowsPerElem = rowsPerElem;
  m->rows = p.E * rowsPerElem;
  int st = ensureDevice((void **)&m->A, &m->Abytes, (size_t)m->rows * m->k3 * 4);
  if (st) return st;
  if ((st = encodeRowsMap(&m->aMap, m->A, m->k3, m->rows))) return st;
  st = ensureDevice((void **)&m->ke, &m->keBytes, (size_t)m->rows * m->ld * 4);
  if (st) return st;
  m->ncomp = ncomp;
  m->groups = groups;
  GemmProblem gp = mixedGemmProblem(plan);
  if (!m->probDev) FG_CUDA(cudaMalloc(&m->probDev, sizeof(GemmProblem)));
  FG_CUDA(cudaMemcpy(m->probDev, &gp, sizeof(GemmProblem), cudaMemcpyHostToDevice));
  return FG_OK;
}

// Factor rows of every term group (group g: rows g * ncomp * blocks onwards
// within an element), then one tensor-core contraction over all of them into
// m->ke ([E][groups][ncomp][n][n]).
int launchMixedElement(fg_plan *plan, const DevTerms *const *dterms, int groups, uint32_t tensorMask, cudaStream_t s) {
  MixedState *m = state(plan);
  const PlanDev &p = plan->d;
  const int ncomp = m->ncomp;
  for (int gi = 0; gi < groups; ++gi) {
    ProfScope prof("k_factors", s);
    const int off = gi * ncomp * m->blocks;
    if (p.form == FG_FORM_1)
      k_factors_hcurl<<<(unsigned)((p.E + 127) / 128), 128, 0, s>>>(p, dterms[gi], m->perm + p.E, m->A, ncomp, m->rowsPerElem, off);
    else if (m->blocks == 9)
      k_factors_elastic<<<(unsigned)((p.E + 127) / 128), 128, 0, s>>>(p, dterms[gi], m->perm + p.E, m->A, ncomp, m->rowsPerElem, off);
    else if (tensorMask >> gi & 1)
      k_factors<true><<<(unsigned)((p.E + 127) / 128), 128, 0, s>>>(p, dterms[gi], m->perm + p.E, m->A, ncomp, m->rowsPerElem, off);
    else k_factors<false><<<(unsigned)((p.E + 127) / 128), 128, 0, s>>>(p, dterms[gi], m->perm + p.E, m->A, ncomp, m->rowsPerElem, off);
    countLaunch();
    FG_CUDA(cudaGetLastError());
  }
  if (m->nTiles == 0) return FG_OK;
  return launchContract(m->probDev, m->tiles, m->ctaStart, m->nCta, m->err, m->k3, gemmSmem(m->Npad, m->k3, m->ctasPerSm), s,
                        512 / m->ctasPerSm, &m->aMap);
}

int launchFactorsBatch(const FactorJob *jobsDev, int nJobs, int64_t total, cudaStream_t s) {
  if (total <= 0) return FG_OK;
  ProfScope prof("k_factors_batch", s);
  k_factors_batch<<<(unsigned)((total + 127) / 128), 128, 0, s>>>(jobsDev, nJobs, total);
  countLaunch();
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

// This plan's factor job (terms on the device, group 0)
FactorJob mixedFactorJob(fg_plan *plan, const DevTerms *dterms, bool tensor, int64_t elemStart) {
  MixedState *m = state(plan);
  FactorJob j;
  std::memset(&j, 0, sizeof(j));
  j.p = plan->d;
  j.terms = dterms;
  j.rankOf = m->perm + plan->d.E;
  j.A = m->A;
  j.ncomp = m->ncomp;
  j.rowsPerElem = m->rowsPerElem;
  j.rowOff = 0;
  j.kind = plan->d.form == FG_FORM_1 ? 2 : (m->blocks == 9 ? 1 : (tensor ? 3 : 0));
  j.elemStart = elemStart;
  return j;
}

// FP64 element right-hand sides of the source terms into be ([E][n] complex)
int launchRhsFp64(fg_plan *plan, const DevTerms *dterms, double *be, cudaStream_t s) {
  const PlanDev &p = plan->d;
  if (p.E == 0) return FG_OK;
  ProfScope prof("k_rhs_fp64", s);
  const int64_t threads = p.E * 32;
  k_rhs_fp64<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(p, dterms, (double2 *)be);
  countLaunch();
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

// Accessors for the multi-frequency path
float *mixedKe(fg_plan *plan, KeLayout *lay) {
  MixedState *m = state(plan);
  *lay = mixedLayout(m);
  return m->ke;
}

// Reports a wait timeout of an earlier call (wait == false) or of this one
// (wait == true, after the outputs were copied back).
int mixedCheckTimeout(fg_plan *plan, bool wait) { return checkTimeout(state(plan), wait); }

// Queues the copy of the device error word behind this call's launches.
int mixedRecordError(fg_plan *plan, cudaStream_t s) {
  MixedState *m = state(plan);
  FG_CUDA(cudaMemcpyAsync(m->errHost, m->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaEventRecord(m->errEvent, s));
  m->errPending = true;
  return FG_OK;
}

}  // namespace femg

using namespace femg;

extern "C" int fg_set_wait_limit(double seconds) {
  if (!(seconds >= 0.0) || seconds > 60.0) {
    femg::setLastError("fg_set_wait_limit: seconds must be in [0, 60]");
    return FG_ERR_ARG;
  }
  // clock64 counts SM cycles: at most 2.07 GHz on GB300, so the bound lasts at
  // least `seconds` of wall time
  g_mmaWaitCycles.store((long long)(seconds * 2.07e9));
  return FG_OK;
}

extern "C" void mixedDestroy(fg_plan *plan) {
  MixedState *m = (MixedState *)plan->mixed;
  if (!m) return;
  cudaFree(m->A);
  cudaFree(m->B);
  cudaFree(m->perm);
  cudaFree(m->tiles);
  cudaFree(m->ctaStart);
  cudaFree(m->probDev);
  cudaFree(m->ke);
  cudaFree(m->err);
  if (m->errHost) cudaFreeHost(m->errHost);
  if (m->errEvent) cudaEventDestroy(m->errEvent);
  delete m;
  plan->mixed = nullptr;
}

extern "C" int fg_assemble_mixed(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, double frequency, const double *dirichlet,
                                 double *csr_values, double *rhs, void *stream, fg_err_report *report) {
  if (!plan) return FG_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  DevTerms dt;
  const DevTerms *dterms = nullptr;
  int st = resolveTerms(plan, terms, n_terms, frequency, &dt, &dterms, s);
  if (st) return st;
  for (int t = 0; t < dt.n; ++t)
    if ((dt.t[t].kind != FG_TERM_SOURCE && dt.t[t].coef.cls == kExprPoint) || dt.tensorPoint) {
      setLastError("mixed path: bilinear coefficients must be constant per element");
      return FG_ERR_UNSUPPORTED;
    }
  if (dt.hasJacMod) {
    setLastError("mixed path: Jacobian modificators make the geometry point-dependent; use the FP64 path");
    return FG_ERR_UNSUPPORTED;
  }
  if (plan->d.coupled) {
    setLastError("mixed path: two-field plans run on the FP64 path");
    return FG_ERR_UNSUPPORTED;
  }
  if (dt.nonSym) {
    setLastError("mixed path: the full-tensor and advection terms run on the FP64 path");
    return FG_ERR_UNSUPPORTED;
  }
  if (report && plan->accumulate) {
    setLastError("mixed path: the error report compares overwritten values; the plan accumulates");
    return FG_ERR_ARG;
  }
  if (!report && fusedApplies(plan, dt)) {
    // contraction and reduction in one kernel: no element matrix in HBM
    const double *uD0 = nullptr;
    if ((st = uploadDirichlet(plan, dirichlet, &uD0, s))) return st;
    Outputs o;
    if ((st = prepareOutputs(plan, csr_values, rhs, &o))) return st;
    const PlanDev &p = plan->d;
    double *be = nullptr;
    if (dt.hasSource && rhs) {
      if ((st = ensureDevice((void **)&plan->be, &plan->beBytes, (size_t)p.E * p.n * 16))) return st;
      be = plan->be;
      if ((st = launchRhsFp64(plan, dterms, be, s))) return st;
    }
    if ((st = launchFused(plan, dt, dterms, (const double2 *)be, (double2 *)o.values, (double2 *)o.rhs, s))) return st;
    if ((st = finishOutputs(plan, o, csr_values, rhs, s))) return st;
    if (o.hostValues || (rhs && o.hostRhs)) return fusedTimeout(plan, true);
    return FG_OK;
  }
  if ((st = prepareMixed(plan, dt.complexKe ? 2 : 1, 1))) return st;
  if ((st = checkTimeout(state(plan), false))) return st;  // a timeout of an earlier call
  const double *uD = nullptr;
  if ((st = uploadDirichlet(plan, dirichlet, &uD, s))) return st;
  Outputs o;
  if ((st = prepareOutputs(plan, csr_values, rhs, &o))) return st;
  const PlanDev &p = plan->d;
  MixedState *m = state(plan);
  double *be = nullptr;
  if (dt.hasSource && rhs) {
    if ((st = ensureDevice((void **)&plan->be, &plan->beBytes, (size_t)p.E * p.n * 16))) return st;
    be = plan->be;
    ProfScope prof("k_rhs_fp64", s);
    const int64_t threads = p.E * 32;
    k_rhs_fp64<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(p, dterms, (double2 *)be);
    countLaunch();
    FG_CUDA(cudaGetLastError());
  }
  if (p.E > 0)
    if ((st = launchMixedElement(plan, &dterms, 1, dt.tensorTerm >= 0 ? 1u : 0u, s))) return st;
  if ((st = gatherToOutputs(plan, (const double *)m->ke, dt.complexKe, 1, mixedLayout(m), be, uD, o, csr_values, s))) return st;
  if (report) {
    // FP64 element matrices and CSR of the same terms, compared on the device
    const int ncomp = dt.complexKe ? 2 : 1;
    const size_t len = (size_t)ncomp * p.n * p.n;
    if ((st = ensureDevice((void **)&plan->ke, &plan->keBytes, (size_t)p.E * len * 8))) return st;
    if ((st = launchElementFp64(plan, dt, dterms, plan->ke, nullptr, s))) return st;
    double *tmp = nullptr, *csr64 = nullptr;
    FG_CUDA(cudaMalloc(&tmp, (size_t)std::max<int64_t>(p.E, 1024) * 16));
    FG_CUDA(cudaMalloc(&csr64, p.nnz * 16));
    k_elem_err<<<(unsigned)((p.E + 7) / 8), 256, 0, s>>>(m->ke, plan->ke, p.E, ncomp, p.n, mixedLayout(m), tmp);
    std::vector<double> h((size_t)p.E * 2);
    FG_CUDA(cudaMemcpyAsync(h.data(), tmp, h.size() * 8, cudaMemcpyDeviceToHost, s));
    if ((st = launchGather(plan, plan->ke, dt.complexKe, 0, keFull(p.n), nullptr, uD, csr64, nullptr, s))) return st;
    k_diff_norms<<<1024, 256, 0, s>>>(o.values, csr64, (int64_t)p.nnz * 2, tmp);
    std::vector<double> g(2048);
    FG_CUDA(cudaMemcpyAsync(g.data(), tmp, g.size() * 8, cudaMemcpyDeviceToHost, s));
    FG_CUDA(cudaStreamSynchronize(s));
    countLaunch(2);
    double mx = 0.0, sum = 0.0;
    for (int64_t e = 0; e < p.E; ++e) {
      const double r = h[2 * e + 1] > 0 ? std::sqrt(h[2 * e] / h[2 * e + 1]) : 0.0;
      mx = std::max(mx, r);
      sum += r;
    }
    double d2 = 0, r2 = 0;
    for (int b = 0; b < 1024; ++b) {
      d2 += g[2 * b];
      r2 += g[2 * b + 1];
    }
    report->max_elem_rel_fro = mx;
    report->mean_elem_rel_fro = p.E ? sum / p.E : 0.0;
    report->global_rel_fro = r2 > 0 ? std::sqrt(d2 / r2) : 0.0;
    cudaFree(tmp);
    cudaFree(csr64);
  }
  // the device error word comes back asynchronously: host outputs synchronize
  // below and report it now; with device outputs the next call reports it
  FG_CUDA(cudaMemcpyAsync(m->errHost, m->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaEventRecord(m->errEvent, s));
  m->errPending = true;
  if ((st = finishOutputs(plan, o, csr_values, rhs, s))) return st;
  if (o.hostValues || (rhs && o.hostRhs)) return checkTimeout(m, true);
  return FG_OK;
}


