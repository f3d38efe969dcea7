// FP64 element matrices by factorization, on the CUDA cores.
//
// For affine elements with element-constant bilinear coefficients the
// quadrature sum of BilinearTerm::evaluate (src/term/BilinearTerm.cpp:304-343)
// factors exactly into per-element factors and per-orientation reference
// tensors (the same identity the tensor-core path uses):
//   scalar H1:  Ke[i][j] = sum_ab c det K_ab T_ab[i][j] + c_m det M[i][j],  K = J^-1 J^-T,
//   HCurl:      Ke[i][j] = sum_ab (c / det) (J^T J)_ab Tc_ab[i][j] + c_m det K_ab Tv_ab[i][j],
// with T summed over the quadrature points in FP64 once per orientation. All
// arithmetic stays FP64, but GB300's narrow FP64 pipe does 2 kp FLOPs per
// entry (kp = 7 or 12) instead of about 8 nq: 17x fewer for order 3 with
// Gauss6. Selected per plan (FG_FP64_FACTORED); the plain method is the
// quadrature loop. Curved elements, point-dependent coefficients and compound
// fields keep the quadrature kernels.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace femg {

constexpr int kFacTile = 64;  // elements per tile (one orientation)
constexpr int kFacMax = 12;   // factors per element row

struct FactoredState {
  int built = 0;
  int kp = 0;        // factors: 7 (scalar H1) or 12 (HCurl)
  double *T = nullptr;       // [nOrient][kp][n*n] reference tensors
  int32_t *perm = nullptr;   // rank -> element, ranks sorted by orientation
  int4 *tiles = nullptr;     // (orientation, first rank, count, -)
  int nTiles = 0;
};

// per-element factors (FP64) of one coefficient component
__device__ inline void elementFactors(const PlanDev &p, const DevTerms *__restrict__ terms, int64_t e, int comp, double *d) {
  double X[kMaxNodes * 3];
  const int nx = p.p1geom ? p.dim + 1 : p.nn;
  for (int k = 0; k < nx; ++k)
    for (int c = 0; c < 3; ++c) X[3 * k + c] = p.xyz[3 * (int64_t)p.enodes[e * p.nn + k] + c];
  double J[9], Ji[9];
  const double det = p.p1geom ? jacobianP1(p.dim, X, J) : jacobian(p.dim, p.nn, X, p.geoGrad, J);
  jacobianInverse(J, det, Ji);
  const int ab[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  double xc[3] = {0.0, 0.0, 0.0};
  double2 cg = make_double2(0.0, 0.0), cm = make_double2(0.0, 0.0);
  for (int t = 0; t < terms->n; ++t) {
    const DevTerm &T = terms->t[t];
    if (T.kind == FG_TERM_GRAD_GRAD) cg = cadd(cg, cmul(T.factor, evalExpr(T.coef, e, xc)));
    else if (T.kind == FG_TERM_MASS) cm = cadd(cm, cmul(T.factor, evalExpr(T.coef, e, xc)));
  }
  const double g = comp == 0 ? cg.x : cg.y, m = comp == 0 ? cm.x : cm.y;
  for (int k = 0; k < 6; ++k) {
    const int a = ab[k][0], b = ab[k][1];
    const double K = Ji[3 * a] * Ji[3 * b] + Ji[3 * a + 1] * Ji[3 * b + 1] + Ji[3 * a + 2] * Ji[3 * b + 2];
    if (p.form == FG_FORM_1) {
      const double M = J[3 * a] * J[3 * b] + J[3 * a + 1] * J[3 * b + 1] + J[3 * a + 2] * J[3 * b + 2];
      d[k] = g / det * M;
      d[6 + k] = m * det * K;
    } else {
      d[k] = g * det * K;
    }
  }
  if (p.form != FG_FORM_1) d[6] = m * det;
}

// One tile of elements of one orientation per block: factors into shared
// memory, the orientation's reference tensors into shared memory, then the
// entries of all element matrices of the tile, consecutive threads on
// consecutive entries of a row (coalesced 8-byte stores).
template <bool CPLX>
__global__ void __launch_bounds__(256) k_element_factored_fp64(const PlanDev p, const DevTerms *__restrict__ terms,
                                                               const double *__restrict__ T, const int32_t *__restrict__ perm,
                                                               const int4 *__restrict__ tiles, int kp, double *__restrict__ ke) {
  extern __shared__ double fsm[];
  const int nn2 = p.n * p.n;
  double *Ts = fsm;                          // [kp][nn2]
  double *F = fsm + (size_t)kp * nn2;         // [kFacTile][2][kFacMax]
  const int4 tile = tiles[blockIdx.x];
  const double *To = T + (size_t)tile.x * kp * nn2;
  for (int k = threadIdx.x; k < kp * nn2; k += blockDim.x) Ts[k] = To[k];
  if (threadIdx.x < tile.z) {
    const int64_t e = perm[tile.y + threadIdx.x];
    elementFactors(p, terms, e, 0, F + (size_t)threadIdx.x * 2 * kFacMax);
    if (CPLX) elementFactors(p, terms, e, 1, F + (size_t)threadIdx.x * 2 * kFacMax + kFacMax);
  }
  __syncthreads();
  const int ncomp = CPLX ? 2 : 1;
  const int total = tile.z * nn2;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int r = idx / nn2, c = idx - r * nn2;
    const double *fr = F + (size_t)r * 2 * kFacMax;
    double re = 0.0, im = 0.0;
    for (int k = 0; k < kp; ++k) {
      const double t = Ts[(size_t)k * nn2 + c];
      re = fma(fr[k], t, re);
      if (CPLX) im = fma(fr[kFacMax + k], t, im);
    }
    double *out = ke + (size_t)perm[tile.y + r] * ncomp * nn2;
    out[c] = re;
    if (CPLX) out[nn2 + c] = im;
  }
}

static FactoredState *factoredState(fg_plan *plan) {
  if (!plan->fp64f) plan->fp64f = new FactoredState();
  return (FactoredState *)plan->fp64f;
}

// Reference tensors per orientation (FP64) and the orientation-sorted tiles.
static int prepareFactored(fg_plan *plan) {
  FactoredState *f = factoredState(plan);
  if (f->built) return FG_OK;
  const PlanDev &p = plan->d;
  const int nb = p.nb, nq = p.nq, n2 = nb * nb;
  const bool hc = p.form == FG_FORM_1;
  f->kp = hc ? 12 : 7;
  std::vector<double> w(nq), bval((size_t)p.nOrient * nq * nb * (hc ? 3 : 1)), bgrad((size_t)p.nOrient * nq * nb * 3);
  FG_CUDA(cudaMemcpy(w.data(), p.w, w.size() * 8, cudaMemcpyDeviceToHost));
  FG_CUDA(cudaMemcpy(bval.data(), p.bval, bval.size() * 8, cudaMemcpyDeviceToHost));
  FG_CUDA(cudaMemcpy(bgrad.data(), p.bgrad, bgrad.size() * 8, cudaMemcpyDeviceToHost));
  const int ab[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  std::vector<double> T((size_t)p.nOrient * f->kp * n2, 0.0);
  for (int o = 0; o < p.nOrient; ++o)
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < nb; ++j) {
        double *t = &T[(size_t)o * f->kp * n2 + (size_t)i * nb + j];
        for (int q = 0; q < nq; ++q) {
          const double *gi = &bgrad[(((size_t)o * nq + q) * nb + i) * 3], *gj = &bgrad[(((size_t)o * nq + q) * nb + j) * 3];
          for (int k = 0; k < 6; ++k) {
            const int a = ab[k][0], b = ab[k][1];
            t[(size_t)k * n2] += w[q] * (gj[a] * gi[b] + (a != b ? gj[b] * gi[a] : 0.0));
          }
          if (hc) {
            const double *vi = &bval[(((size_t)o * nq + q) * nb + i) * 3], *vj = &bval[(((size_t)o * nq + q) * nb + j) * 3];
            for (int k = 0; k < 6; ++k) {
              const int a = ab[k][0], b = ab[k][1];
              t[(size_t)(6 + k) * n2] += w[q] * (vj[a] * vi[b] + (a != b ? vj[b] * vi[a] : 0.0));
            }
          } else {
            t[(size_t)6 * n2] += w[q] * bval[((size_t)o * nq + q) * nb + i] * bval[((size_t)o * nq + q) * nb + j];
          }
        }
      }
  std::vector<int32_t> orient((size_t)p.E, 0);
  if (p.orient && p.E) FG_CUDA(cudaMemcpy(orient.data(), p.orient, (size_t)p.E * 4, cudaMemcpyDeviceToHost));
  std::vector<int32_t> perm((size_t)p.E);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int32_t a, int32_t b) { return orient[a] < orient[b]; });
  std::vector<int4> tiles;
  for (int64_t r = 0; r < p.E;) {
    const int o = orient[perm[r]];
    int64_t e = r;
    while (e < p.E && e - r < kFacTile && orient[perm[e]] == o) ++e;
    tiles.push_back(make_int4(o, (int)r, (int)(e - r), 0));
    r = e;
  }
  FG_CUDA(cudaMalloc(&f->T, std::max<size_t>(T.size(), 1) * 8));
  FG_CUDA(cudaMemcpy(f->T, T.data(), T.size() * 8, cudaMemcpyHostToDevice));
  FG_CUDA(cudaMalloc(&f->perm, std::max<size_t>(perm.size(), 1) * 4));
  if (!perm.empty()) FG_CUDA(cudaMemcpy(f->perm, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice));
  FG_CUDA(cudaMalloc(&f->tiles, std::max<size_t>(tiles.size(), 1) * sizeof(int4)));
  if (!tiles.empty()) FG_CUDA(cudaMemcpy(f->tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice));
  f->nTiles = (int)tiles.size();
  f->built = 1;
  return FG_OK;
}

bool factoredFp64Applies(const fg_plan *plan, const DevTerms &terms) {
  const PlanDev &p = plan->d;
  if (plan->fp64Method != FG_FP64_FACTORED) return false;
  if (!p.affine || p.mult != 1 || terms.hasElastic || terms.hasJacMod || terms.nonSym || terms.tensorTerm >= 0 ||
      terms.tensorMassTerm >= 0)
    return false;
  for (int t = 0; t < terms.n; ++t)
    if (terms.t[t].kind != FG_TERM_SOURCE && terms.t[t].coef.cls == kExprPoint) return false;
  // the reference tensors of a block live in shared memory (HCurl of order 2
  // on tetrahedra, 45 functions, does not fit: the quadrature loop applies)
  const size_t kp = p.form == FG_FORM_1 ? 12 : 7;
  return (kp * p.n * p.n + (size_t)kFacTile * 2 * kFacMax) * sizeof(double) <= 200 * 1024;
}

bool factoredFp64Ready(const fg_plan *plan) {
  const FactoredState *f = (const FactoredState *)plan->fp64f;
  return f && f->built;
}

// The tables are built when the method is chosen (fg_plan_set_fp64_method),
// so a launch allocates nothing and issues no blocking copy.
int launchFactoredFp64(fg_plan *plan, const DevTerms &terms, const DevTerms *dterms, double *ke, cudaStream_t s) {
  if (!factoredFp64Ready(plan)) {
    setLastError("FP64 factored kernel: the plan's reference tensors are not built");
    return FG_ERR_ARG;
  }
  FactoredState *f = factoredState(plan);
  const PlanDev &p = plan->d;
  if (f->nTiles == 0) return FG_OK;
  const size_t smem = ((size_t)f->kp * p.n * p.n + (size_t)kFacTile * 2 * kFacMax) * sizeof(double);
  if (smem > 200 * 1024) {
    setLastError("FP64 factored kernel: reference tensors larger than shared memory");
    return FG_ERR_UNSUPPORTED;
  }
  const bool cplx = terms.complexKe != 0;
  auto kern = cplx ? k_element_factored_fp64<true> : k_element_factored_fp64<false>;
  static SmemAllowance allowed[2];
  FG_CUDA(allowSmem(kern, smem, allowed[cplx]));
  ProfScope prof("k_element_factored_fp64", s);
  kern<<<f->nTiles, 256, smem, s>>>(p, dterms, f->T, f->perm, f->tiles, f->kp, ke);
  countLaunch();
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

}  // namespace femg

extern "C" int fg_plan_set_fp64_method(fg_plan *plan, int32_t method) {
  if (!plan || (method != FG_FP64_QUADRATURE && method != FG_FP64_FACTORED)) {
    femg::setLastError("fg_plan_set_fp64_method: invalid arguments");
    return FG_ERR_ARG;
  }
  // the reference tensors and element tiles are built here, once, so that
  // assemble calls (fg_assemble_fp64_static included) allocate nothing for them
  if (method == FG_FP64_FACTORED && plan->d.E > 0) {
    const int st = femg::prepareFactored(plan);
    if (st) return st;
  }
  plan->fp64Method = method;
  return FG_OK;
}

extern "C" int fg_plan_set_accumulate(fg_plan *plan, int32_t accumulate) {
  if (!plan || (accumulate != 0 && accumulate != 1)) {
    femg::setLastError("fg_plan_set_accumulate: invalid arguments");
    return FG_ERR_ARG;
  }
  plan->accumulate = accumulate;
  return FG_OK;
}

extern "C" void fp64fDestroy(fg_plan *plan) {
  femg::FactoredState *f = (femg::FactoredState *)plan->fp64f;
  if (!f) return;
  cudaFree(f->T);
  cudaFree(f->perm);
  cudaFree(f->tiles);
  delete f;
  plan->fp64f = nullptr;
}
