// A GmshFEM-style program on the host mirror: a Helmholtz formulation built
// with Domain, Field, Formulation::integral(dof, tf, grad), pre(), then
// assembled through the GPU path of the C ABI (fg_plan_create,
// fg_assemble_fp64, fg_assemble_mixed). The checks follow the reference's
// coverage tests of assembled systems (unitTests/coverage/posts.cpp:393-548:
// a Hermitian left-hand side for real wavenumbers, consistent nonzero counts)
// and its exact integrals of 1 over simple domains (:77-118), here as the
// exact energies u^T A u of u = 1 and u = x. A second formulation with a
// TensorFunction coefficient checks the energies x_a^T A x_b = D_ab, and a
// field-node coefficient u = x is checked against the point function x.
//
// Usage: formulation_test [--cpu]   (--cpu: pre() checks only, no GPU)
// Exit status 0 when every check passes.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../fem-g_gb300/host/formulation.h"
#include "../../fem-g_gb300/host/mesh.h"
#include "../../include/fem_g_gb300.h"

using namespace femg;

static int failures = 0;
#define CHECK(cond, ...)                      \
  do {                                        \
    if (!(cond)) {                            \
      std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
      std::printf(__VA_ARGS__);               \
      std::printf("\n");                      \
      ++failures;                             \
    }                                         \
  } while (0)

// u^T A v over the CSR, for real vectors on the unknown DOFs
static double quad(const Formulation &f, const std::vector<std::complex<double>> &A, const std::vector<double> &u,
                   const std::vector<double> &v) {
  double s = 0.0;
  for (uint64_t r = 0; r < f.nUnknown; ++r)
    for (uint64_t k = f.ai[r]; k < f.ai[r + 1]; ++k) s += u[r] * A[k].real() * v[f.aj[k]];
  return s;
}

int main(int argc, char **argv) {
  const bool cpuOnly = argc > 1 && std::strcmp(argv[1], "--cpu") == 0;
  const int m = 6, p = 3;
  const double k = 7.0;

  // geometry and discretisation: unit cube, m^3 x 6 tets, hierarchical H1 order 3
  Mesh mesh = makeCubeTet(m, 1, 0.15, 42);
  Domain omega(mesh, "omega");
  Field u("u", omega, SpaceType::HierarchicalH1, p, 1, 0);
  Formulation formulation("helmholtz");
  formulation.integral(grad(dof(u)), grad(tf(u)), omega, "Gauss6");
  formulation.integral(Function(-k * k) * dof(u), tf(u), omega, "Gauss6");
  formulation.pre(mesh);

  // pre(): DOFs and pattern
  const uint64_t nDofs = (uint64_t)(p * m + 1) * (p * m + 1) * (p * m + 1);
  CHECK(formulation.nUnknown == nDofs, "unknowns %llu, expected %llu", (unsigned long long)formulation.nUnknown,
        (unsigned long long)nDofs);
  const uint64_t nnz = 1311ull * m * m * m + 459ull * m * m + 45ull * m + 1;  // order-3 Kuhn cube pattern
  CHECK(formulation.ai.back() == nnz, "nnz %llu, expected %llu", (unsigned long long)formulation.ai.back(),
        (unsigned long long)nnz);
  bool sorted = true;
  for (uint64_t r = 0; r < formulation.nUnknown; ++r)
    for (uint64_t q = formulation.ai[r] + 1; q < formulation.ai[r + 1]; ++q) sorted = sorted && formulation.aj[q - 1] < formulation.aj[q];
  CHECK(sorted, "columns sorted and unique in every row");
  if (cpuOnly) {
    std::printf("%s (pre only)\n", failures ? "FAILED" : "OK");
    return failures ? 1 : 0;
  }

  // assemble on the GPU, FP64 and mixed precision
  fg_mesh_desc md;
  fg_rule_desc rd;
  fg_space_desc sd;
  fg_system_desc sys;
  formulation.descs(&md, &rd, &sd, &sys);
  fg_plan *plan = nullptr;
  int st = fg_plan_create(&md, &rd, &sd, &sys, &plan);
  if (st != FG_OK) {
    std::printf("FAIL fg_plan_create: %d %s\n", st, fg_last_error());
    return 1;
  }
  const auto &terms = formulation.termDescs;
  std::vector<std::complex<double>> A64(nnz), A32(nnz), b(formulation.nUnknown);
  st = fg_assemble_fp64(plan, terms.data(), (int)terms.size(), 0.0, nullptr, reinterpret_cast<double *>(A64.data()),
                        reinterpret_cast<double *>(b.data()), nullptr);
  CHECK(st == FG_OK, "fg_assemble_fp64: %s", fg_last_error());
  fg_err_report rep;
  st = fg_assemble_mixed(plan, terms.data(), (int)terms.size(), 0.0, nullptr, reinterpret_cast<double *>(A32.data()),
                         reinterpret_cast<double *>(b.data()), nullptr, &rep);
  CHECK(st == FG_OK, "fg_assemble_mixed: %s", fg_last_error());

  // Hermitian (real symmetric here): A[r][c] == A[c][r]
  double asym = 0.0, amax = 0.0;
  for (uint64_t r = 0; r < formulation.nUnknown; ++r)
    for (uint64_t q = formulation.ai[r]; q < formulation.ai[r + 1]; ++q) {
      const uint64_t c = formulation.aj[q];
      const uint64_t *lo = formulation.aj.data() + formulation.ai[c], *hi = formulation.aj.data() + formulation.ai[c + 1];
      const uint64_t *t = std::lower_bound(lo, hi, r);
      CHECK(t != hi && *t == r, "structurally symmetric pattern");
      asym = std::max(asym, std::abs(A64[q] - std::conj(A64[formulation.ai[c] + (t - lo)])));
      amax = std::max(amax, std::abs(A64[q]));
    }
  CHECK(asym <= 1e-13 * amax, "Hermitian left-hand side: %g", asym / amax);

  // exact energies: 1^T A 1 = -k^2 |cube|, x^T A x = |grad x|^2 - k^2 int x^2 = 1 - k^2 / 3
  // (u = 1 and u = x live in the span of the vertex functions)
  std::vector<double> one(formulation.nUnknown, 0.0), xs(formulation.nUnknown, 0.0);
  for (const Dof &d : formulation.field->dofs.pool) {
    if (d.assembleType != 2 && d.assembleType != 3) continue;
    const uint64_t typeKey = d.numType;  // vertex functions have type key 0
    if (typeKey != 0) continue;
    one[d.numDof - 1] = 1.0;
    xs[d.numDof - 1] = mesh.xyz[3 * (d.entity - 1)];
  }
  const double e1 = quad(formulation, A64, one, one), ex = quad(formulation, A64, xs, xs);
  CHECK(std::abs(e1 + k * k) <= 1e-10 * k * k, "1^T A 1 = %.15g, expected %.15g", e1, -k * k);
  CHECK(std::abs(ex - (1.0 - k * k / 3.0)) <= 1e-10 * k * k, "x^T A x = %.15g, expected %.15g", ex, 1.0 - k * k / 3.0);

  // mixed precision against FP64
  double d2 = 0.0, r2 = 0.0;
  for (uint64_t q = 0; q < nnz; ++q) {
    d2 += std::norm(A32[q] - A64[q]);
    r2 += std::norm(A64[q]);
  }
  CHECK(std::sqrt(d2 / r2) <= 1e-6, "mixed vs FP64 relative Frobenius %g", std::sqrt(d2 / r2));
  CHECK(rep.global_rel_fro <= 1e-6 && rep.max_elem_rel_fro <= 1e-5, "error report %g %g", rep.global_rel_fro,
        rep.max_elem_rel_fro);

  fg_plan_destroy(plan);

  // anisotropic medium: integral(D * grad(dof(v)), grad(tf(v))) with a
  // constant symmetric TensorFunction D; for linear a, b in the span of the
  // vertex functions, a^T A b = grad a . D grad b |cube|
  Field v("v", omega, SpaceType::HierarchicalH1, 2, 1, 0);
  Formulation aniso("anisotropic");
  TensorFunction D;
  D.xx = Function(2.0);
  D.yy = Function(3.0);
  D.zz = Function(4.0);
  D.xy = Function(0.5);
  D.xz = Function(0.25);
  D.yz = Function(-0.5);
  aniso.integral(D * grad(dof(v)), grad(tf(v)), omega, "Gauss4");
  aniso.pre(mesh);
  aniso.descs(&md, &rd, &sd, &sys);
  st = fg_plan_create(&md, &rd, &sd, &sys, &plan);
  CHECK(st == FG_OK, "fg_plan_create (anisotropic): %s", fg_last_error());
  if (st == FG_OK) {
    const uint64_t nnzA = aniso.ai.back();
    std::vector<std::complex<double>> B64(nnzA), B32(nnzA);
    const auto &at = aniso.termDescs;
    st = fg_assemble_fp64(plan, at.data(), (int)at.size(), 0.0, nullptr, reinterpret_cast<double *>(B64.data()), nullptr, nullptr);
    CHECK(st == FG_OK, "fg_assemble_fp64 (anisotropic): %s", fg_last_error());
    st = fg_assemble_mixed(plan, at.data(), (int)at.size(), 0.0, nullptr, reinterpret_cast<double *>(B32.data()), nullptr, nullptr,
                           nullptr);
    CHECK(st == FG_OK, "fg_assemble_mixed (anisotropic): %s", fg_last_error());
    std::vector<double> X[3];
    for (int c = 0; c < 3; ++c) X[c].assign(aniso.nUnknown, 0.0);
    for (const Dof &d : aniso.field->dofs.pool) {
      if ((d.assembleType != 2 && d.assembleType != 3) || d.numType != 0) continue;
      for (int c = 0; c < 3; ++c) X[c][d.numDof - 1] = mesh.xyz[3 * (d.entity - 1) + c];
    }
    const double Dm[3][3] = {{2.0, 0.5, 0.25}, {0.5, 3.0, -0.5}, {0.25, -0.5, 4.0}};
    for (const auto *B : {&B64, &B32})
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
          const double e = quad(aniso, *B, X[a], X[c]), tol = B == &B64 ? 1e-11 : 1e-6;
          CHECK(std::abs(e - Dm[a][c]) <= tol * 4.0, "x%d^T A x%d = %.15g, expected %g (%s)", a, c, e, Dm[a][c],
                B == &B64 ? "FP64" : "mixed");
        }
    fg_plan_destroy(plan);
  }

  // field node (Picard-style coefficient): u = x given by its values at the
  // element DOFs (vertex functions; zero on the higher hierarchical ones)
  // against the point function x, in the mass term of a second field
  {
    Field w1("w1", omega, SpaceType::HierarchicalH1, 2, 1, 0), w2("w2", omega, SpaceType::HierarchicalH1, 2, 1, 0);
    Formulation byPoint("by-point");
    byPoint.integral(Function::x() * dof(w1), tf(w1), omega, "Gauss5");
    byPoint.pre(mesh);
    byPoint.descs(&md, &rd, &sd, &sys);
    const int64_t E = md.n_elements;
    const int nd = sd.n_basis;
    std::vector<double> xv(byPoint.nUnknown, 0.0);
    for (const Dof &d : byPoint.field->dofs.pool)
      if ((d.assembleType == 2 || d.assembleType == 3) && d.numType == 0) xv[d.numDof - 1] = mesh.xyz[3 * (d.entity - 1)];
    std::vector<std::complex<double>> ue((size_t)E * nd);
    for (int64_t e = 0; e < E; ++e)
      for (int j = 0; j < nd; ++j) {
        const int32_t t = sys.elem_dof_type[e * nd + j];
        ue[e * nd + j] = (t == FG_AT_UNKNOWN || t == FG_AT_UNKNOWN_BUBBLE) ? xv[sys.elem_dof_idx[e * nd + j]] : 0.0;
      }
    Formulation byField("by-field");
    byField.integral(Function::fieldValues(ue) * dof(w2), tf(w2), omega, "Gauss5");
    byField.pre(mesh);
    std::vector<std::complex<double>> P, F;
    for (Formulation *f : {&byPoint, &byField}) {
      f->descs(&md, &rd, &sd, &sys);
      st = fg_plan_create(&md, &rd, &sd, &sys, &plan);
      CHECK(st == FG_OK, "fg_plan_create (%s): %s", f == &byPoint ? "point" : "field", fg_last_error());
      if (st != FG_OK) continue;
      std::vector<std::complex<double>> &A = f == &byPoint ? P : F;
      A.assign(f->ai.back(), 0.0);
      st = fg_assemble_fp64(plan, f->termDescs.data(), (int)f->termDescs.size(), 0.0, nullptr, reinterpret_cast<double *>(A.data()),
                            nullptr, nullptr);
      CHECK(st == FG_OK, "fg_assemble_fp64 (%s): %s", f == &byPoint ? "point" : "field", fg_last_error());
      fg_plan_destroy(plan);
    }
    double dmax = 0.0, amax = 0.0;
    CHECK(P.size() == F.size() && byPoint.aj == byField.aj, "same pattern for both fields");
    for (size_t k = 0; k < std::min(P.size(), F.size()); ++k) {
      dmax = std::max(dmax, std::abs(P[k] - F[k]));
      amax = std::max(amax, std::abs(P[k]));
    }
    CHECK(dmax <= 1e-12 * amax, "field node u = x against the point function x: %g", dmax / amax);
  }
  std::printf("%s\n", failures ? "FAILED" : "OK");
  return failures ? 1 : 0;
}
