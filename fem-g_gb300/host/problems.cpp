// C ABI of the host mirror (include/fem_g_gb300_host.h): builds the benchmark
// problems the way a GmshFEM user program does (mesh, field, constraints,
// Formulation::integral, pre) and hands their descriptors to the GPU plan.
// Host code only: fg_problem_assemble, which drives the GPU, is in
// problem_assemble.cpp, so this file also builds the host-only library.
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "../../include/fem_g_gb300_host.h"
#include "formulation.h"

namespace femg {
void setLastError(const std::string &msg);
}

#include "problem_internal.h"


using namespace femg;

static void buildProblem(fg_problem *p) {
  const fg_problem_config &c = p->cfg;
  if (c.dim == 2)
    p->mesh = makeSquareTri(c.m, c.mesh_order, c.jitter, c.seed);
  else if (c.dim == 3)
    p->mesh = makeCubeTet(c.m, c.mesh_order, c.jitter, c.seed);
  else
    throw std::invalid_argument("dim must be 2 or 3");
  Domain omega(p->mesh, "omega");
  const SpaceType st = c.space == FG_SPACE_LAGRANGE ? SpaceType::Lagrange
                       : c.space == FG_SPACE_HCURL  ? SpaceType::HCurl
                                                    : SpaceType::HierarchicalH1;
  if ((c.kind == FG_PROBLEM_MAXWELL) != (st == SpaceType::HCurl))
    throw std::invalid_argument("the Maxwell problem takes the HCurl space, and only it does");
  if (c.kind == FG_PROBLEM_COUPLED) {
    // two scalar fields (tags 0 and 1, the reference's field counter),
    // coupled both ways
    p->u.reset(new Field("u", omega, st, c.order, 1, 0));
    p->v.reset(new Field("v", omega, st, c.order2 > 0 ? c.order2 : c.order, 1, 1));
    Field &u = *p->u, &v = *p->v;
    p->form.reset(new Formulation("coupled"));
    p->form->setSymmetric(c.upper != 0);
    Formulation &f = *p->form;
    const std::string gauss = "Gauss" + std::to_string(c.gauss);
    if (c.dirichlet) {
      if (c.dim != 2) throw std::invalid_argument("Dirichlet boundary only on the 2D square");
      u.addConstraint(Domain(p->mesh, "gammaDir"), cplx(c.dirichlet_value, 0.0));
    }
    Function x = Function::x(), y = Function::y();
    f.integral(grad(dof(u)), grad(tf(u)), omega, gauss);
    f.integral(Function(-c.k * c.k) * dof(u), tf(u), omega, gauss);
    f.integral(grad(dof(v)), grad(tf(v)), omega, gauss);
    f.integral(Function(2.0) * dof(v), tf(v), omega, gauss);
    f.integral((Function(0.5) + x) * dof(u), tf(v), omega, gauss);
    VectorFunction b{Function(1.0), Function(cplx(-0.5, 0.2)), Function(0.25)};
    f.integral(b * grad(dof(u)), tf(v), omega, gauss);
    f.integral(Function(0.3) * grad(dof(v)), grad(tf(u)), omega, gauss);
    if (c.source) {
      Function fsrc = heaviside(Function(0.01) - (x - Function(0.5)) * (x - Function(0.5)) - (y - Function(0.5)) * (y - Function(0.5)));
      f.integral(-fsrc, tf(u), omega, gauss);
      f.integral(Function(1.0) + x * y, tf(v), omega, gauss);
    }
    f.pre(p->mesh);
    return;
  }
  const int mult = c.kind == FG_PROBLEM_NAVIER ? 3 : 1;
  p->u.reset(new Field("u", omega, st, c.order, mult, 0));
  Field &u = *p->u;
  p->form.reset(new Formulation(c.kind == FG_PROBLEM_NAVIER ? "navier" : c.kind == FG_PROBLEM_MAXWELL ? "maxwell" : "helmholtz"));
  p->form->setSymmetric(c.upper != 0);
  Formulation &f = *p->form;
  const std::string gauss = "Gauss" + std::to_string(c.gauss);
  const int64_t E = p->mesh.find(c.dim, 1)->blocks[0].size();
  if (c.kind == FG_PROBLEM_HELMHOLTZ) {
    if (c.dirichlet) {
      if (c.dim != 2) throw std::invalid_argument("Dirichlet boundary only on the 2D square");
      u.addConstraint(Domain(p->mesh, "gammaDir"), cplx(c.dirichlet_value, 0.0));
    }
    f.integral(grad(dof(u)), grad(tf(u)), omega, gauss);
    if (c.coef_mode == FG_COEF_MODE_CONSTANT) {
      f.integral(Function(-c.k * c.k) * dof(u), tf(u), omega, gauss);
    } else {
      // c_e = k^2 (1 + 0.3 xi_e), xi_e ~ N(0,1) per element in element order
      Rng rng(c.seed + 1);
      std::vector<cplx> ce((size_t)E);
      for (int64_t e = 0; e < E; ++e) ce[(size_t)e] = cplx(-c.k * c.k * (1.0 + 0.3 * rng.normal()), 0.0);
      f.integral(Function::perElement(ce) * dof(u), tf(u), omega, gauss);
    }
    if (c.source) {
      Function x = Function::x(), y = Function::y();
      Function fsrc = heaviside(Function(0.01) - (x - Function(0.5)) * (x - Function(0.5)) - (y - Function(0.5)) * (y - Function(0.5)));
      f.integral(-fsrc, tf(u), omega, gauss);
    }
  } else if (c.kind == FG_PROBLEM_MAXWELL) {
    // curl curl E - k^2 c E: constant or per-element relative permittivity
    f.integral(curl(dof(u)), curl(tf(u)), omega, gauss);
    if (c.coef_mode == FG_COEF_MODE_CONSTANT) {
      f.integral(Function(-c.k * c.k) * dof(u), tf(u), omega, gauss);
    } else {
      Rng rng(c.seed + 1);
      std::vector<cplx> ce((size_t)E);
      for (int64_t e = 0; e < E; ++e) ce[(size_t)e] = cplx(-c.k * c.k * (1.0 + 0.3 * rng.normal()), 0.0);
      f.integral(Function::perElement(ce) * dof(u), tf(u), omega, gauss);
    }
  } else if (c.kind == FG_PROBLEM_NAVIER) {
    Rng rng(c.seed + 2);
    std::vector<cplx> lam((size_t)E), mu((size_t)E);
    for (int64_t e = 0; e < E; ++e) {
      lam[(size_t)e] = std::exp(c.lame_sigma * rng.normal());
      mu[(size_t)e] = std::exp(c.lame_sigma * rng.normal());
    }
    Tensor4Isotropic C{Function::perElement(lam), Function::perElement(mu)};
    f.integral(C * grad(dof(u)), grad(tf(u)), omega, gauss);
    if (c.omega > 0.0) f.integral(Function(-c.omega * c.omega) * dof(u), tf(u), omega, gauss);  // rho = 1
    else f.integral(dt2_dof(u), tf(u), omega, gauss);  // frequency of the assemble call (AFrequency)
  } else {
    throw std::invalid_argument("unknown problem kind");
  }
  f.pre(p->mesh);
}

extern "C" {

int fg_problem_create(const fg_problem_config *cfg, fg_problem **out) {
  if (!cfg || !out) {
    setLastError("fg_problem_create: null argument");
    return FG_ERR_ARG;
  }
  *out = nullptr;
  fg_problem *p = new (std::nothrow) fg_problem;
  if (!p) return FG_ERR_OOM;
  p->cfg = *cfg;
  try {
    buildProblem(p);
  } catch (const std::bad_alloc &) {
    delete p;
    setLastError("fg_problem_create: out of memory");
    return FG_ERR_OOM;
  } catch (const std::exception &e) {
    delete p;
    setLastError(std::string("fg_problem_create: ") + e.what());
    return FG_ERR_ARG;
  }
  *out = p;
  return FG_OK;
}

void fg_problem_destroy(fg_problem *p) {
  if (!p) return;
  if (p->plan && p->destroyPlan) p->destroyPlan(p->plan);
  delete p;
}

int fg_problem_descs(const fg_problem *p, fg_mesh_desc *mesh, fg_rule_desc *rule, fg_space_desc *space,
                     fg_system_desc *sys, const fg_term_desc **terms, int32_t *n_terms, const double **dirichlet) {
  if (!p) return FG_ERR_ARG;
  fg_mesh_desc m;
  fg_rule_desc r;
  fg_space_desc s;
  fg_system_desc y;
  p->form->descs(&m, &r, &s, &y);
  if (mesh) *mesh = m;
  if (rule) *rule = r;
  if (space) *space = s;
  if (sys) *sys = y;
  if (terms) *terms = p->form->termDescs.data();
  if (n_terms) *n_terms = (int32_t)p->form->termDescs.size();
  if (dirichlet) *dirichlet = p->form->nFixed ? p->form->dirichlet.data() : nullptr;
  return FG_OK;
}

int64_t fg_problem_n_dofs(const fg_problem *p) {
  if (!p) return -1;
  int64_t n = 0;
  for (const Field *f : p->form->fields) n += (int64_t)f->dofs.size();
  return n;
}

int fg_problem_raw_dofs(const fg_problem *p, uint64_t *num_type, uint64_t *entity, uint64_t *num_dof, int32_t *assemble_type, float *xyz) {
  if (!p) return FG_ERR_ARG;
  size_t i = 0;
  for (const Field *f : p->form->fields) {
    const auto &dd = f->dofs;
    for (uint32_t id : dd.table.order()) {
      const Dof &d = dd.pool[id];
      if (num_type) num_type[i] = d.numType;
      if (entity) entity[i] = d.entity;
      if (num_dof) num_dof[i] = d.numDof;
      if (assemble_type) assemble_type[i] = d.assembleType;
      if (xyz)
        for (int c = 0; c < 3; ++c) xyz[3 * i + c] = d.xyz[c];
      ++i;
    }
  }
  return FG_OK;
}

int32_t fg_problem_n_fields(const fg_problem *p) { return p ? (int32_t)p->form->fields.size() : -1; }

int fg_problem_field(const fg_problem *p, int32_t k, fg_space_desc *space, const uint64_t **elem_dof_idx,
                     const int32_t **elem_dof_type) {
  if (!p || k < 0 || k >= (int32_t)p->form->fields.size()) return FG_ERR_ARG;
  if (space) p->form->spaceDesc(k, space);
  if (elem_dof_idx) *elem_dof_idx = p->form->fieldBuckets[(size_t)k].elemDofIdx.data();
  if (elem_dof_type) *elem_dof_type = p->form->fieldBuckets[(size_t)k].elemDofType.data();
  return FG_OK;
}

int32_t fg_problem_n_blocks(const fg_problem *p) { return p ? (int32_t)p->form->blocks.size() : -1; }

int fg_problem_block(const fg_problem *p, int32_t b, int32_t *test_field, int32_t *unknown_field, const fg_term_desc **terms,
                     int32_t *n_terms) {
  if (!p || b < 0 || b >= (int32_t)p->form->blocks.size()) return FG_ERR_ARG;
  const auto &bl = p->form->blocks[(size_t)b];
  if (test_field) *test_field = bl.test;
  if (unknown_field) *unknown_field = bl.unknown;
  if (terms) *terms = bl.terms.data();
  if (n_terms) *n_terms = (int32_t)bl.terms.size();
  return FG_OK;
}

int fg_problem_created_dofs(const fg_problem *p, uint64_t *num_type, uint64_t *entity, int32_t *assemble_type, float *xyz) {
  if (!p) return FG_ERR_ARG;
  const auto &cr = p->form->created;
  for (size_t i = 0; i < cr.size(); ++i) {
    if (num_type) num_type[i] = cr[i].numType;
    if (entity) entity[i] = cr[i].entity;
    if (assemble_type) assemble_type[i] = cr[i].assembleType;
    if (xyz)
      for (int c = 0; c < 3; ++c) xyz[3 * i + c] = cr[i].xyz[c];
  }
  return FG_OK;
}

int64_t fg_problem_reserve_log(const fg_problem *p, uint64_t *at, uint64_t *arg, int64_t cap) {
  if (!p) return -1;
  const auto &log = p->form->reserveLog;
  for (size_t i = 0; i < log.size() && (int64_t)i < cap; ++i) {
    if (at) at[i] = log[i].first;
    if (arg) arg[i] = log[i].second;
  }
  return (int64_t)log.size();
}

int fg_problem_bbox(const fg_problem *p, double *bbox) {
  if (!p || !bbox) return FG_ERR_ARG;
  std::memcpy(bbox, p->mesh.bbox, 6 * sizeof(double));
  return FG_OK;
}

double fg_problem_pre_seconds(const fg_problem *p) { return p ? p->form->preSeconds : -1.0; }

int fg_basis_eval(int32_t space, int32_t order, int32_t dim, int32_t code, int64_t npts, const double *uvw, double *val,
                  double *deriv) {
  if ((space != FG_SPACE_HIERARCHICAL_H1 && space != FG_SPACE_HCURL) || (dim != 2 && dim != 3) || npts < 0 ||
      (npts > 0 && !uvw) || order < (space == FG_SPACE_HCURL ? 0 : 1) || order > 12 || code < 0) {
    setLastError("fg_basis_eval: invalid arguments");
    return -FG_ERR_ARG;
  }
  const bool hc = space == FG_SPACE_HCURL;
  const int n = hc ? hcurlCount(dim, order) : hierarchicalCount(dim, order);
  const int vn = hc ? 3 * n : n;
  std::vector<double> v(vn), d(3 * n);
  for (int64_t q = 0; q < npts; ++q) {
    if (hc) hcurlBasis(dim, order, code, &uvw[3 * q], v.data(), d.data());
    else hierarchicalBasis(dim, order, code, &uvw[3 * q], v.data(), d.data());
    if (val) std::memcpy(val + (size_t)q * vn, v.data(), vn * sizeof(double));
    if (deriv) std::memcpy(deriv + (size_t)q * 3 * n, d.data(), 3 * n * sizeof(double));
  }
  return n;
}

int fg_basis_orientation(int32_t space, int32_t order, int32_t dim, const int64_t *vertex_tags) {
  if ((space != FG_SPACE_HIERARCHICAL_H1 && space != FG_SPACE_HCURL) || (dim != 2 && dim != 3) || !vertex_tags) {
    setLastError("fg_basis_orientation: invalid arguments");
    return -FG_ERR_ARG;
  }
  return space == FG_SPACE_HCURL ? hcurlOrientation(dim, order, vertex_tags) : hierarchicalOrientation(dim, vertex_tags);
}

}  // extern "C"
