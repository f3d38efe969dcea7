// A stand-in for libfemg.so's C ABI on a machine without a GPU — TEST
// INFRASTRUCTURE ONLY. Linked into the drop-in program (ref_dropin: the
// reference's library and a GmshFEM program whose formulation is the
// GpuFormulation of fem-g_gb300/binding/), it takes the calls the binding
// makes (fg_plan_create, fg_plan_create_coupled, fg_assemble_fp64,
// fg_assemble_separate, fg_plan_destroy, fg_last_error),
// computes each assembly with the oracle's restatement (or_assemble) so that
// the program's output can be set against the reference's own assemble(),
// and appends every call's descriptors to the file named by FEMG_RECORD, for
// the GPU tests to replay through the real library.
//
// Record file: "FEMGREC1", then per fg_assemble_fp64 / fg_assemble_separate call
//   entry  i32 0 (fg_assemble_fp64) or 1 (fg_assemble_separate)
//   mesh   i32 dim, nn; i64 n_nodes; f64 xyz[n_nodes][3]; i64 E; i64 elem_nodes[E][nn]
//   rule   i32 nq; f64 w[nq], geo_val[nq][nn], geo_grad[nq][nn][3]
//   space  i32 nb, mult, n_orient, form; f64 val[..], grad[..]; i32 has_orient; i32 orient[E] if has_orient
//   system u64 n_rows; u64 ai[n_rows + 1], aj[nnz], edof[E][n]; i32 etype[E][n]; u64 n_fixed; i32 upper
//   column i32 coupled; if coupled (fg_plan_create_coupled) the unknown field's space and DOF map:
//          i32 nb, n_orient, form; f64 val[..], grad[..]; i32 has_orient; i32 orient[E] if has_orient;
//          u64 edof[E][nb]; i32 etype[E][nb]
//   call   f64 frequency; f64 dirichlet[n_fixed][2]
//   terms  i32 n; per term i32 kind, dt, then its coefficient programs coef and coef2 (mu of the
//          elastic term; n_code 0 otherwise) and i32 n_tensor programs
//          (the vector or tensor of the kind), each program as i32 n_code; per instruction
//          i32 op, arg; f64 re, im; i32 n_arrays; per array u64 count; f64 values[count]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../include/fem_g_gb300.h"

extern "C" {
// the oracle's bucket and entry point (oracle.c)
typedef struct {
  int dim, nn, nq, nb, mult;
  int64_t E;
  const double *xyz;
  const int64_t *enodes;
  const double *w;
  const double *geo_val;
  const double *geo_grad;
  const double *bval;
  const double *bgrad;
  const int32_t *orient;
  int32_t form;
  int32_t upper;
  const uint64_t *linked_row;
  const double *linked_value;
} or_bucket;
int or_assemble(const or_bucket *b, const fg_term_desc *terms, int nterms, double freq, const uint64_t *ai, const uint64_t *aj,
                const uint64_t *edof, const int32_t *etype, const double *dirichlet, double *values, double *rhs);
int or_assemble_coupled(const or_bucket *bt, const or_bucket *bu, const fg_term_desc *terms, int nterms, double freq,
                        const uint64_t *ai, const uint64_t *aj, const uint64_t *edofT, const int32_t *etypeT,
                        const uint64_t *edofU, const int32_t *etypeU, const double *dirichlet, double *values, double *rhs);
}

namespace {

std::string g_error;

struct Recorded {
  int32_t dim, nn, nq, nb, mult, nOrient, form, upper;
  int64_t E;
  std::vector<double> xyz, w, gv, gg, bval, bgrad;
  std::vector<int64_t> enodes;
  std::vector<int32_t> orient, etype;
  std::vector<uint64_t> ai, aj, edof;
  uint64_t nRows, nFixed;
  // the unknown field of a two-field plan
  bool coupled = false;
  int32_t nbU = 0, nOrientU = 1, formU = 0;
  std::vector<double> bvalU, bgradU;
  std::vector<int32_t> orientU, etypeU;
  std::vector<uint64_t> edofU;
};

template <class V>
void put(FILE *f, const V *p, size_t n) {
  if (n) std::fwrite(p, sizeof(V), n, f);
}
template <class V>
void put1(FILE *f, V v) {
  put(f, &v, 1);
}

// programs of a term's vector or tensor
int tensorPrograms(int kind) {
  switch (kind) {
    case FG_TERM_GRAD_GRAD_TENSOR:
    case FG_TERM_MASS_TENSOR: return 6;
    case FG_TERM_GRAD_GRAD_TENSOR_FULL: return 9;
    case FG_TERM_ADVECTION:
    case FG_TERM_VECTOR_GRAD_TEST:
    case FG_TERM_SOURCE_GRAD: return 3;
  }
  return 0;
}

void putExpr(FILE *f, const fg_expr &ex, int64_t E, int nq, int nb) {
  put1<int32_t>(f, ex.n_code);
  for (int k = 0; k < ex.n_code; ++k) {
    put1<int32_t>(f, ex.code[k].op);
    put1<int32_t>(f, ex.code[k].arg);
    put1<double>(f, ex.code[k].re);
    put1<double>(f, ex.code[k].im);
  }
  put1<int32_t>(f, ex.n_arrays);
  for (int a = 0; a < ex.n_arrays; ++a) {
    uint64_t count = 2 * (uint64_t)E;
    for (int k = 0; k < ex.n_code; ++k)
      if (ex.code[k].arg == a && ex.code[k].op == FG_OP_POINT) count = 2 * (uint64_t)E * nq;
      else if (ex.code[k].arg == a && ex.code[k].op == FG_OP_FIELD) count = 2 * (uint64_t)E * nb;
    put1<uint64_t>(f, count);
    put(f, ex.elem_values[a], count);
  }
}

}  // namespace

struct fg_plan {
  Recorded r;
};

extern "C" {

int fg_plan_create(const fg_mesh_desc *mesh, const fg_rule_desc *rule, const fg_space_desc *space, const fg_system_desc *sys,
                   fg_plan **out) {
  if (!mesh || !rule || !space || !sys || !out) {
    g_error = "fg_plan_create: invalid arguments";
    return FG_ERR_ARG;
  }
  if (sys->n_linked) {
    g_error = "recording stand-in: linked DOFs are not recorded";
    return FG_ERR_UNSUPPORTED;
  }
  auto *p = new fg_plan();
  Recorded &r = p->r;
  r.dim = mesh->dim;
  r.nn = mesh->nodes_per_element;
  r.E = mesh->n_elements;
  r.xyz.assign(mesh->node_xyz, mesh->node_xyz + 3 * mesh->n_nodes);
  r.enodes.assign(mesh->elem_nodes, mesh->elem_nodes + r.E * r.nn);
  r.nq = rule->nq;
  r.w.assign(rule->weights, rule->weights + r.nq);
  r.gv.assign(rule->geo_val, rule->geo_val + (size_t)r.nq * r.nn);
  r.gg.assign(rule->geo_grad, rule->geo_grad + (size_t)r.nq * r.nn * 3);
  r.nb = space->n_basis;
  r.mult = space->multiplicity;
  r.nOrient = space->n_orientations;
  r.form = space->form;
  const size_t nv = (size_t)r.nOrient * r.nq * r.nb * (r.form == FG_FORM_1 ? 3 : 1);
  r.bval.assign(space->basis_val, space->basis_val + nv);
  r.bgrad.assign(space->basis_grad, space->basis_grad + (size_t)r.nOrient * r.nq * r.nb * 3);
  if (space->elem_orientation) r.orient.assign(space->elem_orientation, space->elem_orientation + r.E);
  r.nRows = sys->n_rows;
  r.ai.assign(sys->ai, sys->ai + r.nRows + 1);
  r.aj.assign(sys->aj, sys->aj + r.ai[r.nRows]);
  const size_t en = (size_t)r.E * r.nb * r.mult;
  r.edof.assign(sys->elem_dof_idx, sys->elem_dof_idx + en);
  r.etype.assign(sys->elem_dof_type, sys->elem_dof_type + en);
  r.nFixed = sys->n_fixed;
  r.upper = sys->upper;
  *out = p;
  return FG_OK;
}

int fg_plan_create_coupled(const fg_mesh_desc *mesh, const fg_rule_desc *rule, const fg_space_desc *space, const fg_system_desc *sys,
                           const fg_space_desc *uspace, const uint64_t *uidx, const int32_t *utype, fg_plan **out) {
  if (!uspace || !uidx || !utype) {
    g_error = "fg_plan_create_coupled: invalid arguments";
    return FG_ERR_ARG;
  }
  const int st = fg_plan_create(mesh, rule, space, sys, out);
  if (st) return st;
  Recorded &r = (*out)->r;
  r.coupled = true;
  r.nbU = uspace->n_basis;
  r.nOrientU = uspace->n_orientations;
  r.formU = uspace->form;
  const size_t per = (size_t)r.nOrientU * r.nq * r.nbU;
  r.bvalU.assign(uspace->basis_val, uspace->basis_val + per * (r.formU == FG_FORM_1 ? 3 : 1));
  r.bgradU.assign(uspace->basis_grad, uspace->basis_grad + per * 3);
  if (uspace->elem_orientation) r.orientU.assign(uspace->elem_orientation, uspace->elem_orientation + r.E);
  r.edofU.assign(uidx, uidx + (size_t)r.E * r.nbU);
  r.etypeU.assign(utype, utype + (size_t)r.E * r.nbU);
  return FG_OK;
}

void fg_plan_destroy(fg_plan *plan) { delete plan; }

const char *fg_last_error(void) { return g_error.c_str(); }

static int recordCall(const fg_plan *plan, int entry, const fg_term_desc *terms, int32_t n_terms, double frequency,
                      const double *dirichlet) {
  const Recorded &r = plan->r;
  if (const char *path = std::getenv("FEMG_RECORD")) {
    FILE *f = std::fopen(path, "ab");
    if (!f) {
      g_error = std::string("cannot append to ") + path;
      return FG_ERR_ARG;
    }
    if (std::ftell(f) == 0) std::fwrite("FEMGREC1", 1, 8, f);
    put1<int32_t>(f, entry);
    put1<int32_t>(f, r.dim);
    put1<int32_t>(f, r.nn);
    put1<int64_t>(f, (int64_t)(r.xyz.size() / 3));
    put(f, r.xyz.data(), r.xyz.size());
    put1<int64_t>(f, r.E);
    put(f, r.enodes.data(), r.enodes.size());
    put1<int32_t>(f, r.nq);
    put(f, r.w.data(), r.w.size());
    put(f, r.gv.data(), r.gv.size());
    put(f, r.gg.data(), r.gg.size());
    put1<int32_t>(f, r.nb);
    put1<int32_t>(f, r.mult);
    put1<int32_t>(f, r.nOrient);
    put1<int32_t>(f, r.form);
    put(f, r.bval.data(), r.bval.size());
    put(f, r.bgrad.data(), r.bgrad.size());
    put1<int32_t>(f, r.orient.empty() ? 0 : 1);
    put(f, r.orient.data(), r.orient.size());
    put1<uint64_t>(f, r.nRows);
    put(f, r.ai.data(), r.ai.size());
    put(f, r.aj.data(), r.aj.size());
    put(f, r.edof.data(), r.edof.size());
    put(f, r.etype.data(), r.etype.size());
    put1<uint64_t>(f, r.nFixed);
    put1<int32_t>(f, r.upper);
    put1<int32_t>(f, r.coupled ? 1 : 0);
    if (r.coupled) {
      put1<int32_t>(f, r.nbU);
      put1<int32_t>(f, r.nOrientU);
      put1<int32_t>(f, r.formU);
      put(f, r.bvalU.data(), r.bvalU.size());
      put(f, r.bgradU.data(), r.bgradU.size());
      put1<int32_t>(f, r.orientU.empty() ? 0 : 1);
      put(f, r.orientU.data(), r.orientU.size());
      put(f, r.edofU.data(), r.edofU.size());
      put(f, r.etypeU.data(), r.etypeU.size());
    }
    put1<double>(f, frequency);
    put(f, dirichlet, r.nFixed ? 2 * r.nFixed : 0);
    put1<int32_t>(f, n_terms);
    for (int t = 0; t < n_terms; ++t) {
      const fg_term_desc &d = terms[t];
      if (tensorPrograms(d.kind) && !d.tensor) {
        std::fclose(f);
        g_error = "recording stand-in: a tensor term without its programs";
        return FG_ERR_ARG;
      }
      put1<int32_t>(f, d.kind);
      put1<int32_t>(f, d.dt);
      putExpr(f, d.coef, r.E, r.nq, r.nb);
      putExpr(f, d.coef2, r.E, r.nq, r.nb);
      put1<int32_t>(f, tensorPrograms(d.kind));
      for (int k = 0; k < tensorPrograms(d.kind); ++k) putExpr(f, d.tensor[k], r.E, r.nq, r.nb);
    }
    std::fclose(f);
  }
  return FG_OK;
}

// the oracle's assembly of the call into csr_values / rhs (overwritten)
static int compute(const fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, double frequency, const double *dirichlet,
                   double *csr_values, double *rhs) {
  const Recorded &r = plan->r;
  or_bucket b{};
  b.dim = r.dim;
  b.nn = r.nn;
  b.nq = r.nq;
  b.nb = r.nb;
  b.mult = r.mult;
  b.E = r.E;
  b.xyz = r.xyz.data();
  b.enodes = r.enodes.data();
  b.w = r.w.data();
  b.geo_val = r.gv.data();
  b.geo_grad = r.gg.data();
  b.bval = r.bval.data();
  b.bgrad = r.bgrad.data();
  b.orient = r.orient.empty() ? nullptr : r.orient.data();
  b.form = r.form;
  b.upper = r.upper;
  std::memset(csr_values, 0, r.ai[r.nRows] * 16);
  if (rhs) std::memset(rhs, 0, r.nRows * 16);
  int err = 0;
  if (r.coupled) {
    or_bucket bu = b;
    bu.nb = r.nbU;
    bu.bval = r.bvalU.data();
    bu.bgrad = r.bgradU.data();
    bu.orient = r.orientU.empty() ? nullptr : r.orientU.data();
    bu.form = r.formU;
    err = or_assemble_coupled(&b, &bu, terms, n_terms, frequency, r.ai.data(), r.aj.data(), r.edof.data(), r.etype.data(),
                              r.edofU.data(), r.etypeU.data(), dirichlet, csr_values, rhs);
  } else {
    err = or_assemble(&b, terms, n_terms, frequency, r.ai.data(), r.aj.data(), r.edof.data(), r.etype.data(), dirichlet,
                      csr_values, rhs);
  }
  if (err) {
    g_error = "oracle assembly failed with status " + std::to_string(err);
    return FG_ERR_ARG;
  }
  return FG_OK;
}

int fg_assemble_fp64(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, double frequency, const double *dirichlet,
                     double *csr_values, double *rhs, void *stream) {
  (void)stream;
  if (!plan || (n_terms > 0 && !terms) || !csr_values) {
    g_error = "fg_assemble_fp64: invalid arguments";
    return FG_ERR_ARG;
  }
  if (int st = recordCall(plan, 0, terms, n_terms, frequency, dirichlet)) return st;
  return compute(plan, terms, n_terms, frequency, dirichlet, csr_values, rhs);
}

// K from the terms without time derivative (with the sources and the
// lifting), C from the dt terms, M from the dt2 terms, each without the
// frequency factor
int fg_assemble_separate(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, int32_t mixed, const double *dirichlet,
                         double *k_values, double *c_values, double *m_values, double *rhs, void *stream) {
  (void)stream;
  (void)mixed;
  if (!plan || (n_terms > 0 && !terms)) {
    g_error = "fg_assemble_separate: invalid arguments";
    return FG_ERR_ARG;
  }
  if (int st = recordCall(plan, 1, terms, n_terms, 0.0, dirichlet)) return st;
  double *outs[3] = {k_values, c_values, m_values};
  for (int dt = 0; dt < 3; ++dt) {
    std::vector<fg_term_desc> sub;
    for (int t = 0; t < n_terms; ++t)
      if (terms[t].dt == dt) {
        sub.push_back(terms[t]);
        sub.back().dt = FG_DT_NONE;
      }
    std::vector<double> scratch;
    double *v = outs[dt];
    if (!v) {
      scratch.resize(2 * plan->r.ai[plan->r.nRows]);
      v = scratch.data();
    }
    // the right-hand side (sources and the lifting) comes with K alone
    if (int st = compute(plan, sub.data(), (int32_t)sub.size(), 0.0, dirichlet, v, dt == 0 ? rhs : nullptr)) return st;
  }
  return FG_OK;
}

}  // extern "C"
