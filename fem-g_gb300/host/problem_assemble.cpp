// GpuFormulation::assemble of the host mirror: a plan (cached in the problem)
// and the assembly through the C ABI of include/fem_g_gb300.h.
#include "problem_internal.h"

namespace femg {
void setLastError(const std::string &msg);
}

extern "C" {

int fg_problem_assemble(fg_problem *p, int32_t precision, double *csr_values, double *rhs, void *stream) {
  if (!p) return FG_ERR_ARG;
  if (p->form->blocks.size() != 1) {
    femg::setLastError("fg_problem_assemble: a problem of several fields assembles block by block (fg_problem_block)");
    return FG_ERR_UNSUPPORTED;
  }
  fg_mesh_desc m;
  fg_rule_desc r;
  fg_space_desc s;
  fg_system_desc y;
  p->form->descs(&m, &r, &s, &y);
  if (!p->plan) {
    int st = fg_plan_create(&m, &r, &s, &y, &p->plan);
    if (st != FG_OK) return st;
    p->destroyPlan = fg_plan_destroy;
  }
  const auto &t = p->form->termDescs;
  const double *dir = p->form->nFixed ? p->form->dirichlet.data() : nullptr;
  if (precision == 0) return fg_assemble_fp64(p->plan, t.data(), (int32_t)t.size(), 0.0, dir, csr_values, rhs, stream);
  return fg_assemble_mixed(p->plan, t.data(), (int32_t)t.size(), 0.0, dir, csr_values, rhs, stream, nullptr);
}

}  // extern "C"
