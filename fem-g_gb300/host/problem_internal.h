// The problem object behind the host ABI (include/fem_g_gb300_host.h).
#pragma once
#include <memory>

#include "../../include/fem_g_gb300_host.h"
#include "formulation.h"

struct fg_problem {
  fg_problem_config cfg;
  femg::Mesh mesh;
  std::unique_ptr<femg::Field> u, v;  // v: the second field of FG_PROBLEM_COUPLED
  std::unique_ptr<femg::Formulation> form;
  // GPU plan of fg_problem_assemble, created on first use; destroyed through
  // the hook set with it (the host-only library never creates one)
  fg_plan *plan = nullptr;
  void (*destroyPlan)(fg_plan *) = nullptr;
};
