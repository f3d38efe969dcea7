// The reference's own assembly, run as a program — TEST INFRASTRUCTURE ONLY.
//
// Built by oracle/build.py (build_gmshfem_ref) from the reference's src/
// compiled where it lies, the gmsh stand-in of oracle/gmsh_shim/ and this
// project's mesh and reference-element sources (fem-g_gb300/host/). It builds
// one benchmark problem the way a GmshFEM user program does — mesh, Field or
// CompoundField, constraints, Formulation::integral, pre(), assemble() — on
// the reference's own classes (gmshfem::problem::Formulation and everything
// it calls), and writes what the reference produced: the CSR pattern and
// values of its MatrixFactory, the right-hand side, the DOF dictionary in its
// iteration order with the numbering of DofsManager, and the element DOF map
// of its FieldInterface::getIndices. Those outputs pin the oracle's
// restatement and the GPU path.
//
// One problem per process: the reference numbers fields with a process-wide
// counter (src/field/FieldInterface.cpp:137), and a field's tag enters every
// DOF key, so a second problem in one process would be numbered differently.
//
// usage: ref_assemble <out-file> <threads> <repeats> <kind> <dim> <m> <mesh_order> <space> <order> <gauss>
//                     <jitter> <seed> <k> <coef_mode> <dirichlet> <dirichlet_value> <source> <omega>
//                     <lame_sigma> <upper> <order2> [<coefficient programs>]
// (the fields of fg_problem_config in include/fem_g_gb300_host.h, in order).
// The optional last argument names a file of coefficient programs for the
// scalar (Helmholtz-type) problem, each "<term> <count>" followed by count
// lines "<op> <arg> <re> <im>" in the bytecode of include/fem_g_gb300.h:
// term "grad" (integral(g grad(dof u), grad(tf u))), "mass"
// (integral(m dof(u), tf(u))), "source" (integral(f, tf(u))), "damping" and
// "inertia" (integral(c dt_dof(u), tf(u)) and integral(c dt2_dof(u), tf(u)),
// and for the Maxwell problem "dcurl_0" .. "dcurl_8" and "dmass_0" ..
// "dmass_8" (integral(D curl(dof E), curl(tf E)), integral(D dof(E), tf(E))),
// at the angular frequency omega of the configuration), "mass_tf"
// (integral(dof(u), m tf(u)), the coefficient on the test side), "separate"
// (any program: assemble(separate = true), K, C and M written apart), "dfull_0" ..
// "dfull_8" (integral(D grad(dof u), grad(tf u)) with the general tensor D,
// row-major), "adv_0" .. "adv_2" (integral(b . grad(dof u), tf(u))), "vdof_0" ..
// "vdof_2" (integral(b dof(u), grad(tf u))) or "vsrc_0" .. "vsrc_2"
// (integral(f, grad(tf u)) with a vector f). The programs
// become the reference's own expression trees (x(), y(), z(), constants,
// + - * /, heaviside and the scalar operators of scalarUnaryOperators.h).
#include <algorithm>
#include <chrono>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "CompoundField.h"
#include "Domain.h"
#include "Field.h"
#include "Formulation.h"
#include "GmshFem.h"
#include "MatrixCRSFast.h"
#include "NullaryNode.h"
#include "Options.h"
#include "Vector.h"
#include "scalarNullaryOperators.h"
#include "scalarUnaryOperators.h"
#include "tensor4NovenaryOperators.h"
#include "tensorNovenaryOperators.h"
#include "vectorTernaryOperators.h"

#ifdef FEMG_DROPIN
#include "GpuFormulation.h"
#endif

#include "../fem-g_gb300/host/mesh.h"
#include "../include/fem_g_gb300_host.h"
#include "gmsh_shim/shim_model.h"

using T = std::complex<double>;
using namespace gmshfem;

// The drop-in program (ref_dropin, built with FEMG_DROPIN) runs the same
// problems through the GpuFormulation subclass of fem-g_gb300/binding/, whose
// assemble() calls the C ABI (here the recording stand-in of fg_record.cpp)
#ifdef FEMG_DROPIN
template <class S>
using FormulationOf = problem::GpuFormulation<S>;
#else
template <class S>
using FormulationOf = problem::Formulation<S>;
#endif

namespace {

// A coefficient with one value per element of the bucket, as a node of the
// reference's own expression trees: a user-defined nullary operation. The
// evaluator passes the physical points of every element of the bucket, nq
// per element in element order (EquationEvaluator::initialize,
// src/term/evaluator/EquationEvaluator.h:155-168), so point i belongs to
// element i / nq.
class ElementArray final : public function::NullaryOperation<T, Degree::Degree0> {
 public:
  explicit ElementArray(std::shared_ptr<const std::vector<T>> data) : _data(std::move(data)) {}
  ElementArray(const ElementArray &other) : function::NullaryOperation<T, Degree::Degree0>(other), _data(other._data) {}

  void operator()(function::OutputVector<T, Degree::Degree0> &values,
                  const std::vector<double, numa::allocator<double>> &points, const std::vector<double> &gaussPoints,
                  const int, const std::pair<int, int> &) const {
    const size_t nq = gaussPoints.size() / 3;
#pragma omp for
    for (auto i = 0ULL; i < values.size(); ++i) values[i] = (*_data)[i / nq];
    (void)points;
  }
  bool isConstant() const override { return false; }
  bool operator==(const ElementArray &other) const { return _data == other._data; }
  std::string name() const override { return "elementArray"; }

 private:
  std::shared_ptr<const std::vector<T>> _data;
};

function::ScalarFunction<T> elementArray(std::vector<T> values) {
  auto data = std::make_shared<const std::vector<T>>(std::move(values));
  return function::ScalarFunction<T>(new function::NullaryNode<ElementArray>(ElementArray(data)));
}

struct Instr {
  int op, arg;
  double re, im;
};

// A coefficient program as a reference expression tree (stack machine)
function::ScalarFunction<T> fromProgram(const std::vector<Instr> &code) {
  using F = function::ScalarFunction<T>;
  std::vector<F> st;
  for (const Instr &in : code) {
    if (in.op == FG_OP_CONST) {
      st.push_back(F(T(in.re, in.im)));
      continue;
    }
    if (in.op == FG_OP_X || in.op == FG_OP_Y || in.op == FG_OP_Z) {
      st.push_back(in.op == FG_OP_X ? function::x<T>() : in.op == FG_OP_Y ? function::y<T>() : function::z<T>());
      continue;
    }
    if (in.op >= FG_OP_ADD && in.op <= FG_OP_DIV) {
      F b = st.back();
      st.pop_back();
      F a = st.back();
      st.pop_back();
      st.push_back(in.op == FG_OP_ADD ? F(a + b) : in.op == FG_OP_SUB ? F(a - b) : in.op == FG_OP_MUL ? F(a * b) : F(a / b));
      continue;
    }
    F a = st.back();
    st.pop_back();
    switch (in.op) {
      case FG_OP_NEG: st.push_back(-a); break;
      case FG_OP_HEAVISIDE: st.push_back(function::heaviside(a)); break;
      case FG_OP_SQRT: st.push_back(function::sqrt(a)); break;
      case FG_OP_EXP: st.push_back(function::exp(a)); break;
      case FG_OP_LN: st.push_back(function::ln(a)); break;
      case FG_OP_LOG10: st.push_back(function::log(a)); break;
      case FG_OP_POW: st.push_back(function::pow(a, (unsigned)in.arg)); break;
      case FG_OP_CBRT: st.push_back(function::cbrt(a)); break;
      case FG_OP_SIN: st.push_back(function::sin(a)); break;
      case FG_OP_COS: st.push_back(function::cos(a)); break;
      case FG_OP_TAN: st.push_back(function::tan(a)); break;
      case FG_OP_SINH: st.push_back(function::sinh(a)); break;
      case FG_OP_COSH: st.push_back(function::cosh(a)); break;
      case FG_OP_TANH: st.push_back(function::tanh(a)); break;
      case FG_OP_ASIN: st.push_back(function::asin(a)); break;
      case FG_OP_ACOS: st.push_back(function::acos(a)); break;
      case FG_OP_ATAN: st.push_back(function::atan(a)); break;
      case FG_OP_ASINH: st.push_back(function::asinh(a)); break;
      case FG_OP_ACOSH: st.push_back(function::acosh(a)); break;
      case FG_OP_ATANH: st.push_back(function::atanh(a)); break;
      case FG_OP_ABS: st.push_back(function::abs(a)); break;
      case FG_OP_CONJ: st.push_back(function::conj(a)); break;
      case FG_OP_REAL: st.push_back(function::real(a)); break;
      case FG_OP_IMAG: st.push_back(function::imag(a)); break;
      default: throw std::runtime_error("coefficient program: operator " + std::to_string(in.op) + " not available");
    }
  }
  if (st.size() != 1) throw std::runtime_error("coefficient program: malformed");
  return st.back();
}

std::map<std::string, std::vector<Instr>> readPrograms(const char *path) {
  std::map<std::string, std::vector<Instr>> out;
  std::ifstream in(path);
  if (!in) throw std::runtime_error(std::string("cannot read ") + path);
  std::string term;
  int count = 0;
  while (in >> term >> count) {
    std::vector<Instr> code((size_t)count);
    for (auto &c : code) in >> c.op >> c.arg >> c.re >> c.im;
    out[term] = code;
  }
  return out;
}

double median(std::vector<double> v) {
  std::sort(v.begin(), v.end());
  return v.empty() ? 0.0 : v[v.size() / 2];
}

struct Writer {
  FILE *f;
  template <class V>
  void arr(const V *p, size_t n) {
    if (n && std::fwrite(p, sizeof(V), n, f) != n) throw std::runtime_error("write failed");
  }
  void u64(uint64_t v) { arr(&v, 1); }
  void f64(double v) { arr(&v, 1); }
};

template <class F>
void dumpField(F &u, Writer &w) {
  std::vector<uint64_t> nt, en, nd;
  std::vector<int32_t> at;
  for (auto it = u.begin(); it != u.end(); ++it) {
    nt.push_back(it->first->numType());
    en.push_back(it->first->entity());
    nd.push_back(it->first->numDof());
    at.push_back((int32_t)it->first->assembleType());
  }
  w.u64(nt.size());
  w.arr(nt.data(), nt.size());
  w.arr(en.data(), en.size());
  w.arr(nd.data(), nd.size());
  w.arr(at.data(), at.size());
}

// pre(), assemble() (repeats times), then the outputs: the CSR pattern and
// values, the right-hand side, the number of fields and each field's DOF
// dictionary, the timings
// assemble(separate = true) instead of assemble() (set by the "separate" program key)
bool g_separate = false;

template <class FORM, class... F>
void run(FORM &formulation, int repeats, Writer &w, F &...fields) {
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  formulation.pre();
  const double preSeconds = std::chrono::duration<double>(clock::now() - t0).count();
  std::vector<double> times;
  for (int r = 0; r < std::max(1, repeats); ++r) {
    formulation.setSystemToZero();
    const auto a0 = clock::now();
    common::Timer timer = formulation.assemble(g_separate);
    const double wall = std::chrono::duration<double>(clock::now() - a0).count();
    if (r > 0 || repeats == 1) times.push_back(wall);
    (void)timer;
  }
  // separate matrices: K in place of the system matrix, C and M after the timings
  algebra::MatrixCRSFast<T> A, Cm, Mm;
  if (g_separate) {
    formulation.getStiffness(A);
    formulation.getDamping(Cm);
    formulation.getMass(Mm);
  } else {
    formulation.getLHS(A);
  }
  algebra::Vector<T> b;
  formulation.getRHS(b);
  const uint64_t n = A.size(0);
  const uint64_t nnz = n ? A.ai()[n] : 0;
  w.u64(n);
  w.u64(nnz);
  w.arr(A.ai(), n + 1);
  w.arr(A.aj(), nnz);
  w.arr(A.a(), nnz);
  std::vector<T> rhs(n);
  for (uint64_t i = 0; i < n && i < b.size(); ++i) rhs[i] = b[i];
  w.arr(rhs.data(), n);
  w.u64(sizeof...(fields));
  (dumpField(fields, w), ...);
  w.f64(preSeconds);
  w.f64(median(times));
  w.u64(times.size());
  w.u64(g_separate ? 2 : 0);
  if (g_separate)
    for (auto *X : {&Cm, &Mm}) {  // zeros for a matrix the module does not hold
      std::vector<T> vals(nnz, T(0.0));
      if (X->size(0) == n && n && X->ai()[n] == nnz) std::copy(X->a(), X->a() + nnz, vals.begin());
      w.arr(vals.data(), nnz);
    }
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 22 && argc != 23) {
    std::fprintf(stderr, "usage: ref_assemble <out> <threads> <repeats> <fg_problem_config fields...>\n");
    return 2;
  }
  fg_problem_config c;
  std::memset(&c, 0, sizeof c);
  const char *out = argv[1];
  const int threads = std::atoi(argv[2]);
  const int repeats = std::atoi(argv[3]);
  int a = 4;
  c.kind = std::atoi(argv[a++]);
  c.dim = std::atoi(argv[a++]);
  c.m = std::atoi(argv[a++]);
  c.mesh_order = std::atoi(argv[a++]);
  c.space = std::atoi(argv[a++]);
  c.order = std::atoi(argv[a++]);
  c.gauss = std::atoi(argv[a++]);
  c.jitter = std::atof(argv[a++]);
  c.seed = std::strtoull(argv[a++], nullptr, 10);
  c.k = std::atof(argv[a++]);
  c.coef_mode = std::atoi(argv[a++]);
  c.dirichlet = std::atoi(argv[a++]);
  c.dirichlet_value = std::atof(argv[a++]);
  c.source = std::atoi(argv[a++]);
  c.omega = std::atof(argv[a++]);
  c.lame_sigma = std::atof(argv[a++]);
  c.upper = std::atoi(argv[a++]);
  c.order2 = std::atoi(argv[a++]);

  char arg0[] = "ref_assemble";
  char *gargv[] = {arg0, nullptr};
  common::GmshFem gmshFem(1, gargv);
  common::Options::instance()->verbose = 0;
  common::Options::instance()->maxThreads = threads;

  // the mesh, as gmsh would hold it
  femg::Mesh mesh = c.dim == 2 ? femg::makeSquareTri(c.m, c.mesh_order, c.jitter, c.seed)
                               : femg::makeCubeTet(c.m, c.mesh_order, c.jitter, c.seed);
  const int64_t E = mesh.find(c.dim, 1)->blocks[0].size();
  oracleShimSetMesh(std::move(mesh));

  FILE *f = std::fopen(out, "wb");
  if (!f) {
    std::perror(out);
    return 1;
  }
  Writer w{f};
  const uint64_t magic = 0x46454d4752454631ull;  // "FEMGREF1"
  w.u64(magic);
  const std::string gauss = "Gauss" + std::to_string(c.gauss);
  try {
    domain::Domain omega("omega");
    // Symmetric storage: the matrix options string given to the Formulation
    // is cleared again when pre() initialises the MatrixFactory
    // (MatrixFactory::init -> removeMatrix -> MatrixOptions::clean,
    // src/system/MatrixFactory.cpp:100-134), which keeps only the global
    // option, the reference's -forceSymmetric switch
    common::Options::instance()->forceSymmetric = c.upper != 0;
    const std::string matrixOptions = c.upper ? "Symmetric" : "";
    if (c.kind == FG_PROBLEM_HELMHOLTZ && argc == 23) {
      // the terms from the coefficient programs
      auto progs = readPrograms(argv[22]);
      g_separate = progs.count("separate") != 0;
      const bool lagrange = c.space == FG_SPACE_LAGRANGE;
      field::Field<T, field::Form::Form0> u("u", omega,
                                            lagrange ? field::FunctionSpaceTypeForm0::Lagrange
                                                     : field::FunctionSpaceTypeForm0::HierarchicalH1,
                                            lagrange ? c.mesh_order : c.order);
      if (c.dirichlet) u.addConstraint(domain::Domain("gammaDir"), T(c.dirichlet_value, 0.0));
      FormulationOf<T> formulation("coefficients", matrixOptions);
      if (progs.count("dfull_0")) {  // a general TensorFunction, row-major programs dfull_0 .. dfull_8
        std::vector<function::ScalarFunction<T>> d;
        for (int k = 0; k < 9; ++k) d.push_back(fromProgram(progs["dfull_" + std::to_string(k)]));
        formulation.integral(function::tensor<T>(d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]) *
                                 equation::grad(equation::dof(u)),
                             equation::grad(equation::tf(u)), omega, gauss);
      }
      if (progs.count("adv_0"))  // a VectorFunction times grad(dof u), tested against tf(u)
        formulation.integral(function::vector<T>(fromProgram(progs["adv_0"]), fromProgram(progs["adv_1"]),
                                                 fromProgram(progs["adv_2"])) *
                                 equation::grad(equation::dof(u)),
                             equation::tf(u), omega, gauss);
      if (progs.count("vdof_0"))  // a VectorFunction times dof(u), tested against grad(tf(u))
        formulation.integral(function::vector<T>(fromProgram(progs["vdof_0"]), fromProgram(progs["vdof_1"]),
                                                 fromProgram(progs["vdof_2"])) *
                                 equation::dof(u),
                             equation::grad(equation::tf(u)), omega, gauss);
      if (progs.count("vsrc_0"))  // a VectorFunction source tested against grad(tf(u))
        formulation.integral(function::vector<T>(fromProgram(progs["vsrc_0"]), fromProgram(progs["vsrc_1"]),
                                                 fromProgram(progs["vsrc_2"])),
                             equation::grad(equation::tf(u)), omega, gauss);
      if (progs.count("grad"))
        formulation.integral(fromProgram(progs["grad"]) * equation::grad(equation::dof(u)), equation::grad(equation::tf(u)),
                             omega, gauss);
      if (progs.count("mass"))
        formulation.integral(fromProgram(progs["mass"]) * equation::dof(u), equation::tf(u), omega, gauss);
      if (progs.count("source")) formulation.integral(fromProgram(progs["source"]), equation::tf(u), omega, gauss);
      // time derivatives of the unknown, assembled at the angular frequency omega by the AFrequency module
      if (progs.count("damping"))
        formulation.integral(fromProgram(progs["damping"]) * equation::dt_dof(u), equation::tf(u), omega, gauss);
      if (progs.count("inertia"))
        formulation.integral(fromProgram(progs["inertia"]) * equation::dt2_dof(u), equation::tf(u), omega, gauss);
      if (progs.count("damping") || progs.count("inertia")) formulation.setAngularFrequency(c.omega);
      // a coefficient on the test function's side
      if (progs.count("mass_tf"))
        formulation.integral(equation::dof(u), fromProgram(progs["mass_tf"]) * equation::tf(u), omega, gauss);
      run(formulation, repeats, w, u);
    } else if (c.kind == FG_PROBLEM_HELMHOLTZ) {
      const bool lagrange = c.space == FG_SPACE_LAGRANGE;
      field::Field<T, field::Form::Form0> u("u", omega,
                                            lagrange ? field::FunctionSpaceTypeForm0::Lagrange
                                                     : field::FunctionSpaceTypeForm0::HierarchicalH1,
                                            lagrange ? c.mesh_order : c.order);
      if (c.dirichlet) u.addConstraint(domain::Domain("gammaDir"), T(c.dirichlet_value, 0.0));
      FormulationOf<T> formulation("helmholtz", matrixOptions);
      formulation.integral(equation::grad(equation::dof(u)), equation::grad(equation::tf(u)), omega, gauss);
      if (c.coef_mode == FG_COEF_MODE_CONSTANT) {
        formulation.integral(function::ScalarFunction<T>(T(-c.k * c.k, 0.0)) * equation::dof(u), equation::tf(u), omega,
                             gauss);
      } else {
        // c_e = -k^2 (1 + 0.3 xi_e), xi_e ~ N(0,1) per element in element order
        femg::Rng rng(c.seed + 1);
        std::vector<T> ce((size_t)E);
        for (int64_t e = 0; e < E; ++e) ce[(size_t)e] = T(-c.k * c.k * (1.0 + 0.3 * rng.normal()), 0.0);
        formulation.integral(elementArray(std::move(ce)) * equation::dof(u), equation::tf(u), omega, gauss);
      }
      if (c.source) {
        function::ScalarFunction<T> x = function::x<T>(), y = function::y<T>();
        function::ScalarFunction<T> fsrc = function::heaviside<T>(0.01 - (x - 0.5) * (x - 0.5) - (y - 0.5) * (y - 0.5));
        formulation.integral(-fsrc, equation::tf(u), omega, gauss);
      }
      run(formulation, repeats, w, u);
    } else if (c.kind == FG_PROBLEM_COUPLED) {
      // two scalar fields, coupled both ways (the problem of fg_problem_config)
      const bool lagrange = c.space == FG_SPACE_LAGRANGE;
      const auto type = lagrange ? field::FunctionSpaceTypeForm0::Lagrange : field::FunctionSpaceTypeForm0::HierarchicalH1;
      const int orderU = lagrange ? c.mesh_order : c.order;
      const int orderV = lagrange ? c.mesh_order : (c.order2 > 0 ? c.order2 : c.order);
      field::Field<T, field::Form::Form0> u("u", omega, type, orderU);
      field::Field<T, field::Form::Form0> v("v", omega, type, orderV);
      if (c.dirichlet) u.addConstraint(domain::Domain("gammaDir"), T(c.dirichlet_value, 0.0));
      FormulationOf<T> formulation("coupled", matrixOptions);
      function::ScalarFunction<T> x = function::x<T>(), y = function::y<T>();
      formulation.integral(equation::grad(equation::dof(u)), equation::grad(equation::tf(u)), omega, gauss);
      formulation.integral(function::ScalarFunction<T>(T(-c.k * c.k, 0.0)) * equation::dof(u), equation::tf(u), omega, gauss);
      formulation.integral(equation::grad(equation::dof(v)), equation::grad(equation::tf(v)), omega, gauss);
      formulation.integral(function::ScalarFunction<T>(T(2.0, 0.0)) * equation::dof(v), equation::tf(v), omega, gauss);
      formulation.integral((0.5 + x) * equation::dof(u), equation::tf(v), omega, gauss);
      formulation.integral(function::vector<T>(function::ScalarFunction<T>(T(1.0, 0.0)), function::ScalarFunction<T>(T(-0.5, 0.2)),
                                               function::ScalarFunction<T>(T(0.25, 0.0))) *
                               equation::grad(equation::dof(u)),
                           equation::tf(v), omega, gauss);
      formulation.integral(function::ScalarFunction<T>(T(0.3, 0.0)) * equation::grad(equation::dof(v)), equation::grad(equation::tf(u)),
                           omega, gauss);
      if (c.source) {
        function::ScalarFunction<T> fsrc = function::heaviside<T>(0.01 - (x - 0.5) * (x - 0.5) - (y - 0.5) * (y - 0.5));
        formulation.integral(-fsrc, equation::tf(u), omega, gauss);
        formulation.integral(1.0 + x * y, equation::tf(v), omega, gauss);
      }
      run(formulation, repeats, w, u, v);
    } else if (c.kind == FG_PROBLEM_MAXWELL) {
      field::Field<T, field::Form::Form1> u("u", omega, field::FunctionSpaceTypeForm1::HierarchicalHCurl, c.order);
      FormulationOf<T> formulation("maxwell", matrixOptions);
      std::map<std::string, std::vector<Instr>> progs;
      if (argc == 23) progs = readPrograms(argv[22]);
      auto tensorOf = [&](const std::string &name) {  // programs name_0 .. name_8, row-major
        std::vector<function::ScalarFunction<T>> d;
        for (int k = 0; k < 9; ++k) d.push_back(fromProgram(progs[name + "_" + std::to_string(k)]));
        return function::tensor<T>(d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]);
      };
      // anisotropic media: TensorFunction * curl and TensorFunction * dof (the PML form)
      if (progs.count("dcurl_0"))
        formulation.integral(tensorOf("dcurl") * equation::curl(equation::dof(u)), equation::curl(equation::tf(u)), omega, gauss);
      if (progs.count("dmass_0"))
        formulation.integral(tensorOf("dmass") * equation::dof(u), equation::tf(u), omega, gauss);
      formulation.integral(equation::curl(equation::dof(u)), equation::curl(equation::tf(u)), omega, gauss);
      if (c.coef_mode == FG_COEF_MODE_CONSTANT) {
        formulation.integral(function::ScalarFunction<T>(T(-c.k * c.k, 0.0)) * equation::dof(u), equation::tf(u), omega,
                             gauss);
      } else {
        femg::Rng rng(c.seed + 1);
        std::vector<T> ce((size_t)E);
        for (int64_t e = 0; e < E; ++e) ce[(size_t)e] = T(-c.k * c.k * (1.0 + 0.3 * rng.normal()), 0.0);
        formulation.integral(elementArray(std::move(ce)) * equation::dof(u), equation::tf(u), omega, gauss);
      }
      run(formulation, repeats, w, u);
    } else if (c.kind == FG_PROBLEM_NAVIER) {
      field::CompoundField<T, field::Form::Form0, 3> u("u", omega, field::FunctionSpaceTypeForm0::HierarchicalH1, c.order);
      FormulationOf<T> formulation("navier", matrixOptions);
      // lambda, mu ~ lognormal(median 1, sigma) per element, drawn in element order
      femg::Rng rng(c.seed + 2);
      std::vector<T> lam((size_t)E), mu((size_t)E);
      for (int64_t e = 0; e < E; ++e) {
        lam[(size_t)e] = std::exp(c.lame_sigma * rng.normal());
        mu[(size_t)e] = std::exp(c.lame_sigma * rng.normal());
      }
      function::ScalarFunction<T> L = elementArray(std::move(lam)), M = elementArray(std::move(mu));
      function::ScalarFunction<T> zero(T(0.0, 0.0));
      function::ScalarFunction<T> L2M = L + 2.0 * M;
      // isotropic C_ijkl = lambda d_ij d_kl + mu (d_ik d_jl + d_il d_jk): block (i, j), entry (k, l)
      auto blockOf = [&](int i, int j) {
        function::ScalarFunction<T> e[9] = {zero, zero, zero, zero, zero, zero, zero, zero, zero};
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) {
            const bool lamTerm = i == j && k == l;
            const bool mu1 = i == k && j == l, mu2 = i == l && j == k;
            if (lamTerm && mu1 && mu2) e[3 * k + l] = L2M;
            else if (lamTerm) e[3 * k + l] = L;
            else if (mu1 || mu2) e[3 * k + l] = M;
          }
        return function::tensor<T>(e[0], e[1], e[2], e[3], e[4], e[5], e[6], e[7], e[8]);
      };
      function::TensorFunction<T, 4> C = function::tensor<T, 4>(blockOf(0, 0), blockOf(0, 1), blockOf(0, 2), blockOf(1, 0),
                                                             blockOf(1, 1), blockOf(1, 2), blockOf(2, 0), blockOf(2, 1),
                                                             blockOf(2, 2));
      formulation.integral(C * equation::grad(equation::dof(u)), equation::grad(equation::tf(u)), omega, gauss);
      if (c.omega > 0.0) {
        formulation.integral(function::ScalarFunction<T>(T(-c.omega * c.omega, 0.0)) * equation::dof(u), equation::tf(u),
                             omega, gauss);
      } else {
        formulation.integral(equation::dt2_dof(u), equation::tf(u), omega, gauss);
      }
      run(formulation, repeats, w, u);
    } else {
      throw std::runtime_error("unknown problem kind");
    }
  } catch (const std::exception &e) {
    std::fprintf(stderr, "ref_assemble: %s\n", e.what());
    std::fclose(f);
    return 1;
  }
  std::fclose(f);
  return 0;
}
