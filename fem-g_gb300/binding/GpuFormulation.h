// GpuFormulation<T>: GmshFEM's Formulation<T> with assemble() on the GB300
// path, the reference-side binding of the C ABI (include/fem_g_gb300.h).
//
// A maintainer adds this header to GmshFEM (it includes GmshFEM's own
// headers and links libfemg.so); a user program changes only the type of its
// formulation. pre() stays the reference's (DOF dictionary, Hilbert
// numbering, CSR pattern: Formulation::pre, src/problem/Formulation.cpp:
// 897-1039). assemble() replaces Formulation::assemble
// (src/problem/Formulation.cpp:1152-1215) and its _assembleDim loop
// (:1418-1493): one plan per (entity, element type) bucket of the terms,
// built from the same sources the reference's Assembler reads,
//  - the mesh: gmsh::model::mesh::getElementsByType / getNodesByElementType;
//  - the rule: FunctionSpaceInterface::getGaussInfo (GetGaussInfo,
//    src/field/FunctionSpaceInterface.cpp:470-481) and the geometric
//    Lagrange basis of gmsh::model::mesh::getBasisFunctions;
//  - the space: FunctionSpaceInterface::getBasisFunctions with the dense
//    orientations (src/field/FunctionSpaceHierarchicalH1.cpp:83-109);
//  - the DOF map: FunctionSpaceInterface::getKeys and FieldInterface::
//    getIndices (src/field/FieldInterface.cpp:959-976), the pattern through
//    getLHS (MatrixCRSFast, a friend of MatrixFactory), the Dirichlet values
//    through FieldInterface::getFixedValues (s_setDirichletConditions,
//    Formulation.cpp:1041-1054);
//  - the terms: recorded where integral() is called. The reference keeps a
//    term's equations inside the term, out of reach, so the subclass hides
//    integral() with a template that forwards to the reference's overloads
//    and keeps a copy of the equations (EquationInterface::copy). Their
//    coefficients are not described but evaluated by the reference's own
//    evaluators at the bucket's integration points
//    (EquationEvaluatorInterface::initialize and operator(),
//    src/term/evaluator/EquationEvaluator.h:86-103; Function::evaluate for
//    sources), and passed as constants, per-element arrays (FG_OP_ELEM) or
//    point tables (FG_OP_POINT), whichever the values are.
// assemble(separate = true) takes fg_assemble_separate into the MCK, MK or CK
// module's matrices, as the reference does. Terms this binding does not map (Tensor4 coefficients that are not
// isotropic, vector products, compound-field terms other than mass and the
// elastic Tensor4, two-field terms of HCurl or compound fields, Jacobian
// modificators, linked DOFs, coefficients or time derivatives on the test
// function) make assemble() fail with the
// reference's convention: an error message and zero A and b
// (Formulation.cpp:1200-1209). They are assembled by GPU plans through the
// C ABI directly (term kinds FG_TERM_*), or by Formulation<T> itself.
#ifndef FEMG_GPU_FORMULATION_H
#define FEMG_GPU_FORMULATION_H

#include <algorithm>
#include <cmath>
#include <complex>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "Equation.h"
#include "EquationEvaluator.h"
#include "FieldInterface.h"
#include "Formulation.h"
#include "FunctionSpaceInterface.h"
#include "MatrixCRSFast.h"
#include "MatrixFactory.h"
#include "MatrixModule.h"
#include "Message.h"
#include "OmpInterface.h"
#include "UnknownField.h"
#include "VectorFactory.h"
#include "fem_g_gb300.h"
#include "gmsh.h"
#include "numa.h"

namespace gmshfem::problem {

template <class T>
class GpuFormulation : public Formulation<T> {
  static_assert(std::is_same<T, std::complex<double>>::value, "the GB300 path assembles complex<double> systems");
  using PointVec = std::vector<double, numa::allocator<double>>;

  // One side of a term: an equation (the unknown's or the test function's)
  // or the source function of a linear term
  struct Side {
    virtual ~Side() = default;
    virtual field::FieldInterface<T> *field() const { return nullptr; }
    virtual field::Form form() const { return field::Form::Form0; }
    virtual bool derivative() const { return false; }
    virtual int dt() const { return FG_DT_NONE; }  // FG_DT_*: the unknown's time derivative
    // the coefficient's components: 1 (scalar), 3 (vector) or 9 (tensor, row-major)
    virtual int components() const { return 1; }
    // the coefficient at the points (x, y, z) [n][3] of the bucket, element-major:
    // [1][components] when it is constant, else [n][components]
    virtual void values(const PointVec &points, const std::vector<double> &gauss, int elementType,
                        const std::pair<int, int> &entity, std::vector<T> &out) const = 0;
  };

  // c * (dof or tf, gradient or value): the reference's EquationLhs<T, DC, F,
  // ScalarProduct> with a coefficient c of degree DC. Its evaluator applies c
  // to a field (EquationEvaluator.h:107-131, :198-325): a scalar c scales it,
  // a vector b gives b^T field (F a vector form: b . grad) or b field (F =
  // Form0: b times a value), a tensor D gives D field. So a unit field (1 x 1,
  // or the 3 x 3 identity) gives the coefficient itself at each point.
  template <Degree DC, field::Form F>
  struct EquationSide final : Side {
    using Eq = equation::EquationLhs<T, DC, F, equation::Product::ScalarProduct>;
    std::unique_ptr<Eq> eq;
    explicit EquationSide(const Eq &e) : eq(e.copy()) {}
    field::FieldInterface<T> *field() const override { return eq->getField(); }
    field::Form form() const override { return eq->form(); }
    bool derivative() const override { return eq->isDerivative(); }
    int dt() const override {
      const auto *u = eq->getUnknownField();
      if (!u) return FG_DT_NONE;
      if (u->type() == equation::UnknownFieldType::Dt) return FG_DT_1;
      return u->type() == equation::UnknownFieldType::DtDt ? FG_DT_2 : FG_DT_NONE;  // NotDt, or Tf for tf()
    }
    int components() const override { return DC == Degree::Degree0 ? 1 : DC == Degree::Degree1 ? 3 : 9; }
    void values(const PointVec &points, const std::vector<double> &gauss, int elementType, const std::pair<int, int> &entity,
                std::vector<T> &out) const override {
      std::unique_ptr<term::evaluator::EquationEvaluatorInterface<T, F>> ev(eq->getEquationEvaluator());
      ev->initialize(points, gauss, elementType, entity);
      const size_t n = ev->isConstant(entity) ? 1 : points.size() / 3;
      const int nc = components();
      const bool unit3 = DC == Degree::Degree2 || (DC == Degree::Degree1 && F != field::Form::Form0);
      Eigen::MatrixX<double> unit = Eigen::MatrixX<double>::Ones(1, 1);
      if (unit3) unit = Eigen::MatrixX<double>::Identity(3, 3);
      const int rows = DC == Degree::Degree0 ? 1 : DC == Degree::Degree1 ? (F == field::Form::Form0 ? 3 : 1) : 3;
      Eigen::MatrixX<T> value(rows, unit.cols());
      out.resize(n * nc);
      for (size_t k = 0; k < n; ++k) {
        (*ev)(value, unit, (unsigned int)k);
        for (int c = 0; c < nc; ++c) out[k * nc + c] = nc == 9 ? value(c / 3, c % 3) : rows == 1 ? value(0, c) : value(c, 0);
      }
      ev->clear();
    }
  };

  // c * (dof or tf, gradient or value) of a compound field of three
  // components (a vector H1 field): the reference's EquationLhsCompound<T, DC,
  // F, ScalarProduct, 3>. A scalar c scales the field
  // (EquationEvaluator.h:832-895); a Tensor4 C maps a gradient u_kl to C_ijkl
  // u_kl (:1222-1290), so the nine unit gradients give its 81 entries,
  // C_ijkl at (i + 3 j, k + 3 l)... in the evaluator's column order
  // (column m is the unit gradient with k = m % 3, l = m / 3).
  template <Degree DC, field::Form F>
  struct CompoundSide final : Side {
    using Eq = equation::EquationLhsCompound<T, DC, F, equation::Product::ScalarProduct, 3>;
    std::unique_ptr<Eq> eq;
    explicit CompoundSide(const Eq &e) : eq(e.copy()) {}
    field::FieldInterface<T> *field() const override { return eq->getField(); }
    field::Form form() const override { return eq->form(); }
    bool derivative() const override { return eq->isDerivative(); }
    int dt() const override {
      const auto *u = eq->getUnknownField();
      if (!u) return FG_DT_NONE;
      if (u->type() == equation::UnknownFieldType::Dt) return FG_DT_1;
      return u->type() == equation::UnknownFieldType::DtDt ? FG_DT_2 : FG_DT_NONE;
    }
    int components() const override { return DC == Degree::Degree0 ? 1 : 81; }
    void values(const PointVec &points, const std::vector<double> &gauss, int elementType, const std::pair<int, int> &entity,
                std::vector<T> &out) const override {
      std::unique_ptr<term::evaluator::EquationEvaluatorInterface<T, F>> ev(eq->getEquationEvaluator());
      ev->initialize(points, gauss, elementType, entity);
      const size_t n = ev->isConstant(entity) ? 1 : points.size() / 3;
      const int nc = components();
      Eigen::MatrixX<double> unit = Eigen::MatrixX<double>::Ones(1, 1);
      if (nc == 81) unit = Eigen::MatrixX<double>::Identity(9, 9);
      Eigen::MatrixX<T> value(nc == 81 ? 9 : 1, unit.cols());
      out.resize(n * nc);
      for (size_t k = 0; k < n; ++k) {
        (*ev)(value, unit, (unsigned int)k);
        for (int c = 0; c < nc; ++c) out[k * nc + c] = nc == 81 ? value(c / 9, c % 9) : value(0, 0);
      }
      ev->clear();
    }
  };

  // the source function f of integral(f, tf(u)) (scalar) or integral(f, grad(tf(u))) (vector)
  template <Degree D>
  struct FunctionSide final : Side {
    function::Function<T, D> f;
    explicit FunctionSide(const function::Function<T, D> &g) : f(g) {}
    int components() const override { return D == Degree::Degree0 ? 1 : 3; }
    void values(const PointVec &points, const std::vector<double> &gauss, int elementType, const std::pair<int, int> &entity,
                std::vector<T> &out) const override {
      using V = typename MathObject<T, D>::Object;
      std::vector<V, numa::allocator<V>> v(1);
      if (f.isConstant(entity)) f.evaluate(v[0], 0., 0., 0., entity);
      else {
#pragma omp parallel num_threads(omp::getMaxThreads())
        f.evaluate(v, points, gauss, elementType, entity);
      }
      const int nc = components();
      out.resize(v.size() * nc);
      for (size_t k = 0; k < v.size(); ++k) {
        if constexpr (D == Degree::Degree0) out[k] = v[k];
        else
          for (int c = 0; c < 3; ++c) out[k * 3 + c] = v[k](c);
      }
    }
  };

  struct Recorded {
    std::unique_ptr<Side> lhs, rhs;  // lhs: the unknown's side or the source; rhs: the test function's
    bool bilinear = false;
    std::vector<std::pair<int, int>> entities;
    bool jacobianModificators = false;
    std::string integrationType;
    std::string unsupported;  // why the term cannot take the GPU path
    int kind = -1;            // FG_TERM_*
  };

  // The term kind of a recorded term: scalar coefficients on grad-grad (or
  // curl-curl) and mass; on scalar H1 fields also a vector b with
  // (b . grad dof, tf) and (b dof, grad tf), a tensor D with (D grad dof,
  // grad tf), and sources f (tf) and vector f (grad tf)
  static int kindOf(const Recorded &r) {
    const int nc = r.lhs->components();
    if (r.rhs->field()->multiplicity() == 3) {  // compound: mass, and an isotropic Tensor4 on the gradients
      if (nc == 1 && !r.lhs->derivative() && !r.rhs->derivative()) return FG_TERM_MASS;
      if (nc == 81 && r.lhs->derivative() && r.rhs->derivative()) return FG_TERM_ELASTIC;
      return -1;
    }
    const bool h1 = r.rhs->field()->form() == field::Form::Form0;
    const bool gl = r.lhs->derivative(), gr = r.rhs->derivative();
    if (!r.bilinear) {
      if (nc == 1 && !gr) return FG_TERM_SOURCE;
      if (nc == 3 && gr && h1) return FG_TERM_SOURCE_GRAD;
      return -1;
    }
    if (nc == 1) return gl == gr ? (gl ? FG_TERM_GRAD_GRAD : FG_TERM_MASS) : -1;
    if (!h1) {  // HCurl: a symmetric tensor on the curls or on the values (the PML form)
      if (nc == 9 && gl && gr) return FG_TERM_GRAD_GRAD_TENSOR;
      if (nc == 9 && !gl && !gr) return FG_TERM_MASS_TENSOR;
      return -1;
    }
    if (nc == 3 && gl && !gr) return FG_TERM_ADVECTION;
    if (nc == 3 && !gl && gr) return FG_TERM_VECTOR_GRAD_TEST;
    if (nc == 9 && gl && gr) return FG_TERM_GRAD_GRAD_TENSOR_FULL;
    return -1;
  }
  std::vector<Recorded> _recorded;

  template <Degree DC, field::Form F, equation::Product P>
  static std::unique_ptr<Side> side(const equation::EquationLhs<T, DC, F, P> &e) {
    if constexpr (P == equation::Product::ScalarProduct && DC != Degree::Degree4) return std::make_unique<EquationSide<DC, F>>(e);
    else return nullptr;
  }
  template <Degree DC, field::Form F, equation::Product P, unsigned int N>
  static std::unique_ptr<Side> side(const equation::EquationLhsCompound<T, DC, F, P, N> &e) {
    if constexpr (N == 3 && P == equation::Product::ScalarProduct && (DC == Degree::Degree0 || DC == Degree::Degree4))
      return std::make_unique<CompoundSide<DC, F>>(e);
    else return nullptr;
  }
  template <field::Form F, unsigned int N>
  static std::unique_ptr<Side> side(const equation::UnknownCompoundField<T, F, N> &u) {
    const equation::UnknownCompoundField<T, F, N> *own = u.copy();
    return side(static_cast<equation::EquationLhsCompound<T, Degree::Degree0, F, equation::Product::ScalarProduct, N>>(*own));
  }
  // dof(u), tf(u), grad(...): the equation made from an unknown field owns and
  // deletes it (Equation.cpp:19-34), and the reference's integral() makes
  // one from the object the user passed, so the side is made from a copy
  template <field::Form F>
  static std::unique_ptr<Side> side(const equation::UnknownField<T, F> &u) {
    const equation::UnknownField<T, F> *own = u.copy();
    return side(static_cast<equation::EquationLhs<T, Degree::Degree0, F, equation::Product::ScalarProduct>>(*own));
  }
  // a scalar or vector source function (ScalarFunction, VectorFunction and the other Function types), or a form not mapped
  template <class O>
  static std::unique_ptr<Side> side(const O &o) {
    if constexpr (std::is_base_of<function::Function<T, Degree::Degree0>, O>::value)
      return std::make_unique<FunctionSide<Degree::Degree0>>(o);
    else if constexpr (std::is_base_of<function::Function<T, Degree::Degree1>, O>::value)
      return std::make_unique<FunctionSide<Degree::Degree1>>(o);
    else return nullptr;
  }

 public:
  using Formulation<T>::Formulation;
  ~GpuFormulation() override { releasePlans(); }

  // integral() of the reference, and the record of the term for assemble()
  template <class L, class R>
  unsigned int integral(const L &lhs, const R &rhs, const domain::GeometricObject &domain, const std::string &integrationType,
                        const term::ProductType productType = term::ProductType::Hermitian) {
    // the sides are copied first: the reference's integral() takes over the
    // unknown-field objects that dof() and tf() made
    Recorded r;
    r.lhs = side(lhs);
    r.rhs = side(rhs);
    const unsigned int tag = Formulation<T>::integral(lhs, rhs, domain, integrationType, productType);
    r.integrationType = integrationType;
    for (auto it = domain.cbegin(); it != domain.cend(); ++it) {
      r.entities.push_back(*it);
      r.jacobianModificators = r.jacobianModificators || domain.haveJacobiansModificators(*it);
    }
    if (!r.lhs || !r.rhs) r.unsupported = "a coefficient or product of another form (Tensor4, vector products)";
    else {
      r.bilinear = r.lhs->field() != nullptr;
      if (!r.rhs->field()) r.unsupported = "no test function";
      else if (r.jacobianModificators) r.unsupported = "Jacobian modificators";
      else if (r.rhs->dt() != FG_DT_NONE) r.unsupported = "a time derivative of the test function";
      else if (r.bilinear && r.lhs->field() != r.rhs->field() &&
               (r.lhs->field()->form() != field::Form::Form0 || r.rhs->field()->form() != field::Form::Form0 ||
                r.lhs->field()->multiplicity() != 1 || r.rhs->field()->multiplicity() != 1))
        r.unsupported = "two fields that are not both scalar H1 fields";
      else if (!(r.rhs->field()->form() == field::Form::Form0 &&
                 (r.rhs->field()->multiplicity() == 1 || r.rhs->field()->multiplicity() == 3)) &&
               !(r.rhs->field()->form() == field::Form::Form1 && r.rhs->field()->multiplicity() == 1))
        r.unsupported = "a field that is not a scalar or three-component H1 field or an HCurl field";
      else if (!r.bilinear && r.rhs->field()->multiplicity() != 1) r.unsupported = "a source on a compound field";
      else if (!r.bilinear && r.rhs->field()->form() != field::Form::Form0) r.unsupported = "a source on an HCurl field";
      else if (productType != term::ProductType::Hermitian) r.unsupported = "a product other than the hermitian one";
      else if (r.rhs->components() != 1) r.unsupported = "a coefficient on the test function";
      else r.kind = kindOf(r);
      if (r.unsupported.empty() && r.kind < 0) r.unsupported = "a coefficient of this degree on these operators";
    }
    _recorded.push_back(std::move(r));
    return tag;
  }

  void removeTerms() override {
    releasePlans();
    _recorded.clear();
    Formulation<T>::removeTerms();
  }

  common::Timer pre(const DofsSort::Algorithm algo = common::Options::instance()->dofsSortAlgorithm) override {
    releasePlans();
    return Formulation<T>::pre(algo);  // numbering and pattern stay the reference's
  }

  common::Timer assemble(const bool separate = false,
                         const ElementsSort::Algorithm algo = common::Options::instance()->elementsSortAlgorithm) override {
    common::Timer time;
    time.tick();
    try {
      assembleOnGpu(separate);
    } catch (const std::exception &e) {
      msg::error << "Unable to assemble the system" << msg::endl;
      msg::error << e.what() << msg::endl;
      this->_A->setToZero();
      for (auto &bi : this->_multiB) bi.setToZero();
    }
    (void)algo;
    time.tock();
    return time;
  }

 private:
  struct Bucket {
    std::pair<int, int> entity;
    int elementType;
    std::string integrationType;
    field::FieldInterface<T> *field;    // the test field: the rows
    field::FieldInterface<T> *unknown;  // the unknown field: the columns (the test field's for linear terms)
    std::vector<const Recorded *> terms;
  };
  std::map<std::string, fg_plan *> _plans;

  void releasePlans() {
    for (auto &kv : _plans) fg_plan_destroy(kv.second);
    _plans.clear();
  }

  static void check(int status) {
    if (status != FG_OK) throw std::runtime_error(fg_last_error());
  }

  void assembleOnGpu(bool separate) {
    const unsigned long long nRows = this->_dofs.nbrUnknownDofs();
    if (this->numRHS() != this->_multiB.size()) {
      this->_multiB.clear();
      this->_multiB.resize(this->numRHS());
    }
    for (auto &bi : this->_multiB) bi.init(nRows);
    // the module of s_setModule (Formulation.cpp:1096-1149): with time
    // derivatives the AFrequency one, whose single matrix is K + i w C - w^2 M;
    // separate matrices: the MCK, MK or CK one (K, C and M apart)
    if (this->_A->getModule() == nullptr) {
      bool k = false, c = false, m = false;
      for (const auto &r : _recorded)
        if (r.bilinear && r.lhs) {
          const int dt = r.lhs->dt();
          k = k || dt == FG_DT_NONE;
          c = c || dt == FG_DT_1;
          m = m || dt == FG_DT_2;
        }
      if (separate && m && c && k) this->_A->setModule(new system::MCKModule<T>(this->_A));
      else if (separate && m && !c && k) this->_A->setModule(new system::MKModule<T>(this->_A));
      else if (separate && !m && c && k) this->_A->setModule(new system::CKModule<T>(this->_A));
      else if (!separate && (m || c)) {
        auto *mod = new system::AFrequencyModule<T>(this->_A);
        mod->setFrequency(this->_frequency);
        this->_A->setModule(mod);
      } else {
        this->_A->setModule(new system::AModule<T>(this->_A));  // separate without M or C: the reference warns and does this
      }
    }
    const std::string moduleName = this->_A->getModule()->name();
    const bool split = moduleName == "MCK" || moduleName == "MK" || moduleName == "CK";
    if (this->_dofs.nbrLinkedDofs() != 0) throw std::runtime_error("linked DOFs: not mapped by this binding");
    for (const auto &r : _recorded)
      if (!r.unsupported.empty()) throw std::runtime_error("a term takes no GPU path here: " + r.unsupported);
    if (nRows == 0) return;
    // Dirichlet values (s_setDirichletConditions)
    std::vector<T> valuesDC(this->_dofs.nbrFixedDofs());
    for (auto &uf : this->_unknownFields) uf.second->getFixedValues(valuesDC);
    // the pattern of pre() (any of the module's matrices carries it)
    algebra::MatrixCRSFast<T> A;
    if (split) this->getStiffness(A);
    else this->getLHS(A);
    const unsigned long long nnz = A.ai()[nRows];
    std::vector<uint64_t> ai(A.ai(), A.ai() + nRows + 1), aj(A.aj(), A.aj() + nnz);
    const bool upper = this->_A->getOptions().symmetric() || this->_A->getOptions().hermitian();
    // buckets: (entity, element type, rule, test field, unknown field)
    std::map<std::string, Bucket> buckets;
    for (const auto &r : _recorded)
      for (const auto &ent : r.entities) {
        std::vector<int> types;
        gmsh::model::mesh::getElementTypes(types, ent.first, ent.second);
        for (int type : types) {
          field::FieldInterface<T> *unknown = r.bilinear ? r.lhs->field() : r.rhs->field();
          const std::string key = std::to_string(ent.first) + "/" + std::to_string(ent.second) + "/" + std::to_string(type) + "/" +
                                  r.integrationType + "/" + std::to_string(r.rhs->field()->tag()) + "/" +
                                  std::to_string(unknown->tag());
          Bucket &b = buckets[key];
          b.entity = ent;
          b.elementType = type;
          b.integrationType = r.integrationType;
          b.field = r.rhs->field();
          b.unknown = unknown;
          b.terms.push_back(&r);
        }
      }
    // the module's arrays: one (A, AFrequency) or K, C, M (null when the module has none)
    T *out[3] = {nullptr, nullptr, nullptr};
    const char which[3] = {'K', 'C', 'M'};
    if (!split) {
      out[0] = const_cast<T *>(this->_A->getModule()->getMatrix());  // MatrixModule.cpp:167-171
    } else {
      for (int k = 0; k < 3; ++k) {
        if ((k == 1 && moduleName == "MK") || (k == 2 && moduleName == "CK")) continue;
        this->_A->getModule()->activate(which[k]);
        out[k] = const_cast<T *>(this->_A->getModule()->getMatrix());
      }
    }
    std::vector<T> rhs(nRows, T(0.0));
    if (buckets.size() == 1) {  // one plan: its call writes the module arrays themselves
      assembleBucket(buckets.begin()->first, buckets.begin()->second, ai, aj, upper, valuesDC, split, out, rhs.data());
    } else {  // several: each call into scratch, summed here
      std::vector<T> scratch[3], b(nRows);
      T *tmp[3] = {nullptr, nullptr, nullptr};
      for (int k = 0; k < 3; ++k)
        if (out[k]) {
          scratch[k].assign(nnz, T(0.0));
          tmp[k] = scratch[k].data();
          for (unsigned long long x = 0; x < nnz; ++x) out[k][x] = T(0.0);
        }
      for (auto &kv : buckets) {
        assembleBucket(kv.first, kv.second, ai, aj, upper, valuesDC, split, tmp, b.data());
        for (int k = 0; k < 3; ++k)
          if (out[k])
            for (unsigned long long x = 0; x < nnz; ++x) out[k][x] += tmp[k][x];
        for (unsigned long long x = 0; x < nRows; ++x) rhs[x] += b[x];
      }
    }
    for (unsigned long long k = 0; k < nRows; ++k)
      if (rhs[k] != T(0.0)) this->_multiB[this->_currentRHS].addValue(k, rhs[k]);
  }

  // A field's basis tables on a bucket, per dense orientation, and its DOF map
  struct SpaceTables {
    int nb = 0, nOrient = 1, mult = 1;
    int32_t form = FG_FORM_0;
    std::vector<double> bval, bgrad;
    std::vector<int32_t> orient;
    std::vector<uint64_t> edof;  // [E][nb * mult], DOF = basis * mult + component
    std::vector<int32_t> etype;
    fg_space_desc desc() const {
      return fg_space_desc{nb, mult, nOrient, bval.data(), bgrad.data(), nOrient > 1 ? orient.data() : nullptr, form};
    }
  };

  static SpaceTables spaceOf(field::FieldInterface<T> *f, const std::vector<double> &gauss, int type,
                             const std::pair<int, int> &ent) {
    SpaceTables st;
    field::FunctionSpaceInterface<double> *fs = f->getFunctionSpace();
    std::vector<int> orient, orient2;
    st.nb = (int)fs->getBasisFunctions(false, st.bval, orient, gauss, type, ent);
    fs->getBasisFunctions(true, st.bgrad, orient2, gauss, type, ent);
    for (int o : orient) st.nOrient = std::max(st.nOrient, o + 1);
    st.orient.assign(orient.begin(), orient.end());
    // H1: values and gradients; HCurl: values [..][3] and curls, the derivative terms being curl-curl
    st.form = f->form() == field::Form::Form1 ? FG_FORM_1 : FG_FORM_0;
    st.mult = (int)f->multiplicity();
    std::vector<int> typeKeys, typeIdx;
    std::vector<unsigned long long> entityKeys, numIdx;
    std::vector<double> keyCoord;
    fs->getKeys(false, typeKeys, entityKeys, keyCoord, type, ent);
    numIdx.resize(typeKeys.size() * st.mult);
    typeIdx.resize(typeKeys.size() * st.mult);
    f->getIndices(typeKeys, entityKeys, numIdx, typeIdx, 0, typeKeys.size());
    st.edof.assign(numIdx.begin(), numIdx.end());
    st.etype.assign(typeIdx.begin(), typeIdx.end());
    return st;
  }

  // the bucket's values [nnz] (v[0]; or K, C, M in v[0..2] when split) and
  // right-hand side [n_rows], overwritten
  void assembleBucket(const std::string &key, const Bucket &bk, const std::vector<uint64_t> &ai, const std::vector<uint64_t> &aj,
                      bool upper, const std::vector<T> &valuesDC, bool split, T *const *v, T *b) {
    const auto &ent = bk.entity;
    const int type = bk.elementType;
    field::FunctionSpaceInterface<double> *fs = bk.field->getFunctionSpace();
    // mesh: the elements' nodes, one coordinate triple per element node
    std::vector<std::size_t> elementTags, nodeTags, nodeTags2;
    std::vector<double> coord, param;
    gmsh::model::mesh::getElementsByType(type, elementTags, nodeTags, ent.second);
    gmsh::model::mesh::getNodesByElementType(type, nodeTags2, coord, param, ent.second, false);
    const int64_t E = (int64_t)elementTags.size();
    if (E == 0) {
      for (int k = 0; k < 3; ++k)
        if (v[k]) std::fill(v[k], v[k] + aj.size(), T(0.0));
      std::fill(b, b + (ai.size() - 1), T(0.0));
      return;
    }
    const int nn = (int)(nodeTags.size() / (size_t)E);
    std::vector<int64_t> elemNodes((size_t)E * nn);
    for (size_t k = 0; k < elemNodes.size(); ++k) elemNodes[k] = (int64_t)k;
    // rule and geometric basis
    std::vector<double> weights, gauss;
    fs->getGaussInfo(bk.integrationType, type, weights, gauss);
    const int nq = (int)weights.size();
    int nc = 0, no = 0;
    std::vector<double> geoVal, geoGrad;
    gmsh::model::mesh::getBasisFunctions(type, gauss, "Lagrange", nc, geoVal, no);
    gmsh::model::mesh::getBasisFunctions(type, gauss, "GradLagrange", nc, geoGrad, no);
    // the test field's space and DOF map, and the unknown field's when it differs
    const SpaceTables test = spaceOf(bk.field, gauss, type, ent);
    SpaceTables unknown;
    if (bk.unknown != bk.field) unknown = spaceOf(bk.unknown, gauss, type, ent);
    // the points of the coefficients (the reference's Assembler takes them from getJacobians)
    std::vector<double> jac, det, pts;
    gmsh::model::mesh::getJacobians(type, gauss, jac, det, pts, ent.second);
    const PointVec points(pts.begin(), pts.end());

    fg_plan *&plan = _plans[key];
    if (!plan) {
      fg_mesh_desc mesh{ent.first, nn, (int64_t)(coord.size() / 3), coord.data(), E, elemNodes.data()};
      fg_rule_desc rule{nq, weights.data(), geoVal.data(), geoGrad.data()};
      const fg_space_desc space = test.desc();
      fg_system_desc sys{};
      sys.n_rows = ai.size() - 1;
      sys.ai = ai.data();
      sys.aj = aj.data();
      sys.elem_dof_idx = test.edof.data();
      sys.elem_dof_type = test.etype.data();
      sys.n_fixed = valuesDC.size();
      sys.upper = upper ? 1 : 0;
      if (bk.unknown == bk.field) {
        check(fg_plan_create(&mesh, &rule, &space, &sys, &plan));
      } else {  // rows from the test field, columns from the unknown field
        const fg_space_desc uspace = unknown.desc();
        check(fg_plan_create_coupled(&mesh, &rule, &space, &sys, &uspace, unknown.edof.data(), unknown.etype.data(), &plan));
      }
    }
    // the terms, with their coefficients as the reference evaluates them
    std::vector<fg_term_desc> terms(bk.terms.size());
    std::vector<std::vector<double>> tables;  // coefficient arrays (moving a vector keeps its data)
    std::vector<std::vector<fg_expr>> tensors(bk.terms.size());
    for (size_t t = 0; t < bk.terms.size(); ++t) {
      const Recorded &r = *bk.terms[t];
      fg_term_desc &d = terms[t];
      d = fg_term_desc{};
      d.kind = r.kind;
      d.dt = r.bilinear ? r.lhs->dt() : FG_DT_NONE;
      std::vector<T> one;
      r.rhs->values(points, gauss, type, ent, one);
      for (const T &c : one)
        if (c != T(1.0)) throw std::runtime_error("a coefficient on the test function");
      std::vector<T> c;
      r.lhs->values(points, gauss, type, ent, c);
      const int nc = r.lhs->components();
      if (nc == 1) {
        describe(c, E, nq, d.coef, tables);
        continue;
      }
      if (nc == 81) {  // isotropic C = lambda d_ij d_kl + mu (d_ik d_jl + d_il d_jk): lambda, mu
        std::vector<T> lam(c.size() / 81), mu(c.size() / 81);
        for (size_t k = 0; k < lam.size(); ++k) {
          const T *C = &c[k * 81];
          lam[k] = C[0 * 9 + 4];  // C_0011
          mu[k] = C[3 * 9 + 3];   // C_0101
          double scale = 0.0;
          for (int x = 0; x < 81; ++x) scale = std::max(scale, std::abs(C[x]));
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
              for (int kk = 0; kk < 3; ++kk)
                for (int l = 0; l < 3; ++l) {
                  const T want = (i == j && kk == l ? lam[k] : T(0.0)) + ((i == kk && j == l) ? mu[k] : T(0.0)) +
                                 ((i == l && j == kk) ? mu[k] : T(0.0));
                  if (std::abs(C[(i + 3 * j) * 9 + kk + 3 * l] - want) > 1e-12 * scale)
                    throw std::runtime_error("a Tensor4 coefficient that is not isotropic");
                }
        }
        describe(lam, E, nq, d.coef, tables);
        describe(mu, E, nq, d.coef2, tables);
        continue;
      }
      // a vector or tensor: coefficient 1 times one program per component.
      // A symmetric tensor goes as its six entries xx, yy, zz, xy, xz, yz
      // (the symmetric tensor kinds, one of each per call; on H1 fields that
      // lets the tensor-core path take it); HCurl tensors must be symmetric
      d.coef.n_code = 1;
      d.coef.code[0] = fg_instr{FG_OP_CONST, 0, 1.0, 0.0};
      std::vector<int> comps;
      for (int k = 0; k < nc; ++k) comps.push_back(k);
      if (nc == 9) {
        bool sym = true;
        for (size_t i = 0; i + 9 <= c.size() && sym; i += 9)
          sym = c[i + 1] == c[i + 3] && c[i + 2] == c[i + 6] && c[i + 5] == c[i + 7];
        const int symKind = d.kind == FG_TERM_MASS_TENSOR ? FG_TERM_MASS_TENSOR : FG_TERM_GRAD_GRAD_TENSOR;
        bool taken = false;
        for (size_t u = 0; u < t; ++u) taken = taken || terms[u].kind == symKind;
        if (d.kind != FG_TERM_GRAD_GRAD_TENSOR_FULL && (!sym || taken))
          throw std::runtime_error("an HCurl tensor coefficient that is not symmetric, or two of one kind");
        if (sym && !taken) {
          d.kind = symKind;
          comps = {0, 4, 8, 1, 2, 5};
        }
      }
      tensors[t].resize(comps.size());
      for (size_t k = 0; k < comps.size(); ++k) {
        std::vector<T> ck(c.size() / nc);
        for (size_t i = 0; i < ck.size(); ++i) ck[i] = c[i * nc + comps[k]];
        tensors[t][k] = fg_expr{};
        describe(ck, E, nq, tensors[t][k], tables);
      }
      d.tensor = tensors[t].data();
    }
    const std::vector<double> dir = flatten(valuesDC);
    auto d = [](T *x) { return reinterpret_cast<double *>(x); };
    if (split)
      check(fg_assemble_separate(plan, terms.data(), (int32_t)terms.size(), 0, dir.empty() ? nullptr : dir.data(), d(v[0]), d(v[1]),
                                 d(v[2]), d(b), nullptr));
    else
      check(fg_assemble_fp64(plan, terms.data(), (int32_t)terms.size(), this->getAngularFrequency(),
                             dir.empty() ? nullptr : dir.data(), d(v[0]), d(b), nullptr));
  }

  static std::vector<double> flatten(const std::vector<T> &x) {
    std::vector<double> out(2 * x.size());
    for (size_t k = 0; k < x.size(); ++k) {
      out[2 * k] = x[k].real();
      out[2 * k + 1] = x[k].imag();
    }
    return out;
  }

  // values [1] (constant) or [E][nq]: a constant, a per-element array when
  // every element's points agree, a point table otherwise
  static void describe(const std::vector<T> &c, int64_t E, int nq, fg_expr &ex, std::vector<std::vector<double>> &tables) {
    ex.n_code = 1;
    ex.n_arrays = 0;
    bool same = true, perElement = c.size() == (size_t)E * nq;
    for (size_t k = 1; k < c.size() && same; ++k) same = c[k] == c[0];
    if (same) {
      ex.code[0] = fg_instr{FG_OP_CONST, 0, c.empty() ? 0.0 : c[0].real(), c.empty() ? 0.0 : c[0].imag()};
      return;
    }
    for (int64_t e = 0; e < E && perElement; ++e)
      for (int q = 1; q < nq && perElement; ++q) perElement = c[(size_t)e * nq + q] == c[(size_t)e * nq];
    std::vector<double> tab;
    if (perElement) {
      tab.resize(2 * (size_t)E);
      for (int64_t e = 0; e < E; ++e) {
        tab[2 * e] = c[(size_t)e * nq].real();
        tab[2 * e + 1] = c[(size_t)e * nq].imag();
      }
    } else {
      tab = flatten(c);
    }
    tables.push_back(std::move(tab));
    ex.code[0] = fg_instr{perElement ? FG_OP_ELEM : FG_OP_POINT, 0, 0.0, 0.0};
    ex.n_arrays = 1;
    ex.elem_values[0] = tables.back().data();
  }
};

}  // namespace gmshfem::problem

#endif  // FEMG_GPU_FORMULATION_H
