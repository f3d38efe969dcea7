// Host-side mirror of the reference's user-facing assembly interface:
// Domain, Field / CompoundField with a FunctionSpace, the equation DSL
// (dof, tf, grad, dt_dof, dt2_dof), coefficient functions, and
// Formulation::integral / pre / assemble.
//
// Reference interfaces mirrored:
//   Formulation<T>::integral    src/problem/Formulation.cpp:219-746
//   Formulation<T>::pre         src/problem/Formulation.cpp:897-1039
//   Formulation<T>::assemble    src/problem/Formulation.cpp:1152-1215
//   dof / tf / grad / dt_dof    src/equation/UnknownField.h:103-132
//   Field<T, Form0>             src/field/Field.cpp:116-135
//   FieldInterface::fillIndices src/field/FieldInterface.cpp:1012-1076
//
// assemble() is the GPU drop-in: it runs through the C ABI of
// include/fem_g_gb300.h (fg_plan_create + fg_assemble_fp64/mixed).
#pragma once
#include <array>
#include <complex>
#include <deque>
#include <memory>
#include <string>
#include <vector>

#include "../../include/fem_g_gb300.h"
#include "dofs.h"
#include "mesh.h"
#include "refelem.h"

namespace femg {

using cplx = std::complex<double>;

struct Domain {
  std::vector<std::pair<int, int>> entities;  // (dim, tag), sorted
  Domain() = default;
  Domain(const Mesh &mesh, const std::string &physical);
  int maxDim() const;
  bool have(int dim, int tag) const;
};

enum class SpaceType { Lagrange = 0, HierarchicalH1 = 1, HCurl = 2 /* lowest-order edge functions */ };

class FunctionSpace {
 public:
  SpaceType type = SpaceType::Lagrange;
  int order = 1;  // hierarchical order; Lagrange uses the mesh order

  // "None" for Lagrange and hierarchical order 1, "HierarchicalSolin" otherwise
  // (src/field/FunctionSpaceHierarchicalH1.cpp:44-50)
  bool orientationFree() const { return type == SpaceType::Lagrange || (type == SpaceType::HierarchicalH1 && order == 1); }
  int form() const { return type == SpaceType::HCurl ? 1 : 0; }  // FG_FORM_*
  bool isConstantByElements() const { return type == SpaceType::Lagrange; }
  int keysPerElement(int elementType) const;
  // keys of all elements of a block in element order (gmsh getKeys semantics
  // of this mirror): Lagrange -> (0, node tag) per element node; hierarchical
  // -> vertices (0, node tag), edges (1+k, edge tag), faces (p+k, face tag),
  // interior (p+nf+k, element tag). infoDim: dimension of the key's entity.
  void getKeys(const Mesh &mesh, const ElementBlock &blk, bool withCoord, std::vector<int> &typeKeys,
               std::vector<uint64_t> &entityKeys, std::vector<double> &coord, std::vector<int> *infoDim) const;
  // basis tables: returns n; table [nOrient][nq][n][ncomp]; denseOrient per element
  int basisFunctions(bool derivative, const Mesh &mesh, const ElementBlock &blk, const QuadRule &rule,
                     std::vector<double> &table, std::vector<int32_t> &denseOrient, int &nOrient) const;
};

// Complex scalar coefficient: an expression in reverse Polish order
class Function {
 public:
  std::vector<fg_instr> code;
  std::vector<std::shared_ptr<std::vector<double>>> arrays;  // per element (re, im), or per element DOF for field values

  Function(double v = 0.0) : Function(cplx(v, 0.0)) {}
  Function(cplx v);
  static Function x();
  static Function y();
  static Function z();
  static Function perElement(const std::vector<cplx> &values);
  // a scalar field of the bucket's own H1 space at the quadrature points (the
  // reference's field node): its values at every element's local DOFs,
  // [n_elements][n] in the element DOF order of pre()
  static Function fieldValues(const std::vector<cplx> &elemDofValues);

  bool usesPoints() const;
  bool usesElements() const;
  bool isConstant() const { return !usesPoints() && !usesElements(); }
  cplx constantValue() const;
  fg_expr toExpr() const;

  friend Function operator+(const Function &a, const Function &b);
  friend Function operator-(const Function &a, const Function &b);
  friend Function operator*(const Function &a, const Function &b);
  friend Function operator/(const Function &a, const Function &b);
  friend Function operator-(const Function &a);
  friend Function heaviside(const Function &a);
  friend Function atan2(const Function &a, const Function &b);
  // a unary operator of the coefficient language (FG_OP_SQRT ... FG_OP_CBRT)
  static Function unary(const Function &a, int op, int arg = 0);

 private:
  static Function binary(const Function &a, const Function &b, int op);
};

// The reference's scalar operators (src/function/scalarUnaryOperators.h:27-120):
// log() is the decimal logarithm and ln() the natural one, as there.
Function sqrt(const Function &a);
Function exp(const Function &a);
Function ln(const Function &a);
Function log(const Function &a);
Function pow(const Function &a, unsigned n);
Function cbrt(const Function &a);
Function sin(const Function &a);
Function cos(const Function &a);
Function tan(const Function &a);
Function sinh(const Function &a);
Function cosh(const Function &a);
Function tanh(const Function &a);
Function asin(const Function &a);
Function acos(const Function &a);
Function atan(const Function &a);
Function asinh(const Function &a);
Function acosh(const Function &a);
Function atanh(const Function &a);
Function abs(const Function &a);
Function conj(const Function &a);
Function real(const Function &a);
Function imag(const Function &a);

struct Tensor4Isotropic {  // C_ijkl = lambda d_ij d_kl + mu (d_ik d_jl + d_il d_jk)
  Function lambda, mu;
};

// Symmetric 3x3 tensor of coefficient functions (the reference's
// TensorFunction, src/function/TensorFunction.h, restricted to symmetric D)
struct TensorFunction {
  Function xx = Function(1.0), yy = Function(1.0), zz = Function(1.0);
  Function xy = Function(0.0), xz = Function(0.0), yz = Function(0.0);
};

class Field {
 public:
  Field(const std::string &name, const Domain &domain, SpaceType type, int order, int multiplicity, unsigned tag);
  std::string name;
  Domain domain;
  FunctionSpace fs;
  int multiplicity = 1;
  unsigned tag = 0;
  struct Constraint {
    Domain domain;
    cplx value;
  };
  std::vector<Constraint> constraints;
  void addConstraint(const Domain &d, cplx value) { constraints.push_back({d, value}); }
  DofDictionary dofs;
  std::vector<cplx> fixedValues;  // by fixed numDof - 1
};

// Vector of coefficient functions (the reference's VectorFunction,
// src/function/VectorFunction.h) multiplying the gradient of the unknown in
// integral(b * grad(dof(u)), tf(v)): the advection term
struct VectorFunction {
  Function x = Function(0.0), y = Function(0.0), z = Function(0.0);
};

struct Operand {
  Field *field = nullptr;
  bool grad = false;
  bool test = false;
  int dt = 0;
  Function coef = Function(1.0);
  bool tensor4 = false;
  Tensor4Isotropic C;
  bool tensor2 = false;  // D * grad(...) with a TensorFunction D
  TensorFunction D;
  bool vec = false;      // b * grad(dof(u)) with a VectorFunction b
  VectorFunction b;
};
Operand dof(Field &f);
Operand tf(Field &f);
Operand dt_dof(Field &f);
Operand dt2_dof(Field &f);
Operand grad(Operand o);
Operand curl(Operand o);  // the derivative of an HCurl field
Operand operator*(const Function &c, Operand o);
Operand operator*(const Tensor4Isotropic &C, Operand o);
Operand operator*(const TensorFunction &D, Operand o);
Operand operator*(const VectorFunction &b, Operand o);

class Formulation {
 public:
  explicit Formulation(const std::string &name) : name_(name) {}
  void integral(const Operand &unknown, const Operand &test, const Domain &d, const std::string &gauss);
  void integral(const Function &f, const Operand &test, const Domain &d, const std::string &gauss);

  // the formulation's symmetric() / hermitian() option: upper-triangle
  // storage of the system matrix (MatrixFactory::addPattern/addValues)
  void setSymmetric(bool on) { symmetric_ = on; }
  bool symmetric() const { return symmetric_; }

  // DOFs, Hilbert numbering, CSR pattern, element bucket data
  void pre(const Mesh &mesh);

  // results of pre()
  uint64_t nUnknown = 0, nBubble = 0, nFixed = 0;
  std::vector<uint64_t> ai, aj;
  // the unknown fields in the reference's registration order
  // (Formulation::_addField, src/problem/Formulation.cpp:149-159: the unknown
  // field of each bilinear term, by first appearance); field = fields[0]
  std::vector<Field *> fields;
  Field *field = nullptr;
  const Mesh *mesh = nullptr;
  const ElementBlock *bucket = nullptr;
  QuadRule rule;
  std::vector<double> geoVal, geoGrad;    // [nq][nn], [nq][nn][3]
  // per field: its basis on the bucket and its element DOF map (fillIndices)
  struct FieldBucket {
    std::vector<double> basisVal, basisGrad;
    std::vector<int32_t> orient;
    int nBasis = 0, nOrient = 1;
    std::vector<uint64_t> elemDofIdx;
    std::vector<int32_t> elemDofType;
  };
  std::vector<FieldBucket> fieldBuckets;
  std::vector<double> dirichlet;          // [nFixed][2], every field's fixed DOFs
  // the terms by (test field, unknown field), in order of first appearance;
  // linear terms join the block (k, k) of their test field k
  struct Block {
    int test = 0, unknown = 0;
    std::vector<fg_term_desc> terms;
  };
  std::vector<Block> blocks;
  std::vector<fg_term_desc> termDescs;    // the terms of blocks[0] (the whole formulation with one field)
  std::deque<std::array<fg_expr, 9>> tensorExprs;  // entries of the tensor / vector terms (stable addresses)
  // reserve calls on the DOF dictionary: (DOFs created before the call, argument)
  std::vector<std::pair<uint64_t, uint64_t>> reserveLog;
  double preSeconds = 0.0;

  // C ABI descriptors over the data above (field 0 / the rows of blocks[0])
  void descs(fg_mesh_desc *m, fg_rule_desc *r, fg_space_desc *s, fg_system_desc *sys) const;
  // the space of field k on the bucket
  void spaceDesc(int k, fg_space_desc *s) const;

  // created DOFs in creation order (before numbering), for numbering checks
  std::vector<Dof> created;

 private:
  bool symmetric_ = false;
  struct BTerm {
    Operand unknown, test;
    Domain domain;
    std::string gauss;
  };
  struct LTerm {
    Function f;
    Operand test;
    Domain domain;
    std::string gauss;
  };
  std::string name_;
  std::vector<BTerm> bterms_;
  std::vector<LTerm> lterms_;
  void fillIndices(const Field &f, const ElementBlock &blk, std::vector<uint64_t> &idx, std::vector<int32_t> &type) const;
  fg_term_desc describe(const BTerm &t);
};

}  // namespace femg
