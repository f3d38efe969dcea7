#include "formulation.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <stdexcept>

namespace femg {

// ---------------------------------------------------------------- Domain

Domain::Domain(const Mesh &mesh, const std::string &physical) {
  auto it = mesh.physicals.find(physical);
  if (it == mesh.physicals.end()) throw std::invalid_argument("unknown physical group " + physical);
  entities = it->second;
  std::sort(entities.begin(), entities.end());
}

int Domain::maxDim() const {
  int d = 0;
  for (auto &e : entities) d = std::max(d, e.first);
  return d;
}

bool Domain::have(int dim, int tag) const {
  return std::find(entities.begin(), entities.end(), std::make_pair(dim, tag)) != entities.end();
}

// --------------------------------------------------------- FunctionSpace

int FunctionSpace::keysPerElement(int elementType) const {
  if (type == SpaceType::Lagrange) return elementNodes(elementType);
  if (type == SpaceType::HCurl) return hcurlCount(elementDim(elementType), order);
  const int dim = elementDim(elementType);
  if (dim == 1) return 2 + (order - 1);
  return hierarchicalCount(dim, order);
}

void FunctionSpace::getKeys(const Mesh &mesh, const ElementBlock &blk, bool withCoord, std::vector<int> &typeKeys,
                            std::vector<uint64_t> &entityKeys, std::vector<double> &coord,
                            std::vector<int> *infoDim) const {
  typeKeys.clear();
  entityKeys.clear();
  coord.clear();
  if (infoDim) infoDim->clear();
  const int nn = blk.nodesPerElement;
  const int dim = elementDim(blk.type);
  const int nv = elementVertices(blk.type);
  const int64_t E = blk.size();
  const int nk = keysPerElement(blk.type);
  typeKeys.reserve((size_t)E * nk);
  entityKeys.reserve((size_t)E * nk);
  if (withCoord) coord.reserve((size_t)E * nk * 3);
  auto pushCoord = [&](const double *p) {
    if (withCoord) coord.insert(coord.end(), p, p + 3);
  };
  if (type == SpaceType::Lagrange) {
    for (int64_t e = 0; e < E; ++e)
      for (int k = 0; k < nn; ++k) {
        const int64_t node = blk.nodes[(size_t)(e * nn + k)];
        typeKeys.push_back(0);
        entityKeys.push_back((uint64_t)node + 1);
        pushCoord(&mesh.xyz[3 * node]);
        if (infoDim) infoDim->push_back(k < nv ? 0 : 1);
      }
    return;
  }
  if (type == SpaceType::HCurl) {
    // per edge (1 + k, edge tag) at the edge midpoint, k < perEdge; per face
    // (1 + perEdge + k, face tag) at the face centroid, k < perFace (in 2D the
    // element's own interior functions, with the element tag at its
    // centroid); per tetrahedron (1 + perEdge + perFace + k, element tag) at
    // its centroid, k < perCell
    int perEdge = 1, perFace = 0, perCell = 0;
    if (order > 0) hcurlEntityCounts(dim, order, perEdge, perFace, perCell);
    for (int64_t e = 0; e < E; ++e) {
      const int64_t *v = &blk.nodes[(size_t)(e * nn)];
      double cen[3] = {0, 0, 0};
      for (int a = 0; a < nv; ++a)
        for (int c = 0; c < 3; ++c) cen[c] += mesh.xyz[3 * v[a] + c] / nv;
      for (auto &ed : simplexEdges(dim)) {
        double mid[3];
        for (int c = 0; c < 3; ++c) mid[c] = 0.5 * (mesh.xyz[3 * v[ed[0]] + c] + mesh.xyz[3 * v[ed[1]] + c]);
        const int64_t tag = mesh.edgeTagOf(v[ed[0]], v[ed[1]]);
        for (int k = 0; k < perEdge; ++k) {
          typeKeys.push_back(1 + k);
          entityKeys.push_back((uint64_t)tag);
          pushCoord(mid);
          if (infoDim) infoDim->push_back(1);
        }
      }
      if (dim == 2) {
        for (int k = 0; k < perFace; ++k) {
          typeKeys.push_back(1 + perEdge + k);
          entityKeys.push_back((uint64_t)blk.tags[(size_t)e]);
          pushCoord(cen);
          if (infoDim) infoDim->push_back(2);
        }
        continue;
      }
      if (perFace > 0)
        for (auto &fc : simplexFaces(3)) {
          const int64_t tag = mesh.faceTagOf(v[fc[0]], v[fc[1]], v[fc[2]]);
          double fcen[3];
          for (int c = 0; c < 3; ++c)
            fcen[c] = (mesh.xyz[3 * v[fc[0]] + c] + mesh.xyz[3 * v[fc[1]] + c] + mesh.xyz[3 * v[fc[2]] + c]) / 3.0;
          for (int k = 0; k < perFace; ++k) {
            typeKeys.push_back(1 + perEdge + k);
            entityKeys.push_back((uint64_t)tag);
            pushCoord(fcen);
            if (infoDim) infoDim->push_back(2);
          }
        }
      for (int k = 0; k < perCell; ++k) {
        typeKeys.push_back(1 + perEdge + perFace + k);
        entityKeys.push_back((uint64_t)blk.tags[(size_t)e]);
        pushCoord(cen);
        if (infoDim) infoDim->push_back(3);
      }
    }
    return;
  }
  const int p = order;
  const int nf = (p - 1) * (p - 2) / 2;
  const int ni3 = (p - 1) * (p - 2) * (p - 3) / 6;
  for (int64_t e = 0; e < E; ++e) {
    const int64_t *v = &blk.nodes[(size_t)(e * nn)];
    double cen[3] = {0, 0, 0};
    for (int a = 0; a < nv; ++a)
      for (int c = 0; c < 3; ++c) cen[c] += mesh.xyz[3 * v[a] + c] / nv;
    for (int a = 0; a < nv; ++a) {
      typeKeys.push_back(0);
      entityKeys.push_back((uint64_t)v[a] + 1);
      pushCoord(&mesh.xyz[3 * v[a]]);
      if (infoDim) infoDim->push_back(0);
    }
    for (auto &ed : simplexEdges(dim)) {
      const int64_t tag = mesh.edgeTagOf(v[ed[0]], v[ed[1]]);
      double mid[3];
      for (int c = 0; c < 3; ++c) mid[c] = 0.5 * (mesh.xyz[3 * v[ed[0]] + c] + mesh.xyz[3 * v[ed[1]] + c]);
      for (int k = 0; k <= p - 2; ++k) {
        typeKeys.push_back(1 + k);
        entityKeys.push_back((uint64_t)tag);
        pushCoord(mid);
        if (infoDim) infoDim->push_back(1);
      }
    }
    if (dim == 2) {
      for (int k = 0; k < nf; ++k) {
        typeKeys.push_back(p + k);
        entityKeys.push_back((uint64_t)blk.tags[(size_t)e]);
        pushCoord(cen);
        if (infoDim) infoDim->push_back(2);
      }
    } else if (dim == 3) {
      for (auto &fc : simplexFaces(3)) {
        const int64_t tag = mesh.faceTagOf(v[fc[0]], v[fc[1]], v[fc[2]]);
        double fcen[3];
        for (int c = 0; c < 3; ++c) fcen[c] = (mesh.xyz[3 * v[fc[0]] + c] + mesh.xyz[3 * v[fc[1]] + c] + mesh.xyz[3 * v[fc[2]] + c]) / 3.0;
        for (int k = 0; k < nf; ++k) {
          typeKeys.push_back(p + k);
          entityKeys.push_back((uint64_t)tag);
          pushCoord(fcen);
          if (infoDim) infoDim->push_back(2);
        }
      }
      for (int k = 0; k < ni3; ++k) {
        typeKeys.push_back(p + nf + k);
        entityKeys.push_back((uint64_t)blk.tags[(size_t)e]);
        pushCoord(cen);
        if (infoDim) infoDim->push_back(3);
      }
    }
  }
}

int FunctionSpace::basisFunctions(bool derivative, const Mesh &mesh, const ElementBlock &blk, const QuadRule &rule,
                                  std::vector<double> &table, std::vector<int32_t> &denseOrient, int &nOrient) const {
  const int64_t E = blk.size();
  const int ncomp = (derivative || type == SpaceType::HCurl) ? 3 : 1;
  denseOrient.assign((size_t)E, 0);
  table.clear();
  if (type == SpaceType::Lagrange) {
    const int n = elementNodes(blk.type);
    nOrient = 1;
    std::vector<double> val(n), grad(3 * n);
    for (int q = 0; q < rule.nq; ++q) {
      lagrangeBasis(blk.type, &rule.points[3 * q], val.data(), grad.data());
      for (int i = 0; i < n; ++i)
        for (int c = 0; c < ncomp; ++c) table.push_back(derivative ? grad[3 * i + c] : val[i]);
    }
    return n;
  }
  const int dim = elementDim(blk.type);
  const bool hcurl = type == SpaceType::HCurl;
  const int n = hcurl ? hcurlCount(dim, order) : hierarchicalCount(dim, order);
  const int nn = blk.nodesPerElement;
  const int nv = elementVertices(blk.type);
  // raw orientation per element, then the dense numbering of first
  // appearance (getDenseOrientations, src/field/FunctionSpaceInterface.cpp:495-519)
  std::vector<int> unique;
  std::map<int, int> denseOf;
  for (int64_t e = 0; e < E; ++e) {
    int64_t tags[4];
    for (int a = 0; a < nv; ++a) tags[a] = blk.nodes[(size_t)(e * nn + a)] + 1;
    const int code = orientationFree() ? 0 : (hcurl ? hcurlOrientation(dim, order, tags) : hierarchicalOrientation(dim, tags));
    auto it = denseOf.find(code);
    if (it == denseOf.end()) {
      it = denseOf.emplace(code, (int)unique.size()).first;
      unique.push_back(code);
    }
    denseOrient[(size_t)e] = it->second;
  }
  nOrient = (int)unique.size();
  std::vector<double> val(3 * n), grad(3 * n);
  for (int o = 0; o < nOrient; ++o)
    for (int q = 0; q < rule.nq; ++q) {
      if (hcurl) {  // values [n][3], curls [n][3]
        hcurlBasis(dim, order, unique[o], &rule.points[3 * q], val.data(), grad.data());
        for (int i = 0; i < n; ++i)
          for (int c = 0; c < 3; ++c) table.push_back(derivative ? grad[3 * i + c] : val[3 * i + c]);
        continue;
      }
      hierarchicalBasis(dim, order, unique[o], &rule.points[3 * q], val.data(), grad.data());
      for (int i = 0; i < n; ++i)
        for (int c = 0; c < ncomp; ++c) table.push_back(derivative ? grad[3 * i + c] : val[i]);
    }
  (void)mesh;
  return n;
}

// -------------------------------------------------------------- Function

Function::Function(cplx v) { code.push_back({FG_OP_CONST, 0, v.real(), v.imag()}); }

Function Function::x() {
  Function f;
  f.code = {{FG_OP_X, 0, 0.0, 0.0}};
  return f;
}
Function Function::y() {
  Function f;
  f.code = {{FG_OP_Y, 0, 0.0, 0.0}};
  return f;
}
Function Function::z() {
  Function f;
  f.code = {{FG_OP_Z, 0, 0.0, 0.0}};
  return f;
}

Function Function::perElement(const std::vector<cplx> &values) {
  Function f;
  auto arr = std::make_shared<std::vector<double>>(2 * values.size());
  for (size_t i = 0; i < values.size(); ++i) {
    (*arr)[2 * i] = values[i].real();
    (*arr)[2 * i + 1] = values[i].imag();
  }
  f.arrays = {arr};
  f.code = {{FG_OP_ELEM, 0, 0.0, 0.0}};
  return f;
}

Function Function::fieldValues(const std::vector<cplx> &elemDofValues) {
  Function f = perElement(elemDofValues);
  f.code[0].op = FG_OP_FIELD;
  return f;
}

bool Function::usesPoints() const {
  for (auto &i : code)
    if (i.op == FG_OP_X || i.op == FG_OP_Y || i.op == FG_OP_Z || i.op == FG_OP_FIELD) return true;
  return false;
}

bool Function::usesElements() const {
  for (auto &i : code)
    if (i.op == FG_OP_ELEM) return true;
  return false;
}

cplx Function::constantValue() const {
  if (!isConstant()) throw std::logic_error("not a constant function");
  std::vector<cplx> st;
  for (auto &in : code) {
    if (in.op == FG_OP_CONST) {
      st.push_back(cplx(in.re, in.im));
      continue;
    }
    if (in.op == FG_OP_NEG) {
      st.back() = -st.back();
      continue;
    }
    if (in.op == FG_OP_HEAVISIDE) {
      const double r = st.back().real();
      st.back() = r > 0 ? 1.0 : (r < 0 ? 0.0 : 0.5);
      continue;
    }
    cplx b = st.back();
    st.pop_back();
    cplx &a = st.back();
    if (in.op == FG_OP_ADD) a += b;
    else if (in.op == FG_OP_SUB) a -= b;
    else if (in.op == FG_OP_MUL) a *= b;
    else if (in.op == FG_OP_DIV) a /= b;
  }
  return st.back();
}

fg_expr Function::toExpr() const {
  fg_expr e;
  std::memset(&e, 0, sizeof(e));
  if (code.size() > FG_EXPR_MAX_CODE) throw std::length_error("expression too long");
  if (arrays.size() > FG_EXPR_MAX_ARRAYS) throw std::length_error("too many per-element arrays");
  e.n_code = (int32_t)code.size();
  for (size_t i = 0; i < code.size(); ++i) e.code[i] = code[i];
  e.n_arrays = (int32_t)arrays.size();
  for (size_t i = 0; i < arrays.size(); ++i) e.elem_values[i] = arrays[i]->data();
  return e;
}

Function Function::binary(const Function &a, const Function &b, int op) {
  Function r;
  r.code = a.code;
  r.arrays = a.arrays;
  const int32_t shift = (int32_t)a.arrays.size();
  for (auto in : b.code) {
    if (in.op == FG_OP_ELEM || in.op == FG_OP_FIELD) in.arg += shift;
    r.code.push_back(in);
  }
  r.arrays.insert(r.arrays.end(), b.arrays.begin(), b.arrays.end());
  r.code.push_back({op, 0, 0.0, 0.0});
  return r;
}

Function operator+(const Function &a, const Function &b) { return Function::binary(a, b, FG_OP_ADD); }
Function operator-(const Function &a, const Function &b) { return Function::binary(a, b, FG_OP_SUB); }
Function operator*(const Function &a, const Function &b) { return Function::binary(a, b, FG_OP_MUL); }
Function operator/(const Function &a, const Function &b) { return Function::binary(a, b, FG_OP_DIV); }
Function operator-(const Function &a) {
  Function r = a;
  r.code.push_back({FG_OP_NEG, 0, 0.0, 0.0});
  return r;
}
Function heaviside(const Function &a) {
  Function r = a;
  r.code.push_back({FG_OP_HEAVISIDE, 0, 0.0, 0.0});
  return r;
}

Function Function::unary(const Function &a, int op, int arg) {
  Function r = a;
  r.code.push_back({op, arg, 0.0, 0.0});
  return r;
}
Function sqrt(const Function &a) { return Function::unary(a, FG_OP_SQRT); }
Function exp(const Function &a) { return Function::unary(a, FG_OP_EXP); }
Function ln(const Function &a) { return Function::unary(a, FG_OP_LN); }
Function log(const Function &a) { return Function::unary(a, FG_OP_LOG10); }
Function pow(const Function &a, unsigned n) { return Function::unary(a, FG_OP_POW, (int)n); }
Function cbrt(const Function &a) { return Function::unary(a, FG_OP_CBRT); }
Function sin(const Function &a) { return Function::unary(a, FG_OP_SIN); }
Function cos(const Function &a) { return Function::unary(a, FG_OP_COS); }
Function tan(const Function &a) { return Function::unary(a, FG_OP_TAN); }
Function sinh(const Function &a) { return Function::unary(a, FG_OP_SINH); }
Function cosh(const Function &a) { return Function::unary(a, FG_OP_COSH); }
Function tanh(const Function &a) { return Function::unary(a, FG_OP_TANH); }
Function asin(const Function &a) { return Function::unary(a, FG_OP_ASIN); }
Function acos(const Function &a) { return Function::unary(a, FG_OP_ACOS); }
Function atan(const Function &a) { return Function::unary(a, FG_OP_ATAN); }
Function asinh(const Function &a) { return Function::unary(a, FG_OP_ASINH); }
Function acosh(const Function &a) { return Function::unary(a, FG_OP_ACOSH); }
Function atanh(const Function &a) { return Function::unary(a, FG_OP_ATANH); }
Function abs(const Function &a) { return Function::unary(a, FG_OP_ABS); }
Function conj(const Function &a) { return Function::unary(a, FG_OP_CONJ); }
Function real(const Function &a) { return Function::unary(a, FG_OP_REAL); }
Function imag(const Function &a) { return Function::unary(a, FG_OP_IMAG); }
Function atan2(const Function &a, const Function &b) { return Function::binary(a, b, FG_OP_ATAN2); }

// ------------------------------------------------------------ Field / DSL

Field::Field(const std::string &n, const Domain &d, SpaceType t, int order, int mult, unsigned tg)
    : name(n), domain(d), multiplicity(mult), tag(tg) {
  fs.type = t;
  fs.order = order;
}

Operand dof(Field &f) {
  Operand o;
  o.field = &f;
  return o;
}
Operand tf(Field &f) {
  Operand o;
  o.field = &f;
  o.test = true;
  return o;
}
Operand dt_dof(Field &f) {
  Operand o = dof(f);
  o.dt = 1;
  return o;
}
Operand dt2_dof(Field &f) {
  Operand o = dof(f);
  o.dt = 2;
  return o;
}
Operand grad(Operand o) {
  if (o.field && o.field->fs.type == SpaceType::HCurl) throw std::invalid_argument("grad of an HCurl field: use curl");
  o.grad = true;
  return o;
}
Operand curl(Operand o) {
  if (!o.field || o.field->fs.type != SpaceType::HCurl) throw std::invalid_argument("curl needs an HCurl field");
  o.grad = true;  // the derivative term of a Form1 field is its curl (Form2)
  return o;
}
Operand operator*(const Function &c, Operand o) {
  o.coef = c * o.coef;
  return o;
}
Operand operator*(const Tensor4Isotropic &C, Operand o) {
  o.tensor4 = true;
  o.C = C;
  return o;
}

Operand operator*(const TensorFunction &D, Operand o) {
  o.tensor2 = true;
  o.D = D;
  return o;
}

Operand operator*(const VectorFunction &b, Operand o) {
  o.vec = true;
  o.b = b;
  return o;
}

// ----------------------------------------------------------- Formulation

void Formulation::integral(const Operand &unknown, const Operand &test, const Domain &d, const std::string &gauss) {
  if (unknown.test || !test.test) throw std::invalid_argument("integral(dof(...), tf(...)) expected");
  bterms_.push_back({unknown, test, d, gauss});
}

void Formulation::integral(const Function &f, const Operand &test, const Domain &d, const std::string &gauss) {
  if (!test.test) throw std::invalid_argument("integral(f, tf(...)) expected");
  lterms_.push_back({f, test, d, gauss});
}

void Formulation::fillIndices(const Field &f, const ElementBlock &blk, std::vector<uint64_t> &idx, std::vector<int32_t> &type) const {
  std::vector<int> typeKeys;
  std::vector<uint64_t> entityKeys;
  std::vector<double> coord;
  f.fs.getKeys(*mesh, blk, false, typeKeys, entityKeys, coord, nullptr);
  const size_t nk = typeKeys.size();
  const int multi = f.multiplicity;
  idx.assign(nk * multi, 0);
  type.assign(nk * multi, 0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)nk; ++i)
    for (int j = 0; j < multi; ++j) {
      const Dof *d = f.dofs.find((uint64_t)typeKeys[(size_t)i] + kDofFieldOffset * (f.tag + j), entityKeys[(size_t)i]);
      if (d) {
        idx[(size_t)i * multi + j] = d->numDof - 1;
        type[(size_t)i * multi + j] = d->assembleType;
      }
    }
}

fg_term_desc Formulation::describe(const BTerm &t) {
  fg_term_desc d;
  std::memset(&d, 0, sizeof(d));
  if (!t.test.coef.isConstant() || t.test.coef.constantValue() != cplx(1.0, 0.0))
    throw std::invalid_argument("coefficients on the test function are not supported");
  d.dt = t.unknown.dt;
  if (t.unknown.vec) {
    // b . grad(dof(u)) tested against tf(v): the advection term
    if (!t.unknown.grad || t.test.grad) throw std::invalid_argument("a vector function multiplies grad(dof(u)), tested by tf(v)");
    const VectorFunction &b = t.unknown.b;
    d.kind = FG_TERM_ADVECTION;
    d.coef = t.unknown.coef.toExpr();
    tensorExprs.push_back({b.x.toExpr(), b.y.toExpr(), b.z.toExpr()});
    d.tensor = tensorExprs.back().data();
    return d;
  }
  if (t.unknown.grad != t.test.grad) throw std::invalid_argument("mixed value/gradient terms are not supported");
  if (t.unknown.tensor4) {
    if (!t.unknown.grad) throw std::invalid_argument("Tensor4 needs gradients");
    d.kind = FG_TERM_ELASTIC;
    d.coef = (t.unknown.coef * t.unknown.C.lambda).toExpr();
    d.coef2 = (t.unknown.coef * t.unknown.C.mu).toExpr();
  } else if (t.unknown.tensor2) {
    // D * grad (H1), D * curl (HCurl) or D * dof (HCurl values)
    if (!t.unknown.grad && t.unknown.field->fs.form() != 1)
      throw std::invalid_argument("a tensor function multiplies gradients, curls or HCurl values");
    const TensorFunction &D = t.unknown.D;
    d.kind = t.unknown.grad ? FG_TERM_GRAD_GRAD_TENSOR : FG_TERM_MASS_TENSOR;
    d.coef = t.unknown.coef.toExpr();
    tensorExprs.push_back({D.xx.toExpr(), D.yy.toExpr(), D.zz.toExpr(), D.xy.toExpr(), D.xz.toExpr(), D.yz.toExpr()});
    d.tensor = tensorExprs.back().data();
  } else {
    d.kind = t.unknown.grad ? FG_TERM_GRAD_GRAD : FG_TERM_MASS;
    d.coef = t.unknown.coef.toExpr();
  }
  return d;
}

void Formulation::pre(const Mesh &m) {
  auto t0 = std::chrono::steady_clock::now();
  mesh = &m;
  if (bterms_.empty()) throw std::invalid_argument("no bilinear term");
  // the unknown fields: Formulation::_addField on each bilinear term's
  // unknown field (src/problem/Formulation.cpp:149-159, :219-300)
  fields.clear();
  for (auto &t : bterms_)
    if (std::find(fields.begin(), fields.end(), t.unknown.field) == fields.end()) fields.push_back(t.unknown.field);
  if (fields.size() > 2)
    throw std::invalid_argument(
        "at most two fields: the reference numbers the DOFs of its fields in the iteration order of an unordered_set of "
        "field pointers (DofsManager::_fields), which with three or more depends on the fields' addresses");
  auto fieldIndex = [&](const Field *f) -> int {
    for (size_t k = 0; k < fields.size(); ++k)
      if (fields[k] == f) return (int)k;
    throw std::invalid_argument("a test field that is the unknown of no bilinear term has no DOFs");
  };
  for (auto &t : bterms_) fieldIndex(t.test.field);
  for (auto &t : lterms_) fieldIndex(t.test.field);
  field = fields[0];
  for (Field *fp : fields)
    if (fields.size() > 1 && (fp->multiplicity != 1 || fp->fs.form() != 0))
      throw std::invalid_argument("several fields: scalar H1 fields only in this mirror");

  // ---- DofsFactory::generate (src/dofs/DofsFactory.cpp:725-839): the fixed
  // DOFs of every field, then the unknown DOFs of every field, numbered by
  // counters shared across the fields; maxDim over all fields' domains
  int maxDim = 0;
  for (Field *fp : fields) maxDim = std::max(maxDim, fp->domain.maxDim());
  nFixed = nUnknown = nBubble = 0;
  reserveLog.clear();
  created.clear();
  for (Field *fp : fields) {
    fp->dofs = DofDictionary();
    fp->fixedValues.clear();
  }
  std::vector<cplx> fixedAll;
  // DofsManager::addField order (a field enters on each of its constraints,
  // and every field once its unknown DOFs are made)
  std::vector<Field *> registered;
  auto registerField = [&](Field *f) {
    if (std::find(registered.begin(), registered.end(), f) == registered.end()) registered.push_back(f);
  };
  std::vector<int> typeKeys, info;
  std::vector<uint64_t> entityKeys;
  std::vector<double> coord;
  for (Field *fp : fields) {
    Field &f = *fp;
    for (auto &c : f.constraints) {
      if (!f.fs.orientationFree() || f.multiplicity != 1)
        throw std::invalid_argument("constraints need a Lagrange / order-1 scalar field in this mirror");
      for (auto &de : c.domain.entities) {
        const Entity *ent = m.find(de.first, de.second);
        if (!ent) continue;
        for (auto &blk : ent->blocks) {
          f.fs.getKeys(m, blk, true, typeKeys, entityKeys, coord, nullptr);
          reserveLog.push_back({f.dofs.size(), f.dofs.size() + typeKeys.size()});
          f.dofs.reserve(f.dofs.size() + typeKeys.size());
          for (size_t j = 0; j < typeKeys.size(); ++j) {
            Dof d;
            d.numType = (uint64_t)typeKeys[j] + kDofFieldOffset * f.tag;
            d.entity = entityKeys[j];
            d.assembleType = kAtFixed;
            for (int k = 0; k < 3; ++k) d.xyz[k] = (float)coord[3 * j + k];
            d.numDof = nFixed + 1;
            if (f.dofs.insert(d)) {
              ++nFixed;
              f.fixedValues.push_back(c.value);
              fixedAll.push_back(c.value);
              created.push_back(d);
            }
          }
        }
      }
      registerField(fp);
    }
  }
  for (Field *fp : fields) {
    Field &f = *fp;
    for (auto &de : f.domain.entities) {
      const Entity *ent = m.find(de.first, de.second);
      if (!ent) continue;
      for (auto &blk : ent->blocks) {
        const bool top = de.first == maxDim;
        f.fs.getKeys(m, blk, true, typeKeys, entityKeys, coord, top ? &info : nullptr);
        reserveLog.push_back({f.dofs.size(), f.dofs.size() + typeKeys.size() * f.multiplicity});
        f.dofs.reserve(f.dofs.size() + typeKeys.size() * f.multiplicity);
        for (size_t j = 0; j < typeKeys.size(); ++j)
          for (int k = 0; k < f.multiplicity; ++k) {
            const bool bubble = top && info[j] == maxDim;
            Dof d;
            d.numType = (uint64_t)typeKeys[j] + kDofFieldOffset * (f.tag + k);
            d.entity = entityKeys[j];
            d.assembleType = bubble ? kAtUnknownBubble : kAtUnknown;
            for (int c = 0; c < 3; ++c) d.xyz[c] = (float)coord[3 * j + c];
            d.numDof = nUnknown + 1;
            if (f.dofs.insert(d)) {
              ++nUnknown;
              if (bubble) ++nBubble;
              created.push_back(d);
            }
          }
      }
    }
    registerField(fp);
  }

  // ---- DofsManager::reorderWithHilbert(true) over the fields of
  // DofsManager::_fields, a std::unordered_set of field pointers
  // (src/dofs/DofsManager.h:47, DofsManager.cpp:137-151): with one or two
  // elements libstdc++ keeps them in one bucket chain (even addresses, two
  // buckets) and iterates the later insertion first
  if (m.dim == 2 || m.dim == 3) {
    std::vector<DofDictionary *> dicts;
    for (auto it = registered.rbegin(); it != registered.rend(); ++it) dicts.push_back(&(*it)->dofs);
    reorderWithHilbert(m.dim, m.bbox, dicts, nUnknown, nBubble);
  }

  // ---- the element bucket (one) and every field's element DOF map on it
  bucket = nullptr;
  for (auto &ent : m.entities) {
    bool have = false;
    for (auto &t : bterms_) have = have || t.domain.have(ent.dim, ent.tag);
    if (!have) continue;
    for (auto &blk : ent.blocks) {
      if (bucket) throw std::invalid_argument("this mirror assembles a single element bucket");
      bucket = &blk;
    }
  }
  if (!bucket) throw std::invalid_argument("no element carries a bilinear term");
  fieldBuckets.assign(fields.size(), FieldBucket());
  for (size_t k = 0; k < fields.size(); ++k)
    fillIndices(*fields[k], *bucket, fieldBuckets[k].elemDofIdx, fieldBuckets[k].elemDofType);

  // ---- pattern: MatrixFactory::addPattern per bilinear term
  // (src/term/Pattern.cpp:69): rows the test field's DOFs, columns the
  // unknown field's
  PatternBuilder pb;
  pb.init(nUnknown);
  pb.symmetric = symmetric_;
  const int64_t E = (int64_t)bucket->size();
  for (auto &t : bterms_) {
    const FieldBucket &ft = fieldBuckets[(size_t)fieldIndex(t.test.field)];
    const FieldBucket &fu = fieldBuckets[(size_t)fieldIndex(t.unknown.field)];
    const int nt = (int)(ft.elemDofIdx.size() / std::max<int64_t>(E, 1));
    const int nu = (int)(fu.elemDofIdx.size() / std::max<int64_t>(E, 1));
    pb.addElements(E, nt, nu, ft.elemDofIdx.data(), ft.elemDofType.data(), fu.elemDofIdx.data(), fu.elemDofType.data());
  }
  pb.finalize(ai, aj);

  // ---- bucket data (Assembler::assemblyInitialization)
  std::string gauss = bterms_[0].gauss;
  for (auto &t : bterms_)
    if (t.gauss != gauss) throw std::invalid_argument("one integration type per formulation in this mirror");
  for (auto &t : lterms_)
    if (t.gauss != gauss) throw std::invalid_argument("one integration type per formulation in this mirror");
  rule = gaussRule(gauss, bucket->type);
  const int nn = bucket->nodesPerElement;
  geoVal.assign((size_t)rule.nq * nn, 0.0);
  geoGrad.assign((size_t)rule.nq * nn * 3, 0.0);
  for (int q = 0; q < rule.nq; ++q) lagrangeBasis(bucket->type, &rule.points[3 * q], &geoVal[(size_t)q * nn], &geoGrad[(size_t)q * nn * 3]);
  for (size_t k = 0; k < fields.size(); ++k) {
    FieldBucket &fb = fieldBuckets[k];
    int no2 = 1;
    std::vector<int32_t> o2;
    fb.nBasis = fields[k]->fs.basisFunctions(false, m, *bucket, rule, fb.basisVal, fb.orient, fb.nOrient);
    fields[k]->fs.basisFunctions(true, m, *bucket, rule, fb.basisGrad, o2, no2);
  }
  dirichlet.assign(2 * nFixed, 0.0);
  for (uint64_t i = 0; i < nFixed; ++i) {
    dirichlet[2 * i] = fixedAll[i].real();
    dirichlet[2 * i + 1] = fixedAll[i].imag();
  }

  // ---- terms for the C ABI, by (test field, unknown field)
  blocks.clear();
  tensorExprs.clear();
  auto blockOf = [&](int test, int unknown) -> Block & {
    for (auto &b : blocks)
      if (b.test == test && b.unknown == unknown) return b;
    blocks.push_back(Block{test, unknown, {}});
    return blocks.back();
  };
  for (auto &t : bterms_) {
    const fg_term_desc d = describe(t);
    blockOf(fieldIndex(t.test.field), fieldIndex(t.unknown.field)).terms.push_back(d);
  }
  for (auto &t : lterms_) {
    fg_term_desc d;
    std::memset(&d, 0, sizeof(d));
    if (t.test.grad) throw std::invalid_argument("gradient test functions in linear terms are not supported");
    d.kind = FG_TERM_SOURCE;
    d.coef = t.f.toExpr();
    const int k = fieldIndex(t.test.field);
    blockOf(k, k).terms.push_back(d);
  }
  termDescs = blocks[0].terms;
  preSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void Formulation::spaceDesc(int k, fg_space_desc *sd) const {
  const FieldBucket &fb = fieldBuckets[(size_t)k];
  sd->n_basis = fb.nBasis;
  sd->multiplicity = fields[(size_t)k]->multiplicity;
  sd->n_orientations = fb.nOrient;
  sd->basis_val = fb.basisVal.data();
  sd->basis_grad = fb.basisGrad.data();
  sd->elem_orientation = fb.nOrient > 1 ? fb.orient.data() : nullptr;
  sd->form = fields[(size_t)k]->fs.form();
}

void Formulation::descs(fg_mesh_desc *md, fg_rule_desc *rd, fg_space_desc *sd, fg_system_desc *sys) const {
  md->dim = elementDim(bucket->type);
  md->nodes_per_element = bucket->nodesPerElement;
  md->n_nodes = mesh->nNodes();
  md->node_xyz = mesh->xyz.data();
  md->n_elements = bucket->size();
  md->elem_nodes = bucket->nodes.data();
  rd->nq = rule.nq;
  rd->weights = rule.weights.data();
  rd->geo_val = geoVal.data();
  rd->geo_grad = geoGrad.data();
  const int rows = blocks.empty() ? 0 : blocks[0].test;
  spaceDesc(rows, sd);
  sys->n_rows = nUnknown;
  sys->ai = ai.data();
  sys->aj = aj.data();
  sys->elem_dof_idx = fieldBuckets[(size_t)rows].elemDofIdx.data();
  sys->elem_dof_type = fieldBuckets[(size_t)rows].elemDofType.data();
  sys->n_fixed = nFixed;
  sys->upper = symmetric_ ? 1 : 0;
  sys->n_linked = 0;
  sys->linked_row = nullptr;
  sys->linked_value = nullptr;
}

}  // namespace femg
