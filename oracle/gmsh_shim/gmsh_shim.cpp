// The gmsh stand-in behind the oracle's reference build — TEST INFRASTRUCTURE
// ONLY.
//
// Implements the part of the gmsh API (gmsh.h in this directory) that the
// reference's Formulation::pre() and assemble() reach, over one in-memory
// model installed by oracleShimSetMesh(): this project's synthetic simplex
// meshes (fem-g_gb300/host/mesh.cpp), its quadrature rules, geometric
// Lagrange basis, hierarchical H1 and hierarchical HCurl bases and DOF keys
// (fem-g_gb300/host/refelem.cpp, formulation.cpp). These are the same tables
// the GPU path's host mirror hands to the C ABI, so the reference's own DOF
// creation, numbering, pattern, element integration and scatter run on
// exactly the inputs the GPU path gets. Every other gmsh call throws.
//
// Conventions followed (those of the gmsh API the reference is written for):
//   * entities (dim, tag) sorted by dimension then tag; element blocks per
//     (element type, entity) in element order;
//   * Jacobians by columns, J[9 * (e * nq + q) + 3 * c + r] = d x_r / d u_c,
//     2D elements completed by their unit normal (det = |t1 x t2|);
//   * basis tables [orientation][point][function][component];
//   * task / numTasks split the elements of a block into contiguous ranges;
//     the output vectors are preallocated to the whole block.
#include "gmsh.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../fem-g_gb300/host/formulation.h"
#include "shim_model.h"

namespace {

struct ShimModel {
  std::string name = "oracle";
  femg::Mesh mesh;
  bool have = false;
  std::map<std::string, double> numbers;
};

ShimModel &shim() {
  static ShimModel m;
  return m;
}

[[noreturn]] void unavailable(const char *what) {
  throw std::runtime_error(std::string("gmsh stand-in: ") + what + " is not available in the oracle build");
}

const femg::Mesh &shimMesh() {
  if (!shim().have) throw std::runtime_error("gmsh stand-in: no mesh installed (oracleShimSetMesh)");
  return shim().mesh;
}

// the element block of (type, entity tag) at the mesh's dimension or below
const femg::ElementBlock &block(int type, int tag) {
  const femg::Mesh &m = shimMesh();
  const int dim = femg::elementDim(type);
  for (auto &ent : m.entities) {
    if (ent.dim != dim || (tag >= 0 && ent.tag != tag)) continue;
    for (auto &b : ent.blocks)
      if (b.type == type) {
        if (tag < 0) {
          // gmsh without an entity tag means every entity of the type; the
          // meshes here hold one entity per dimension on the assembly path
          int count = 0;
          for (auto &e2 : m.entities)
            if (e2.dim == dim)
              for (auto &b2 : e2.blocks)
                if (b2.type == type) ++count;
          if (count > 1) unavailable("an element query over several entities");
        }
        return b;
      }
  }
  throw std::runtime_error("gmsh stand-in: no elements of type " + std::to_string(type) + " on entity " +
                           std::to_string(tag));
}

void taskRange(int64_t n, std::size_t task, std::size_t numTasks, int64_t &b, int64_t &e) {
  if (numTasks == 0) numTasks = 1;
  b = (int64_t)(n * (int64_t)task / (int64_t)numTasks);
  e = (int64_t)(n * (int64_t)(task + 1) / (int64_t)numTasks);
}

// gmsh function-space names used by the reference's function spaces
femg::FunctionSpace parseSpace(const std::string &name, bool *derivative) {
  femg::FunctionSpace fs;
  auto num = [&](const std::string &prefix) { return std::stoi(name.substr(prefix.size())); };
  *derivative = false;
  if (name == "Lagrange" || name == "GradLagrange") {
    fs.type = femg::SpaceType::Lagrange;
    *derivative = name[0] == 'G';
  } else if (name.rfind("GradH1Legendre", 0) == 0) {
    fs.type = femg::SpaceType::HierarchicalH1;
    fs.order = num("GradH1Legendre");
    *derivative = true;
  } else if (name.rfind("H1Legendre", 0) == 0) {
    fs.type = femg::SpaceType::HierarchicalH1;
    fs.order = num("H1Legendre");
  } else if (name.rfind("CurlHcurlLegendre", 0) == 0) {
    fs.type = femg::SpaceType::HCurl;
    fs.order = num("CurlHcurlLegendre");
    *derivative = true;
  } else if (name.rfind("HcurlLegendre", 0) == 0) {
    fs.type = femg::SpaceType::HCurl;
    fs.order = num("HcurlLegendre");
  } else {
    throw std::runtime_error("gmsh stand-in: function space " + name + " is not available");
  }
  return fs;
}

int orientationOf(const femg::FunctionSpace &fs, const femg::ElementBlock &blk, int64_t e) {
  if (fs.orientationFree()) return 0;
  const int dim = femg::elementDim(blk.type);
  const int nv = femg::elementVertices(blk.type);
  int64_t tags[4];
  for (int a = 0; a < nv; ++a) tags[a] = blk.nodes[(size_t)(e * blk.nodesPerElement + a)] + 1;
  return fs.type == femg::SpaceType::HCurl ? femg::hcurlOrientation(dim, fs.order, tags) : femg::hierarchicalOrientation(dim, tags);
}

// reference coordinates of the geometric nodes (vertices, then the edge
// midpoints in the local edge order of the meshes)
std::vector<double> referenceNodes(int type) {
  const int dim = femg::elementDim(type);
  std::vector<std::array<double, 3>> v;
  v.push_back({0, 0, 0});
  for (int d = 0; d < dim; ++d) {
    std::array<double, 3> p = {0, 0, 0};
    p[d] = 1.0;
    v.push_back(p);
  }
  if (femg::elementOrder(type) == 2) {
    const int nv = (int)v.size();
    for (auto &ed : femg::simplexEdges(dim)) {
      std::array<double, 3> p;
      for (int c = 0; c < 3; ++c) p[c] = 0.5 * (v[ed[0]][c] + v[ed[1]][c]);
      v.push_back(p);
    }
    (void)nv;
  }
  std::vector<double> out;
  for (auto &p : v)
    for (int c = 0; c < dim; ++c) out.push_back(p[c]);
  return out;
}

const char *elementName(int type) {
  switch (type) {
    case femg::kPoint: return "Point";
    case femg::kLine2: return "Line 2";
    case femg::kLine3: return "Line 3";
    case femg::kTri3: return "Triangle 3";
    case femg::kTri6: return "Triangle 6";
    case femg::kTet4: return "Tetrahedron 4";
    case femg::kTet10: return "Tetrahedron 10";
  }
  return "Unknown";
}

}  // namespace

void oracleShimSetMesh(femg::Mesh &&m) {
  shim().mesh = std::move(m);
  shim().have = true;
}

const femg::Mesh &oracleShimMesh() { return shimMesh(); }

namespace gmsh {

void initialize(int, char **, const bool, const bool) {}
void finalize() {}

namespace option {
void setNumber(const std::string &name, const double value) { shim().numbers[name] = value; }
void getNumber(const std::string &name, double &value) {
  auto it = shim().numbers.find(name);
  value = it == shim().numbers.end() ? 0.0 : it->second;
}
void setString(const std::string &, const std::string &) {}
void getString(const std::string &, std::string &value) { value.clear(); }
}  // namespace option

namespace logger {
void write(const std::string &message, const std::string &level) {
  std::fprintf(level == "error" ? stderr : stdout, "%s\n", message.c_str());
}
}  // namespace logger

namespace fltk {
void initialize() { unavailable("fltk::initialize (no graphics)"); }
void run() { unavailable("fltk::run (no graphics)"); }
}  // namespace fltk

namespace model {
void add(const std::string &) { unavailable("model::add"); }
void remove() { unavailable("model::remove"); }
void setCurrent(const std::string &name) {
  if (name != shim().name) unavailable("model::setCurrent on another model");
}
void getCurrent(std::string &name) { name = shim().name; }
int getDimension() { return shimMesh().dim; }

void getEntities(vectorpair &dimTags, const int dim) {
  dimTags.clear();
  for (auto &e : shimMesh().entities)
    if (dim < 0 || e.dim == dim) dimTags.emplace_back(e.dim, e.tag);
}

void getBoundary(const vectorpair &, vectorpair &, const bool, const bool, const bool) { unavailable("model::getBoundary"); }

void getBoundingBox(const int dim, const int tag, double &xmin, double &ymin, double &zmin, double &xmax, double &ymax,
                    double &zmax) {
  if (dim != -1 || tag != -1) unavailable("model::getBoundingBox of one entity");
  const double *b = shimMesh().bbox;
  xmin = b[0], ymin = b[1], zmin = b[2], xmax = b[3], ymax = b[4], zmax = b[5];
}

void getEntitiesForPhysicalGroup(const int, const int, std::vector<int> &) { unavailable("physical groups by number"); }

void getEntitiesForPhysicalName(const std::string &name, vectorpair &dimTags) {
  dimTags.clear();
  auto it = shimMesh().physicals.find(name);
  if (it != shimMesh().physicals.end()) dimTags = it->second;
}

int addDiscreteEntity(const int, const int, const std::vector<int> &) { unavailable("model::addDiscreteEntity"); }
int addPhysicalGroup(const int, const std::vector<int> &, const int, const std::string &) { unavailable("model::addPhysicalGroup"); }
void setPhysicalName(const int, const int, const std::string &) { unavailable("model::setPhysicalName"); }

namespace mesh {
void generate(const int) { unavailable("mesh::generate"); }

void getElementTypes(std::vector<int> &elementTypes, const int dim, const int tag) {
  elementTypes.clear();
  for (auto &e : shimMesh().entities) {
    if ((dim >= 0 && e.dim != dim) || (tag >= 0 && e.tag != tag)) continue;
    for (auto &b : e.blocks)
      if (std::find(elementTypes.begin(), elementTypes.end(), b.type) == elementTypes.end()) elementTypes.push_back(b.type);
  }
  std::sort(elementTypes.begin(), elementTypes.end());
}

void getElementProperties(const int elementType, std::string &elementName_, int &dim, int &order, int &numNodes,
                          std::vector<double> &localNodeCoord, int &numPrimaryNodes) {
  elementName_ = elementName(elementType);
  dim = femg::elementDim(elementType);
  order = femg::elementOrder(elementType);
  numNodes = femg::elementNodes(elementType);
  numPrimaryNodes = femg::elementVertices(elementType);
  localNodeCoord = referenceNodes(elementType);
}

int getElementType(const std::string &familyName, const int order, const bool serendip) {
  if (serendip) unavailable("serendipity elements");
  if (familyName == "Point") return femg::kPoint;
  if (familyName == "Line") return order == 1 ? femg::kLine2 : order == 2 ? femg::kLine3 : (unavailable("line order > 2"), 0);
  if (familyName == "Triangle") return order == 1 ? femg::kTri3 : order == 2 ? femg::kTri6 : (unavailable("triangle order > 2"), 0);
  if (familyName == "Tetrahedron") return order == 1 ? femg::kTet4 : order == 2 ? femg::kTet10 : (unavailable("tetrahedron order > 2"), 0);
  unavailable(("element family " + familyName).c_str());
}

void getElementsByType(const int elementType, std::vector<std::size_t> &elementTags, std::vector<std::size_t> &nodeTags,
                       const int tag, const std::size_t task, const std::size_t numTasks) {
  const femg::ElementBlock &b = block(elementType, tag);
  const int nn = b.nodesPerElement;
  if (numTasks <= 1) {
    elementTags.assign(b.tags.begin(), b.tags.end());
    nodeTags.resize(b.nodes.size());
    for (size_t i = 0; i < b.nodes.size(); ++i) nodeTags[i] = (std::size_t)b.nodes[i] + 1;
    return;
  }
  int64_t e0, e1;
  taskRange(b.size(), task, numTasks, e0, e1);
  for (int64_t e = e0; e < e1; ++e) {
    if (!elementTags.empty()) elementTags[(size_t)e] = (std::size_t)b.tags[(size_t)e];
    if (!nodeTags.empty())
      for (int k = 0; k < nn; ++k) nodeTags[(size_t)(e * nn + k)] = (std::size_t)b.nodes[(size_t)(e * nn + k)] + 1;
  }
}

void preallocateElementsByType(const int elementType, const bool elementTag, const bool nodeTag,
                               std::vector<std::size_t> &elementTags, std::vector<std::size_t> &nodeTags, const int tag) {
  const femg::ElementBlock &b = block(elementType, tag);
  if (elementTag) elementTags.assign((size_t)b.size(), 0);
  if (nodeTag) nodeTags.assign(b.nodes.size(), 0);
}

void addElementsByType(const int, const int, const std::vector<std::size_t> &, const std::vector<std::size_t> &) {
  unavailable("mesh::addElementsByType");
}

void getNodes(std::vector<std::size_t> &, std::vector<double> &, std::vector<double> &, const int, const int, const bool,
              const bool) {
  unavailable("mesh::getNodes");
}

void getNode(const std::size_t nodeTag, std::vector<double> &coord, std::vector<double> &parametricCoord, int &dim, int &tag) {
  const femg::Mesh &m = shimMesh();
  if (nodeTag < 1 || (int64_t)nodeTag > m.nNodes()) throw std::runtime_error("gmsh stand-in: unknown node");
  coord.assign(&m.xyz[3 * (nodeTag - 1)], &m.xyz[3 * (nodeTag - 1)] + 3);
  parametricCoord.clear();
  dim = m.dim;
  tag = 1;
}

void getNodesByElementType(const int elementType, std::vector<std::size_t> &nodeTags, std::vector<double> &coord,
                           std::vector<double> &parametricCoord, const int tag, const bool returnParametricCoord) {
  const femg::Mesh &m = shimMesh();
  const femg::ElementBlock &b = block(elementType, tag);
  if (returnParametricCoord) unavailable("parametric node coordinates");
  nodeTags.resize(b.nodes.size());
  coord.resize(3 * b.nodes.size());
  parametricCoord.clear();
  for (size_t i = 0; i < b.nodes.size(); ++i) {
    nodeTags[i] = (std::size_t)b.nodes[i] + 1;
    for (int c = 0; c < 3; ++c) coord[3 * i + c] = m.xyz[3 * (size_t)b.nodes[i] + c];
  }
}

void getElement(const std::size_t, int &, std::vector<std::size_t> &, int &, int &) { unavailable("mesh::getElement"); }
void getElementByCoordinates(const double, const double, const double, std::size_t &, int &, std::vector<std::size_t> &,
                             double &, double &, double &, const int, const bool) {
  unavailable("mesh::getElementByCoordinates");
}
void rebuildElementCache(const bool) {}

void preallocateJacobians(const int elementType, const int numEvaluationPoints, const bool allocateJacobians,
                          const bool allocateDeterminants, const bool allocateCoord, std::vector<double> &jacobians,
                          std::vector<double> &determinants, std::vector<double> &coord, const int tag) {
  const size_t n = (size_t)block(elementType, tag).size() * (size_t)numEvaluationPoints;
  if (allocateJacobians) jacobians.assign(9 * n, 0.0);
  if (allocateDeterminants) determinants.assign(n, 0.0);
  if (allocateCoord) coord.assign(3 * n, 0.0);
}

void getJacobians(const int elementType, const std::vector<double> &localCoord, std::vector<double> &jacobians,
                  std::vector<double> &determinants, std::vector<double> &coord, const int tag, const std::size_t task,
                  const std::size_t numTasks) {
  const femg::Mesh &m = shimMesh();
  const femg::ElementBlock &b = block(elementType, tag);
  const int nq = (int)(localCoord.size() / 3);
  const int nn = b.nodesPerElement;
  const int dim = femg::elementDim(elementType);
  const size_t total = (size_t)b.size() * nq;
  if (numTasks <= 1) {
    if (jacobians.size() != 9 * total) jacobians.assign(9 * total, 0.0);
    if (determinants.size() != total) determinants.assign(total, 0.0);
    if (coord.size() != 3 * total) coord.assign(3 * total, 0.0);
  }
  std::vector<double> val((size_t)nq * nn), grad((size_t)nq * nn * 3);
  for (int q = 0; q < nq; ++q) femg::lagrangeBasis(elementType, &localCoord[3 * q], &val[(size_t)q * nn], &grad[(size_t)q * nn * 3]);
  int64_t e0, e1;
  taskRange(b.size(), task, numTasks, e0, e1);
  for (int64_t e = e0; e < e1; ++e) {
    const int64_t *v = &b.nodes[(size_t)(e * nn)];
    for (int q = 0; q < nq; ++q) {
      double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, x[3] = {0, 0, 0};
      for (int k = 0; k < nn; ++k) {
        const double *X = &m.xyz[3 * (size_t)v[k]];
        const double *g = &grad[((size_t)q * nn + k) * 3];
        const double w = val[(size_t)q * nn + k];
        for (int c = 0; c < dim; ++c)
          for (int r = 0; r < 3; ++r) J[3 * c + r] += X[r] * g[c];
        for (int r = 0; r < 3; ++r) x[r] += X[r] * w;
      }
      if (dim == 2) {
        const double nx = J[1] * J[5] - J[2] * J[4], ny = J[2] * J[3] - J[0] * J[5], nz = J[0] * J[4] - J[1] * J[3];
        const double len = std::sqrt(nx * nx + ny * ny + nz * nz);
        J[6] = nx / len, J[7] = ny / len, J[8] = nz / len;
      } else if (dim == 1) {
        // a curve in the xy-plane: its unit normal in the plane, then z
        const double len = std::sqrt(J[0] * J[0] + J[1] * J[1] + J[2] * J[2]);
        if (J[2] != 0.0) unavailable("curves out of the xy-plane");
        J[3] = -J[1] / len, J[4] = J[0] / len, J[5] = 0.0;
        J[6] = 0.0, J[7] = 0.0, J[8] = 1.0;
      } else if (dim == 0) {
        J[0] = J[4] = J[8] = 1.0;
      }
      const double det = J[0] * (J[4] * J[8] - J[7] * J[5]) - J[3] * (J[1] * J[8] - J[7] * J[2]) + J[6] * (J[1] * J[5] - J[4] * J[2]);
      const size_t at = (size_t)e * nq + q;
      if (!jacobians.empty())
        for (int k = 0; k < 9; ++k) jacobians[9 * at + k] = J[k];
      if (!determinants.empty()) determinants[at] = det;
      if (!coord.empty())
        for (int r = 0; r < 3; ++r) coord[3 * at + r] = x[r];
    }
  }
}

void getJacobian(const std::size_t, const std::vector<double> &, std::vector<double> &, std::vector<double> &,
                 std::vector<double> &) {
  unavailable("mesh::getJacobian of one element");
}

void getIntegrationPoints(const int elementType, const std::string &integrationType, std::vector<double> &localCoord,
                          std::vector<double> &weights) {
  const femg::QuadRule r = femg::gaussRule(integrationType, elementType);
  localCoord = r.points;
  weights = r.weights;
}

void preallocateBasisFunctionsOrientation(const int elementType, std::vector<int> &basisFunctionsOrientation, const int tag) {
  basisFunctionsOrientation.assign((size_t)block(elementType, tag).size(), 0);
}

void getBasisFunctionsOrientation(const int elementType, const std::string &functionSpaceType,
                                  std::vector<int> &basisFunctionsOrientation, const int tag, const std::size_t task,
                                  const std::size_t numTasks) {
  bool der = false;
  const femg::FunctionSpace fs = parseSpace(functionSpaceType, &der);
  const femg::ElementBlock &b = block(elementType, tag);
  if (numTasks <= 1 && basisFunctionsOrientation.size() != (size_t)b.size())
    basisFunctionsOrientation.assign((size_t)b.size(), 0);
  int64_t e0, e1;
  taskRange(b.size(), task, numTasks, e0, e1);
  for (int64_t e = e0; e < e1; ++e) basisFunctionsOrientation[(size_t)e] = orientationOf(fs, b, e);
}

void getBasisFunctionsOrientationForElement(const std::size_t, const std::string &, int &) {
  unavailable("mesh::getBasisFunctionsOrientationForElement");
}

int getNumberOfOrientations(const int elementType, const std::string &functionSpaceType) {
  bool der = false;
  const femg::FunctionSpace fs = parseSpace(functionSpaceType, &der);
  if (fs.orientationFree()) return 1;
  const int dim = femg::elementDim(elementType);
  int n = 1;
  for (size_t k = 0; k < femg::simplexEdges(dim).size(); ++k) n *= 2;  // edge reversal bits
  if (dim == 3 && !(fs.type == femg::SpaceType::HCurl && fs.order == 0))
    for (int f = 0; f < 4; ++f) n *= 6;  // face permutations
  return n;
}

void getBasisFunctions(const int elementType, const std::vector<double> &localCoord, const std::string &functionSpaceType,
                       int &numComponents, std::vector<double> &basisFunctions, int &numOrientations,
                       const std::vector<int> &wantedOrientations) {
  bool derivative = false;
  const femg::FunctionSpace fs = parseSpace(functionSpaceType, &derivative);
  const int dim = femg::elementDim(elementType);
  const int nq = (int)(localCoord.size() / 3);
  std::vector<int> orient = wantedOrientations;
  if (orient.empty()) {
    if (!fs.orientationFree()) unavailable("basis functions of every orientation");
    orient = {0};
  }
  numOrientations = (int)orient.size();
  basisFunctions.clear();
  if (fs.type == femg::SpaceType::Lagrange) {
    const int n = femg::elementNodes(elementType);
    numComponents = derivative ? 3 : 1;
    std::vector<double> val(n), grad(3 * n);
    for (size_t o = 0; o < orient.size(); ++o)
      for (int q = 0; q < nq; ++q) {
        femg::lagrangeBasis(elementType, &localCoord[3 * q], val.data(), grad.data());
        for (int i = 0; i < n; ++i)
          for (int c = 0; c < numComponents; ++c) basisFunctions.push_back(derivative ? grad[3 * i + c] : val[i]);
      }
    return;
  }
  if (fs.type == femg::SpaceType::HCurl) {
    const int n = femg::hcurlCount(dim, fs.order);
    numComponents = 3;
    std::vector<double> val(3 * n), curl(3 * n);
    for (int code : orient)
      for (int q = 0; q < nq; ++q) {
        femg::hcurlBasis(dim, fs.order, code, &localCoord[3 * q], val.data(), curl.data());
        for (int i = 0; i < n; ++i)
          for (int c = 0; c < 3; ++c) basisFunctions.push_back(derivative ? curl[3 * i + c] : val[3 * i + c]);
      }
    return;
  }
  const int n = femg::hierarchicalCount(dim, fs.order);
  numComponents = derivative ? 3 : 1;
  std::vector<double> val(n), grad(3 * n);
  for (int code : orient)
    for (int q = 0; q < nq; ++q) {
      femg::hierarchicalBasis(dim, fs.order, code, &localCoord[3 * q], val.data(), grad.data());
      for (int i = 0; i < n; ++i)
        for (int c = 0; c < numComponents; ++c) basisFunctions.push_back(derivative ? grad[3 * i + c] : val[i]);
    }
}

void getKeys(const int elementType, const std::string &functionSpaceType, std::vector<int> &typeKeys,
             std::vector<std::size_t> &entityKeys, std::vector<double> &coord, const int tag, const bool returnCoord) {
  bool der = false;
  const femg::FunctionSpace fs = parseSpace(functionSpaceType, &der);
  std::vector<uint64_t> ek;
  fs.getKeys(shimMesh(), block(elementType, tag), returnCoord, typeKeys, ek, coord, nullptr);
  entityKeys.assign(ek.begin(), ek.end());
}

void getKeysForElement(const std::size_t, const std::string &, std::vector<int> &, std::vector<std::size_t> &,
                       std::vector<double> &, const bool) {
  unavailable("mesh::getKeysForElement");
}

int getNumberOfKeys(const int elementType, const std::string &functionSpaceType) {
  bool der = false;
  return parseSpace(functionSpaceType, &der).keysPerElement(elementType);
}

// (dimension of the key's entity, order) per key. The keys are those getKeys
// returned for one element block, element by element, so the local position
// of a key in its element gives its entity.
void getKeysInformation(const std::vector<int> &typeKeys, const std::vector<std::size_t> &entityKeys, const int elementType,
                        const std::string &functionSpaceType, gmsh::vectorpair &infoKeys) {
  bool der = false;
  const femg::FunctionSpace fs = parseSpace(functionSpaceType, &der);
  const int nk = fs.keysPerElement(elementType);
  if (nk <= 0 || typeKeys.size() % (size_t)nk != 0 || entityKeys.size() != typeKeys.size())
    throw std::runtime_error("gmsh stand-in: keys are not whole elements of the type");
  // the key dimensions of one element, from a one-element block
  femg::ElementBlock one;
  const femg::ElementBlock *pb = nullptr;
  for (auto &ent : shimMesh().entities)
    for (auto &bb : ent.blocks)
      if (!pb && bb.type == elementType && bb.size() > 0) pb = &bb;
  if (!pb) throw std::runtime_error("gmsh stand-in: no element of the type");
  const femg::ElementBlock &b = *pb;
  one.type = b.type;
  one.nodesPerElement = b.nodesPerElement;
  one.tags.assign(b.tags.begin(), b.tags.begin() + 1);
  one.nodes.assign(b.nodes.begin(), b.nodes.begin() + b.nodesPerElement);
  std::vector<int> tk, info;
  std::vector<uint64_t> ek;
  std::vector<double> co;
  fs.getKeys(shimMesh(), one, false, tk, ek, co, &info);
  infoKeys.resize(typeKeys.size());
  for (size_t j = 0; j < typeKeys.size(); ++j) infoKeys[j] = {info[j % (size_t)nk], std::max(1, fs.order)};
}

void getPeriodicKeys(const int, const std::string &, const int, int &, std::vector<int> &, std::vector<int> &,
                     std::vector<std::size_t> &, std::vector<std::size_t> &, std::vector<double> &, std::vector<double> &,
                     const bool) {
  unavailable("mesh::getPeriodicKeys");
}
void getPeriodicNodes(const int, const int, int &, std::vector<std::size_t> &, std::vector<std::size_t> &,
                      std::vector<double> &, const bool) {
  unavailable("mesh::getPeriodicNodes");
}
void getPeriodic(const int, const std::vector<int> &, std::vector<int> &) { unavailable("mesh::getPeriodic"); }
void preallocateBarycenters(const int, std::vector<double> &, const int) { unavailable("mesh::preallocateBarycenters"); }
void getBarycenters(const int, const int, const bool, const bool, std::vector<double> &, const std::size_t, const std::size_t) {
  unavailable("mesh::getBarycenters");
}
void reorderElements(const int, const int, const std::vector<std::size_t> &) { unavailable("mesh::reorderElements"); }
void setTransfiniteCurve(const int, const int, const std::string &, const double) { unavailable("mesh::setTransfiniteCurve"); }
}  // namespace mesh

namespace geo {
int addPoint(const double, const double, const double, const double, const int) { unavailable("geo::addPoint"); }
int addLine(const int, const int, const int) { unavailable("geo::addLine"); }
int addCircleArc(const int, const int, const int, const int, const double, const double, const double) {
  unavailable("geo::addCircleArc");
}
int addCurveLoop(const std::vector<int> &, const int, const bool) { unavailable("geo::addCurveLoop"); }
int addPlaneSurface(const std::vector<int> &, const int) { unavailable("geo::addPlaneSurface"); }
int addSurfaceFilling(const std::vector<int> &, const int, const int) { unavailable("geo::addSurfaceFilling"); }
int addSurfaceLoop(const std::vector<int> &, const int) { unavailable("geo::addSurfaceLoop"); }
int addVolume(const std::vector<int> &, const int) { unavailable("geo::addVolume"); }
void extrude(const vectorpair &, const double, const double, const double, vectorpair &, const std::vector<int> &,
             const std::vector<double> &, const bool) {
  unavailable("geo::extrude");
}
void synchronize() { unavailable("geo::synchronize"); }
}  // namespace geo
}  // namespace model

namespace view {
int add(const std::string &, const int) { unavailable("view::add"); }
void remove(const int) { unavailable("view::remove"); }
void addModelData(const int, const int, const std::string &, const std::string &, const std::vector<std::size_t> &,
                  const std::vector<std::vector<double>> &, const double, const int, const int) {
  unavailable("view::addModelData");
}
void write(const int, const std::string &, const bool) { unavailable("view::write"); }
void probe(const int, const double, const double, const double, std::vector<double> &, double &, const int, const int,
           const bool, const double, const std::vector<double> &, const std::vector<double> &, const std::vector<double> &,
           const int) {
  unavailable("view::probe");
}
}  // namespace view

}  // namespace gmsh
