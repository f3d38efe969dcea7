// Stand-in declarations of the gmsh C++ API — TEST INFRASTRUCTURE ONLY.
//
// The reference (GmshFEM) calls gmsh for its meshes, quadrature rules, basis
// tables, DOF keys and Jacobians. gmsh is neither vendored with the reference
// nor installed here, so the oracle build compiles the reference's own
// src/ against these declarations, written from the reference's call sites,
// and links gmsh_shim.cpp, which answers them from this project's synthetic
// meshes and reference-element tables (the same ones the GPU path's host
// mirror uses). Functions the assembly path never reaches throw.
#pragma once
#include <cstddef>
#include <string>
#include <utility>
#include <vector>

#define GMSH_API_VERSION "stand-in (oracle)"

namespace gmsh {

typedef std::vector<std::pair<int, int>> vectorpair;

void initialize(int argc = 0, char **argv = 0, const bool readConfigFiles = true, const bool run = false);
void finalize();

namespace option {
void setNumber(const std::string &name, const double value);
void getNumber(const std::string &name, double &value);
void setString(const std::string &name, const std::string &value);
void getString(const std::string &name, std::string &value);
}  // namespace option

namespace logger {
void write(const std::string &message, const std::string &level = "info");
}  // namespace logger

namespace fltk {
void initialize();
void run();
}  // namespace fltk

namespace model {
void add(const std::string &name);
void remove();
void setCurrent(const std::string &name);
void getCurrent(std::string &name);
int getDimension();
void getEntities(vectorpair &dimTags, const int dim = -1);
void getBoundary(const vectorpair &dimTags, vectorpair &outDimTags, const bool combined = true, const bool oriented = true,
                 const bool recursive = false);
void getBoundingBox(const int dim, const int tag, double &xmin, double &ymin, double &zmin, double &xmax, double &ymax,
                    double &zmax);
void getEntitiesForPhysicalGroup(const int dim, const int tag, std::vector<int> &tags);
void getEntitiesForPhysicalName(const std::string &name, vectorpair &dimTags);
int addDiscreteEntity(const int dim, const int tag = -1, const std::vector<int> &boundary = std::vector<int>());
int addPhysicalGroup(const int dim, const std::vector<int> &tags, const int tag = -1, const std::string &name = "");
void setPhysicalName(const int dim, const int tag, const std::string &name);

namespace mesh {
void generate(const int dim = 3);
void getElementTypes(std::vector<int> &elementTypes, const int dim = -1, const int tag = -1);
void getElementProperties(const int elementType, std::string &elementName, int &dim, int &order, int &numNodes,
                          std::vector<double> &localNodeCoord, int &numPrimaryNodes);
int getElementType(const std::string &familyName, const int order, const bool serendip = false);
void getElementsByType(const int elementType, std::vector<std::size_t> &elementTags, std::vector<std::size_t> &nodeTags,
                       const int tag = -1, const std::size_t task = 0, const std::size_t numTasks = 1);
void preallocateElementsByType(const int elementType, const bool elementTag, const bool nodeTag,
                               std::vector<std::size_t> &elementTags, std::vector<std::size_t> &nodeTags, const int tag = -1);
void addElementsByType(const int tag, const int elementType, const std::vector<std::size_t> &elementTags,
                       const std::vector<std::size_t> &nodeTags);
void getNodes(std::vector<std::size_t> &nodeTags, std::vector<double> &coord, std::vector<double> &parametricCoord,
              const int dim = -1, const int tag = -1, const bool includeBoundary = false,
              const bool returnParametricCoord = true);
void getNode(const std::size_t nodeTag, std::vector<double> &coord, std::vector<double> &parametricCoord, int &dim, int &tag);
void getNodesByElementType(const int elementType, std::vector<std::size_t> &nodeTags, std::vector<double> &coord,
                           std::vector<double> &parametricCoord, const int tag = -1, const bool returnParametricCoord = true);
void getElement(const std::size_t elementTag, int &elementType, std::vector<std::size_t> &nodeTags, int &dim, int &tag);
void getElementByCoordinates(const double x, const double y, const double z, std::size_t &elementTag, int &elementType,
                             std::vector<std::size_t> &nodeTags, double &u, double &v, double &w, const int dim = -1,
                             const bool strict = false);
void rebuildElementCache(const bool onlyIfNecessary = true);
void preallocateJacobians(const int elementType, const int numEvaluationPoints, const bool allocateJacobians,
                          const bool allocateDeterminants, const bool allocateCoord, std::vector<double> &jacobians,
                          std::vector<double> &determinants, std::vector<double> &coord, const int tag = -1);
void getJacobians(const int elementType, const std::vector<double> &localCoord, std::vector<double> &jacobians,
                  std::vector<double> &determinants, std::vector<double> &coord, const int tag = -1,
                  const std::size_t task = 0, const std::size_t numTasks = 1);
void getJacobian(const std::size_t elementTag, const std::vector<double> &localCoord, std::vector<double> &jacobians,
                 std::vector<double> &determinants, std::vector<double> &coord);
void getIntegrationPoints(const int elementType, const std::string &integrationType, std::vector<double> &localCoord,
                          std::vector<double> &weights);
void preallocateBasisFunctionsOrientation(const int elementType, std::vector<int> &basisFunctionsOrientation,
                                          const int tag = -1);
void getBasisFunctionsOrientation(const int elementType, const std::string &functionSpaceType,
                                  std::vector<int> &basisFunctionsOrientation, const int tag = -1,
                                  const std::size_t task = 0, const std::size_t numTasks = 1);
void getBasisFunctionsOrientationForElement(const std::size_t elementTag, const std::string &functionSpaceType,
                                            int &basisFunctionsOrientation);
int getNumberOfOrientations(const int elementType, const std::string &functionSpaceType);
void getBasisFunctions(const int elementType, const std::vector<double> &localCoord, const std::string &functionSpaceType,
                       int &numComponents, std::vector<double> &basisFunctions, int &numOrientations,
                       const std::vector<int> &wantedOrientations = std::vector<int>());
void getKeys(const int elementType, const std::string &functionSpaceType, std::vector<int> &typeKeys,
             std::vector<std::size_t> &entityKeys, std::vector<double> &coord, const int tag = -1,
             const bool returnCoord = true);
void getKeysForElement(const std::size_t elementTag, const std::string &functionSpaceType, std::vector<int> &typeKeys,
                       std::vector<std::size_t> &entityKeys, std::vector<double> &coord, const bool returnCoord = true);
int getNumberOfKeys(const int elementType, const std::string &functionSpaceType);
void getKeysInformation(const std::vector<int> &typeKeys, const std::vector<std::size_t> &entityKeys, const int elementType,
                        const std::string &functionSpaceType, gmsh::vectorpair &infoKeys);
void getPeriodicKeys(const int elementType, const std::string &functionSpaceType, const int tag, int &tagMaster,
                     std::vector<int> &typeKeys, std::vector<int> &typeKeysMaster, std::vector<std::size_t> &entityKeys,
                     std::vector<std::size_t> &entityKeysMaster, std::vector<double> &coord,
                     std::vector<double> &coordMaster, const bool returnCoord = true);
void getPeriodicNodes(const int dim, const int tag, int &tagMaster, std::vector<std::size_t> &nodeTags,
                      std::vector<std::size_t> &nodeTagsMaster, std::vector<double> &affineTransform,
                      const bool includeHighOrderNodes = false);
void getPeriodic(const int dim, const std::vector<int> &tags, std::vector<int> &tagMaster);
void preallocateBarycenters(const int elementType, std::vector<double> &barycenters, const int tag = -1);
void getBarycenters(const int elementType, const int tag, const bool fast, const bool primary,
                    std::vector<double> &barycenters, const std::size_t task = 0, const std::size_t numTasks = 1);
void reorderElements(const int elementType, const int tag, const std::vector<std::size_t> &ordering);
void setTransfiniteCurve(const int tag, const int numNodes, const std::string &meshType = "Progression",
                         const double coef = 1.);
}  // namespace mesh

namespace geo {
int addPoint(const double x, const double y, const double z, const double meshSize = 0., const int tag = -1);
int addLine(const int startTag, const int endTag, const int tag = -1);
int addCircleArc(const int startTag, const int centerTag, const int endTag, const int tag = -1, const double nx = 0.,
                 const double ny = 0., const double nz = 0.);
int addCurveLoop(const std::vector<int> &curveTags, const int tag = -1, const bool reorient = false);
int addPlaneSurface(const std::vector<int> &wireTags, const int tag = -1);
int addSurfaceFilling(const std::vector<int> &wireTags, const int tag = -1, const int sphereCenterTag = -1);
int addSurfaceLoop(const std::vector<int> &surfaceTags, const int tag = -1);
int addVolume(const std::vector<int> &shellTags, const int tag = -1);
void extrude(const vectorpair &dimTags, const double dx, const double dy, const double dz, vectorpair &outDimTags,
             const std::vector<int> &numElements = std::vector<int>(), const std::vector<double> &heights = std::vector<double>(),
             const bool recombine = false);
void synchronize();
}  // namespace geo
}  // namespace model

namespace view {
int add(const std::string &name, const int tag = -1);
void remove(const int tag);
void addModelData(const int tag, const int step, const std::string &modelName, const std::string &dataType,
                  const std::vector<std::size_t> &tags, const std::vector<std::vector<double>> &data, const double time = 0.,
                  const int numComponents = -1, const int partition = 0);
void write(const int tag, const std::string &fileName, const bool append = false);
void probe(const int tag, const double x, const double y, const double z, std::vector<double> &values, double &distance,
           const int step = -1, const int numComp = -1, const bool gradient = false, const double distanceMax = 0.,
           const std::vector<double> &xElemCoord = std::vector<double>(),
           const std::vector<double> &yElemCoord = std::vector<double>(),
           const std::vector<double> &zElemCoord = std::vector<double>(), const int dim = -1);
}  // namespace view

}  // namespace gmsh
