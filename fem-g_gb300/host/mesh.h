// Synthetic meshes and the mesh queries the assembly path needs.
//
// The reference obtains its mesh from gmsh (gmsh::model::mesh::getElementTypes,
// getNodesByElementType, getKeys, getJacobians; called from
// src/problem/Formulation.cpp:1418-1493 and src/term/Assembler.cpp:69-155).
// gmsh is not part of the reference tree, so this file is the stand-in: it
// builds the structured, jittered simplex meshes of the benchmark workloads and
// answers the same questions (entities, element blocks, node coordinates,
// global edge/face numbering used for hierarchical keys).
#pragma once
#include <array>
#include <cstdint>
#include <map>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>

namespace femg {

// gmsh element type codes (same numbers as gmsh's MSH format)
enum ElementType : int {
  kPoint = 15,
  kLine2 = 1,
  kLine3 = 8,
  kTri3 = 2,
  kTri6 = 9,
  kTet4 = 4,
  kTet10 = 11,
};

int elementDim(int type);
int elementNodes(int type);
int elementOrder(int type);
int elementVertices(int type);  // primary (corner) nodes

struct ElementBlock {
  int type = 0;
  int nodesPerElement = 0;
  std::vector<int64_t> tags;   // element tags (1-based, unique in the mesh)
  std::vector<int64_t> nodes;  // [E][nodesPerElement], 0-based node indices
  int64_t size() const { return (int64_t)tags.size(); }
};

struct Entity {
  int dim = 0;
  int tag = 0;
  std::vector<ElementBlock> blocks;
};

struct Mesh {
  int dim = 0;                      // model dimension
  std::vector<double> xyz;          // [nNodes][3]; node tag = index + 1
  std::vector<Entity> entities;     // sorted by (dim, tag) like gmsh::model::getEntities
  std::map<std::string, std::vector<std::pair<int, int>>> physicals;  // name -> (dim, tag)
  double bbox[6] = {0, 0, 0, 0, 0, 0};

  int64_t nNodes() const { return (int64_t)xyz.size() / 3; }
  const Entity *find(int dim, int tag) const;
  void finalize();  // bbox + global edge/face numbering

  // Global edge / face numbering (1-based tags) keyed by sorted node indices,
  // numbered in order of first appearance over entities of decreasing
  // dimension, elements in order, local edges/faces in local order.
  struct KeyHash {
    size_t operator()(const std::array<int64_t, 3> &k) const noexcept;
  };
  std::unordered_map<std::array<int64_t, 3>, int64_t, KeyHash> edgeTag;  // {a, b, -1}
  std::unordered_map<std::array<int64_t, 3>, int64_t, KeyHash> faceTag;
  int64_t edgeTagOf(int64_t a, int64_t b) const;
  int64_t faceTagOf(int64_t a, int64_t b, int64_t c) const;
};

// Local edge and face tables of the reference simplices (shared by the
// geometric basis, the keys and the hierarchical basis).
const std::vector<std::array<int, 2>> &simplexEdges(int dim);
const std::vector<std::array<int, 3>> &simplexFaces(int dim);

// Unit square, m x m cells, each split into 2 triangles along the (0,0)-(1,1)
// diagonal; interior vertices jittered uniformly by +-jitter*h in x and y;
// order 1 (3-node) or 2 (6-node, mid-edge nodes at the midpoints). Entities:
// surface 1 (physical "omega"), curves 1..4 (bottom, right, top, left; physical
// "gammaDir"), points 1..4.
Mesh makeSquareTri(int m, int order, double jitter, uint64_t seed);

// Unit cube, m^3 cells, each split into 6 Kuhn tetrahedra sharing the
// (0,0,0)-(1,1,1) diagonal, interior vertices jittered by +-jitter*h in x,y,z.
// Order 1 (4-node) or 2 (10-node, mid-edge nodes at midpoints). Entities:
// volume 1 (physical "omega"), boundary faces 1..6 (physical "gamma").
Mesh makeCubeTet(int m, int order, double jitter, uint64_t seed);

// Seeded generator used for every synthetic input: std::mt19937_64 with an
// explicit 53-bit mantissa conversion so x86 and Arm produce identical values.
struct Rng {
  std::mt19937_64 gen;  // the standard fixes its output sequence
  explicit Rng(uint64_t seed) : gen(seed) {}
  uint64_t next() { return gen(); }
  double uniform();          // [0,1)
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  double normal();           // Box-Muller
};

}  // namespace femg
