#include "mesh.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <unordered_map>

namespace femg {

int elementDim(int type) {
  switch (type) {
    case kPoint: return 0;
    case kLine2: case kLine3: return 1;
    case kTri3: case kTri6: return 2;
    case kTet4: case kTet10: return 3;
  }
  throw std::invalid_argument("unsupported element type");
}

int elementNodes(int type) {
  switch (type) {
    case kPoint: return 1;
    case kLine2: return 2;
    case kLine3: return 3;
    case kTri3: return 3;
    case kTri6: return 6;
    case kTet4: return 4;
    case kTet10: return 10;
  }
  throw std::invalid_argument("unsupported element type");
}

int elementOrder(int type) {
  switch (type) {
    case kPoint: return 0;
    case kLine2: case kTri3: case kTet4: return 1;
    case kLine3: case kTri6: case kTet10: return 2;
  }
  throw std::invalid_argument("unsupported element type");
}

int elementVertices(int type) { return elementDim(type) + 1; }

const std::vector<std::array<int, 2>> &simplexEdges(int dim) {
  static const std::vector<std::array<int, 2>> e1 = {{0, 1}};
  static const std::vector<std::array<int, 2>> e2 = {{0, 1}, {1, 2}, {2, 0}};
  static const std::vector<std::array<int, 2>> e3 = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
  static const std::vector<std::array<int, 2>> e0 = {};
  switch (dim) {
    case 1: return e1;
    case 2: return e2;
    case 3: return e3;
  }
  return e0;
}

const std::vector<std::array<int, 3>> &simplexFaces(int dim) {
  static const std::vector<std::array<int, 3>> f2 = {{0, 1, 2}};
  static const std::vector<std::array<int, 3>> f3 = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
  static const std::vector<std::array<int, 3>> f0 = {};
  if (dim == 2) return f2;
  if (dim == 3) return f3;
  return f0;
}

double Rng::uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }

double Rng::normal() {
  // Box-Muller; one draw per call (the second variate is discarded so the
  // sequence does not depend on call parity)
  double u1 = uniform(), u2 = uniform();
  if (u1 <= 0.0) u1 = 1.0 / 9007199254740992.0;
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586476925 * u2);
}

const Entity *Mesh::find(int d, int t) const {
  for (auto &e : entities)
    if (e.dim == d && e.tag == t) return &e;
  return nullptr;
}

namespace {
struct PairHash {
  size_t operator()(const std::pair<int64_t, int64_t> &p) const noexcept {
    uint64_t h = (uint64_t)p.first * 0x9E3779B97F4A7C15ull ^ ((uint64_t)p.second + 0x632BE59BD9B4E019ull);
    h ^= h >> 29;
    return (size_t)(h * 0xBF58476D1CE4E5B9ull);
  }
};
}  // namespace

size_t Mesh::KeyHash::operator()(const std::array<int64_t, 3> &k) const noexcept {
  uint64_t h = 0x243F6A8885A308D3ull;
  for (int i = 0; i < 3; ++i) {
    h ^= (uint64_t)k[i] + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xBF58476D1CE4E5B9ull;
  }
  return (size_t)(h ^ (h >> 31));
}

int64_t Mesh::edgeTagOf(int64_t a, int64_t b) const {
  auto it = edgeTag.find({std::min(a, b), std::max(a, b), -1});
  if (it == edgeTag.end()) throw std::runtime_error("edge not in mesh");
  return it->second;
}

int64_t Mesh::faceTagOf(int64_t a, int64_t b, int64_t c) const {
  std::array<int64_t, 3> k = {a, b, c};
  std::sort(k.begin(), k.end());
  auto it = faceTag.find(k);
  if (it == faceTag.end()) throw std::runtime_error("face not in mesh");
  return it->second;
}

void Mesh::finalize() {
  const int64_t n = nNodes();
  for (int c = 0; c < 3; ++c) {
    bbox[c] = n ? xyz[c] : 0.0;
    bbox[3 + c] = n ? xyz[c] : 0.0;
  }
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      bbox[c] = std::min(bbox[c], xyz[3 * i + c]);
      bbox[3 + c] = std::max(bbox[3 + c], xyz[3 * i + c]);
    }
  std::sort(entities.begin(), entities.end(), [](const Entity &a, const Entity &b) {
    return a.dim != b.dim ? a.dim < b.dim : a.tag < b.tag;
  });
  // global edges / faces, first appearance over entities of decreasing dimension
  edgeTag.clear();
  faceTag.clear();
  edgeTag.reserve(8 * (size_t)nNodes());
  faceTag.reserve(12 * (size_t)nNodes());
  int64_t nextEdge = 1, nextFace = 1;
  for (int d = 3; d >= 1; --d) {
    for (auto &ent : entities) {
      if (ent.dim != d) continue;
      for (auto &blk : ent.blocks) {
        const int nn = blk.nodesPerElement;
        const auto &le = simplexEdges(d);
        const auto &lf = simplexFaces(d);
        for (int64_t e = 0; e < blk.size(); ++e) {
          const int64_t *v = &blk.nodes[e * nn];
          for (auto &ed : le) {
            std::array<int64_t, 3> k = {std::min(v[ed[0]], v[ed[1]]), std::max(v[ed[0]], v[ed[1]]), -1};
            if (edgeTag.emplace(k, nextEdge).second) ++nextEdge;
          }
          for (auto &fc : lf) {
            std::array<int64_t, 3> k = {v[fc[0]], v[fc[1]], v[fc[2]]};
            std::sort(k.begin(), k.end());
            if (faceTag.emplace(k, nextFace).second) ++nextFace;
          }
        }
      }
    }
  }
}

Mesh makeSquareTri(int m, int order, double jitter, uint64_t seed) {
  if (m < 1 || (order != 1 && order != 2)) throw std::invalid_argument("makeSquareTri");
  Mesh mesh;
  mesh.dim = 2;
  const double h = 1.0 / m;
  const int64_t nv = (int64_t)(m + 1) * (m + 1);
  mesh.xyz.assign(3 * nv, 0.0);
  Rng rng(seed);
  for (int j = 0; j <= m; ++j)
    for (int i = 0; i <= m; ++i) {
      int64_t v = i + (int64_t)j * (m + 1);
      double x = i * h, y = j * h;
      if (i > 0 && i < m && j > 0 && j < m) {
        x += rng.uniform(-jitter * h, jitter * h);
        y += rng.uniform(-jitter * h, jitter * h);
      }
      mesh.xyz[3 * v] = x;
      mesh.xyz[3 * v + 1] = y;
    }
  auto V = [&](int i, int j) { return (int64_t)i + (int64_t)j * (m + 1); };
  std::unordered_map<std::pair<int64_t, int64_t>, int64_t, PairHash> mid;
  auto midNode = [&](int64_t a, int64_t b) -> int64_t {
    std::pair<int64_t, int64_t> k = {std::min(a, b), std::max(a, b)};
    auto it = mid.find(k);
    if (it != mid.end()) return it->second;
    int64_t id = mesh.nNodes();
    for (int c = 0; c < 3; ++c) mesh.xyz.push_back(0.5 * (mesh.xyz[3 * a + c] + mesh.xyz[3 * b + c]));
    mid.emplace(k, id);
    return id;
  };
  const int triType = order == 1 ? kTri3 : kTri6;
  const int lineType = order == 1 ? kLine2 : kLine3;
  int64_t nextTag = 1;
  Entity surf;
  surf.dim = 2;
  surf.tag = 1;
  ElementBlock tb;
  tb.type = triType;
  tb.nodesPerElement = elementNodes(triType);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) {
      int64_t tri[2][3] = {{V(i, j), V(i + 1, j), V(i + 1, j + 1)}, {V(i, j), V(i + 1, j + 1), V(i, j + 1)}};
      for (auto &t : tri) {
        tb.tags.push_back(nextTag++);
        for (int k = 0; k < 3; ++k) tb.nodes.push_back(t[k]);
        if (order == 2)
          for (auto &ed : simplexEdges(2)) tb.nodes.push_back(midNode(t[ed[0]], t[ed[1]]));
      }
    }
  surf.blocks.push_back(std::move(tb));
  mesh.entities.push_back(std::move(surf));
  // boundary curves
  for (int c = 1; c <= 4; ++c) {
    Entity cur;
    cur.dim = 1;
    cur.tag = c;
    ElementBlock lb;
    lb.type = lineType;
    lb.nodesPerElement = elementNodes(lineType);
    for (int s = 0; s < m; ++s) {
      int64_t a, b;
      if (c == 1) { a = V(s, 0); b = V(s + 1, 0); }
      else if (c == 2) { a = V(m, s); b = V(m, s + 1); }
      else if (c == 3) { a = V(m - s, m); b = V(m - s - 1, m); }
      else { a = V(0, m - s); b = V(0, m - s - 1); }
      lb.tags.push_back(nextTag++);
      lb.nodes.push_back(a);
      lb.nodes.push_back(b);
      if (order == 2) lb.nodes.push_back(midNode(a, b));
    }
    cur.blocks.push_back(std::move(lb));
    mesh.entities.push_back(std::move(cur));
  }
  mesh.physicals["omega"] = {{2, 1}};
  mesh.physicals["gammaDir"] = {{1, 1}, {1, 2}, {1, 3}, {1, 4}};
  mesh.finalize();
  return mesh;
}

Mesh makeCubeTet(int m, int order, double jitter, uint64_t seed) {
  if (m < 1 || (order != 1 && order != 2)) throw std::invalid_argument("makeCubeTet");
  Mesh mesh;
  mesh.dim = 3;
  const double h = 1.0 / m;
  const int64_t m1 = m + 1;
  const int64_t nv = m1 * m1 * m1;
  mesh.xyz.assign(3 * nv, 0.0);
  Rng rng(seed);
  for (int k = 0; k <= m; ++k)
    for (int j = 0; j <= m; ++j)
      for (int i = 0; i <= m; ++i) {
        int64_t v = i + m1 * (j + m1 * k);
        double p[3] = {i * h, j * h, k * h};
        if (i > 0 && i < m && j > 0 && j < m && k > 0 && k < m)
          for (int c = 0; c < 3; ++c) p[c] += rng.uniform(-jitter * h, jitter * h);
        for (int c = 0; c < 3; ++c) mesh.xyz[3 * v + c] = p[c];
      }
  auto V = [&](int i, int j, int k) { return (int64_t)i + m1 * ((int64_t)j + m1 * k); };
  static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  static const bool oddPerm[6] = {false, true, true, false, false, true};
  const int tetType = order == 1 ? kTet4 : kTet10;
  std::unordered_map<std::pair<int64_t, int64_t>, int64_t, PairHash> mid;
  auto midNode = [&](int64_t a, int64_t b) -> int64_t {
    std::pair<int64_t, int64_t> key = {std::min(a, b), std::max(a, b)};
    auto it = mid.find(key);
    if (it != mid.end()) return it->second;
    int64_t id = mesh.nNodes();
    for (int c = 0; c < 3; ++c) mesh.xyz.push_back(0.5 * (mesh.xyz[3 * a + c] + mesh.xyz[3 * b + c]));
    mid.emplace(key, id);
    return id;
  };
  Entity vol;
  vol.dim = 3;
  vol.tag = 1;
  ElementBlock tb;
  tb.type = tetType;
  tb.nodesPerElement = elementNodes(tetType);
  tb.tags.reserve((size_t)6 * m * m * m);
  tb.nodes.reserve((size_t)6 * m * m * m * tb.nodesPerElement);
  int64_t nextTag = 1;
  for (int k = 0; k < m; ++k)
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i)
        for (int p = 0; p < 6; ++p) {
          int c[3] = {i, j, k};
          int64_t t[4];
          t[0] = V(c[0], c[1], c[2]);
          c[perms[p][0]]++;
          t[1] = V(c[0], c[1], c[2]);
          c[perms[p][1]]++;
          t[2] = V(c[0], c[1], c[2]);
          t[3] = V(i + 1, j + 1, k + 1);
          if (oddPerm[p]) std::swap(t[2], t[3]);  // positive orientation
          tb.tags.push_back(nextTag++);
          for (int q = 0; q < 4; ++q) tb.nodes.push_back(t[q]);
          if (order == 2)
            for (auto &ed : simplexEdges(3)) tb.nodes.push_back(midNode(t[ed[0]], t[ed[1]]));
        }
  vol.blocks.push_back(std::move(tb));
  mesh.entities.push_back(std::move(vol));
  mesh.physicals["omega"] = {{3, 1}};
  mesh.finalize();
  return mesh;
}

}  // namespace femg
