// DOF dictionary, DOF numbering and the CSR pattern, reproducing the
// reference's pre-processing bit for bit (given the same keys):
//
//  - the per-field dictionary is robin_hood::unordered_map<Dof*, T> (vendored
//    robin-hood 3.8.0, src/field/FieldInterface.h:112); its slot order is the
//    iteration order that feeds the Hilbert sort, so DofTable restates that
//    table's insert / reserve / rehash rules (robin_hood.h Table::doInsert,
//    insert_move, shiftUp, increase_size, try_increase_info, reserve);
//  - Dof::hash (src/dofs/Dof.h:87-92) is the user hash the table mixes;
//  - DOF creation order follows DofsFactory::generate
//    (src/dofs/DofsFactory.cpp:725-839, _generateFixedDofs :37-103,
//    _generateUnknownDofs :405-462);
//  - numbering follows DofsManager::reorderWithHilbert(true)
//    (src/dofs/DofsManager.cpp:118-241) with Hilbert<2,4>/<3,8>::apply
//    (src/reorder/Hilbert.cpp:174-288): float coordinates, 64-bit Hilbert key,
//    stable sort, bubbles numbered last;
//  - the pattern follows MatrixFactory::addPattern / finalizePattern
//    (src/system/MatrixFactory.cpp:459-539, :188-213).
#pragma once
#include <cstdint>
#include <vector>

namespace femg {

enum AssembleType : int {
  kAtUndefined = 0,
  kAtFixed = 1,
  kAtUnknown = 2,
  kAtUnknownBubble = 3,
  kAtUnknownGlobal = 4,
  kAtLinked = 5,
  kAtLinkedBubble = 6,
};

constexpr uint64_t kDofFieldOffset = 1024;  // GMSHFEM_DOF_FIELD_OFFSET default

struct Dof {
  uint64_t numType = 0;
  uint64_t entity = 0;
  uint64_t numDof = 0;  // 1-based
  float xyz[3] = {0, 0, 0};
  int assembleType = kAtUndefined;
  uint64_t hash() const {
    uint64_t seed = entity + 0x9e3779b9ull;
    seed ^= numType + 0x9e3779b9ull + (seed << 6) + (seed >> 2);
    return seed;
  }
};

// Open-addressing table with the slot layout of robin_hood's flat map; values
// are indices into DofDictionary::pool.
class DofTable {
 public:
  DofTable();
  // insert: true if new (index stored), false if an equal key exists
  bool insert(uint32_t id, const std::vector<Dof> &pool);
  void reserve(size_t c);  // always rehashes, like robin_hood's reserve
  // index of an equal key or -1
  int64_t find(uint64_t numType, uint64_t entity, const std::vector<Dof> &pool) const;
  // ids in iteration order
  std::vector<uint32_t> order() const;
  size_t size() const { return numElements_; }

 private:
  void keyToIdx(uint64_t userHash, size_t *idx, uint32_t *info) const;
  size_t calcMax(size_t n) const;
  size_t calcWithBuffer(size_t n) const;
  void initData(size_t maxElements);
  void shiftUp(size_t startIdx, size_t insertionIdx);
  bool tryIncreaseInfo();
  void increaseSize();
  void rehash(size_t numBuckets);
  void insertMove(uint32_t id, uint64_t userHash);

  std::vector<uint32_t> keys_;
  std::vector<uint64_t> hashes_;  // user hash of each occupied slot
  std::vector<uint8_t> info_;  // a zero byte when nothing is allocated
  size_t mask_ = 0;
  size_t numElements_ = 0;
  size_t maxAllowed_ = 0;
  uint32_t infoInc_ = 32;
  uint32_t infoHashShift_ = 59;
};

// One field's DOF dictionary (FieldInterface::_values)
struct DofDictionary {
  std::vector<Dof> pool;  // creation order
  DofTable table;
  bool insert(const Dof &d);  // setDof / setValue
  void reserve(size_t n) { table.reserve(n); }
  size_t size() const { return table.size(); }
  const Dof *find(uint64_t numType, uint64_t entity) const;
};

// Hilbert key of integer coordinates (dim 2: 32 levels, dim 3: 21 levels)
// the Hilbert state tables (code[state][corner], nextED[state][corner], 24 x 8)
void hilbertTableData(int dim, uint8_t *code, uint8_t *next);
uint64_t hilbertKey(int dim, const uint32_t *u);
// Hilbert order of float points (stable by key): returns the permutation
std::vector<uint32_t> hilbertOrder(int dim, const std::vector<float> &pts, const float *mn, const float *mx);

// DofsManager::reorderWithHilbert(true): renumber the unknown DOFs of the
// dictionaries (one per field), bubbles last.
void reorderWithHilbert(int dim, const double bbox[6], std::vector<DofDictionary *> &fields, uint64_t nUnknown, uint64_t nBubble);

// CSR pattern from element DOF index/type arrays (rows = test DOFs, columns =
// unknown DOFs): one block of elements with nTest x nUnk local DOFs.
struct PatternBuilder {
  uint64_t nRows = 0;
  bool symmetric = false;
  std::vector<std::vector<uint64_t>> rows;
  std::vector<int64_t> alias;  // bubble rows aliasing another row (-1 = own)
  void init(uint64_t n);
  void addElements(int64_t nElements, int nTest, int nUnk, const uint64_t *testIdx, const int *testType, const uint64_t *unkIdx, const int *unkType);
  void finalize(std::vector<uint64_t> &ai, std::vector<uint64_t> &aj) const;
};

}  // namespace femg
