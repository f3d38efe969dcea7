#include "dofs.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>

namespace femg {

// ---------------------------------------------------------------------------
// DofTable: robin-hood flat table slot layout (robin_hood.h 3.8.0, Table with
// MaxLoadFactor100 = 80, InitialNumElements = 8, InitialInfoNumBits = 5)
// ---------------------------------------------------------------------------

namespace {
inline uint64_t rotr64(uint64_t x, unsigned r) { return (x >> r) | (x << (64 - r)); }
// robin_hood::hash_int: the mixing applied on top of a user hash
inline uint64_t mixHash(uint64_t x) {
  const uint64_t h1 = x * 0xA24BAED4963EE407ull;
  const uint64_t h2 = rotr64(x, 32) * 0x9FB21C651E98DF25ull;
  return rotr64(h1 + h2, 32);
}
}  // namespace

DofTable::DofTable() : info_(8, 0) {}

size_t DofTable::calcMax(size_t n) const { return n <= SIZE_MAX / 100 ? n * 80 / 100 : (n / 100) * 80; }

size_t DofTable::calcWithBuffer(size_t n) const { return n + std::min(calcMax(n), (size_t)0xFF); }

void DofTable::keyToIdx(uint64_t userHash, size_t *idx, uint32_t *info) const {
  const uint64_t h = mixHash(userHash);
  *info = infoInc_ + (uint32_t)(h >> infoHashShift_);
  *idx = (size_t)h & mask_;
}

void DofTable::initData(size_t maxElements) {
  numElements_ = 0;
  mask_ = maxElements - 1;
  maxAllowed_ = calcMax(maxElements);
  const size_t nb = calcWithBuffer(maxElements);
  keys_.assign(nb, 0);
  hashes_.assign(nb, 0);
  info_.assign(nb + 8, 0);
  info_[nb] = 1;  // sentinel
  infoInc_ = 32;
  infoHashShift_ = 59;
}

void DofTable::shiftUp(size_t startIdx, size_t insertionIdx) {
  for (size_t i = startIdx; i != insertionIdx; --i) {
    keys_[i] = keys_[i - 1];
    hashes_[i] = hashes_[i - 1];
  }
  for (size_t i = startIdx; i != insertionIdx; --i) {
    info_[i] = (uint8_t)(info_[i - 1] + infoInc_);
    if (info_[i] + infoInc_ > 0xFF) maxAllowed_ = 0;
  }
}

bool DofTable::tryIncreaseInfo() {
  if (infoInc_ <= 2) return false;
  infoInc_ >>= 1;
  ++infoHashShift_;
  const size_t nb = calcWithBuffer(mask_ + 1);
  for (size_t i = 0; i < nb; i += 8)
    for (size_t b = i; b < i + 8; ++b) info_[b] = (uint8_t)(info_[b] >> 1);
  info_[nb] = 1;
  maxAllowed_ = calcMax(mask_ + 1);
  return true;
}

void DofTable::insertMove(uint32_t id, uint64_t userHash) {
  if (maxAllowed_ == 0 && !tryIncreaseInfo()) throw std::overflow_error("DofTable overflow");
  size_t idx;
  uint32_t info;
  keyToIdx(userHash, &idx, &info);
  while (info <= info_[idx]) {
    ++idx;
    info += infoInc_;
  }
  const size_t insIdx = idx;
  const uint8_t insInfo = (uint8_t)info;
  if (insInfo + infoInc_ > 0xFF) maxAllowed_ = 0;
  while (info_[idx] != 0) {
    ++idx;
    info += infoInc_;
  }
  if (idx != insIdx) shiftUp(idx, insIdx);
  keys_[insIdx] = id;
  hashes_[insIdx] = userHash;
  info_[insIdx] = insInfo;
  ++numElements_;
}

void DofTable::rehash(size_t numBuckets) {
  const size_t oldWithBuffer = calcWithBuffer(mask_ + 1);
  std::vector<uint32_t> oldKeys = std::move(keys_);
  std::vector<uint64_t> oldHashes = std::move(hashes_);
  std::vector<uint8_t> oldInfo = std::move(info_);
  const bool hadData = !oldKeys.empty();
  initData(numBuckets);
  if (hadData && oldWithBuffer > 1)
    for (size_t i = 0; i < oldWithBuffer; ++i)
      if (oldInfo[i] != 0) insertMove(oldKeys[i], oldHashes[i]);
}

void DofTable::increaseSize() {
  if (mask_ == 0 && keys_.empty()) {
    initData(8);
    return;
  }
  const size_t maxAllowed = calcMax(mask_ + 1);
  if (numElements_ < maxAllowed && tryIncreaseInfo()) return;
  if (numElements_ * 2 < calcMax(mask_ + 1)) throw std::overflow_error("DofTable: bad hash");
  rehash((mask_ + 1) * 2);
}

bool DofTable::insert(uint32_t id, const std::vector<Dof> &pool) {
  const Dof &key = pool[id];
  while (true) {
    size_t idx;
    uint32_t info;
    keyToIdx(key.hash(), &idx, &info);
    while (info < info_[idx]) {
      ++idx;
      info += infoInc_;
    }
    while (info == info_[idx]) {
      const Dof &o = pool[keys_[idx]];
      if (o.entity == key.entity && o.numType == key.numType) return false;
      ++idx;
      info += infoInc_;
    }
    if (numElements_ >= maxAllowed_) {
      increaseSize();
      continue;
    }
    const size_t insIdx = idx;
    const uint32_t insInfo = info;
    if (insInfo + infoInc_ > 0xFF) maxAllowed_ = 0;
    while (info_[idx] != 0) {
      ++idx;
      info += infoInc_;
    }
    if (idx != insIdx) shiftUp(idx, insIdx);
    keys_[insIdx] = id;
    hashes_[insIdx] = key.hash();
    info_[insIdx] = (uint8_t)insInfo;
    ++numElements_;
    return true;
  }
}

void DofTable::reserve(size_t c) {
  const size_t minAllowed = std::max(c, numElements_);
  size_t newSize = 8;
  while (calcMax(newSize) < minAllowed && newSize != 0) newSize *= 2;
  if (newSize == 0) throw std::overflow_error("DofTable reserve");
  rehash(newSize);
}

int64_t DofTable::find(uint64_t numType, uint64_t entity, const std::vector<Dof> &pool) const {
  if (keys_.empty()) return -1;
  Dof probe;
  probe.numType = numType;
  probe.entity = entity;
  size_t idx;
  uint32_t info;
  keyToIdx(probe.hash(), &idx, &info);
  do {
    if (info == info_[idx]) {
      const Dof &o = pool[keys_[idx]];
      if (o.entity == entity && o.numType == numType) return keys_[idx];
    }
    ++idx;
    info += infoInc_;
  } while (info <= info_[idx]);
  return -1;
}

std::vector<uint32_t> DofTable::order() const {
  std::vector<uint32_t> out;
  out.reserve(numElements_);
  if (keys_.empty()) return out;
  const size_t nb = calcWithBuffer(mask_ + 1);
  for (size_t i = 0; i < nb; ++i)
    if (info_[i] != 0) out.push_back(keys_[i]);
  return out;
}

bool DofDictionary::insert(const Dof &d) {
  pool.push_back(d);
  if (!table.insert((uint32_t)(pool.size() - 1), pool)) {
    pool.pop_back();
    return false;
  }
  return true;
}

const Dof *DofDictionary::find(uint64_t numType, uint64_t entity) const {
  const int64_t i = table.find(numType, entity, pool);
  return i < 0 ? nullptr : &pool[(size_t)i];
}

// ---------------------------------------------------------------------------
// Hilbert key (state machine over Gray-code sub-cells) and ordering
// ---------------------------------------------------------------------------

namespace {

struct HilbertTables {
  int dim = 0;
  int N = 0;
  uint8_t nextED[24][8];
  uint8_t code[24][8];

  explicit HilbertTables(int d) : dim(d), N(1 << d) {
    const unsigned mask = (1u << dim) - 1u;
    uint8_t gray[8], inv[8], e0[8], d0[8];
    for (int i = 0; i < N; ++i) gray[i] = (uint8_t)(i ^ (i >> 1));
    for (int i = 0; i < N; ++i) {
      unsigned v = (unsigned)i;
      for (int j = 1; j < dim; ++j) v ^= (unsigned)i >> j;
      inv[i] = (uint8_t)v;
    }
    // entry corner and axis of each sub-cell along the curve
    e0[0] = 0;
    for (int i = 1; i < N; ++i) e0[i] = gray[2 * ((i - 1) / 2)];
    d0[0] = 0;
    for (int i = 1; i < N; ++i) {
      if (i < N / 2)
        d0[i] = (uint8_t)((i % 2 == 0) ? gray[i - 1] % dim : gray[i] % dim);
      else
        d0[i] = d0[N - i - 1];
    }
    std::memset(nextED, 0, sizeof(nextED));
    std::memset(code, 0, sizeof(code));
    for (int e = 0; e < N; ++e)
      for (int a = 0; a < dim; ++a) {
        const int state = (a << dim) | e;
        for (int l = 0; l < N; ++l) {
          // rotate the corner label into the frame of (entry e, axis a)
          const unsigned k = (unsigned)(l ^ e);
          const unsigned rot = (k >> (a + 1)) | ((k << (dim - a - 1)) & mask);
          const uint8_t pos = inv[rot];
          const unsigned le = e0[pos];
          const unsigned ne = (unsigned)e ^ (((le << (a + 1)) & mask) | (le >> (dim - a - 1)));
          const unsigned na = (unsigned)(a + d0[pos] + 1) % dim;
          code[state][l] = pos;
          nextED[state][l] = (uint8_t)((na << dim) | ne);
        }
      }
  }
};

const HilbertTables &tables(int dim) {
  static const HilbertTables t2(2), t3(3);
  return dim == 2 ? t2 : t3;
}

}  // namespace

void hilbertTableData(int dim, uint8_t *code, uint8_t *next) {
  const HilbertTables &t = tables(dim);
  std::memcpy(code, t.code, sizeof(t.code));
  std::memcpy(next, t.nextED, sizeof(t.nextED));
}

uint64_t hilbertKey(int dim, const uint32_t *u) {
  const HilbertTables &t = tables(dim);
  const int begBit = (64 / dim) - 1;
  uint64_t h = 0;
  unsigned ed = 0;
  for (int m = begBit; m >= 0; --m) {
    unsigned l = 0;
    for (int n = dim - 1; n >= 0; --n) l ^= ((u[n] >> m) & 1u) << n;
    h <<= dim;
    h ^= t.code[ed][l];
    ed = t.nextED[ed][l];
  }
  return h;
}

std::vector<uint32_t> hilbertOrder(int dim, const std::vector<float> &pts, const float *mn, const float *mx) {
  const size_t n = pts.size() / dim;
  const unsigned nbrBits = 64 / dim;
  const unsigned twoPow = 1u << (nbrBits - 1);
  float scale[3], scaleMin[3];
  for (int i = 0; i < dim; ++i) {
    scale[i] = (float)twoPow / (mx[i] - mn[i]);
    scaleMin[i] = -mn[i] * scale[i];
  }
  std::vector<uint64_t> keys(n);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint32_t u[3];
    for (int j = 0; j < dim; ++j) {
      // unfused float multiply then add (the host code is built with
      // -ffp-contract=off so this does not become an fma)
      const float p = pts[(size_t)i * dim + j] * scale[j];
      u[j] = (uint32_t)(p + scaleMin[j]);
    }
    keys[(size_t)i] = hilbertKey(dim, u);
  }
  std::vector<uint32_t> perm(n);
  std::iota(perm.begin(), perm.end(), 0u);
  std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
  return perm;
}

void reorderWithHilbert(int dim, const double bbox[6], std::vector<DofDictionary *> &fields, uint64_t nUnknown, uint64_t nBubble) {
  if (nUnknown == 0) return;
  std::vector<float> pts, bpts;
  std::vector<std::pair<DofDictionary *, uint32_t>> ids, bids;
  for (DofDictionary *f : fields) {
    for (uint32_t id : f->table.order()) {
      Dof &d = f->pool[id];
      if (d.assembleType != kAtUnknown && d.assembleType != kAtUnknownBubble) continue;
      auto &P = d.assembleType == kAtUnknownBubble ? bpts : pts;
      auto &I = d.assembleType == kAtUnknownBubble ? bids : ids;
      for (int c = 0; c < dim; ++c) P.push_back(d.xyz[c]);
      I.push_back({f, id});
    }
  }
  float mn[3], mx[3];
  for (int c = 0; c < dim; ++c) {
    mn[c] = (float)(bbox[c] - 0.000001 * std::fabs(bbox[c]));
    mx[c] = (float)(bbox[3 + c] + 0.000001 * std::fabs(bbox[3 + c]));
  }
  std::vector<uint32_t> perm = hilbertOrder(dim, pts, mn, mx);
  for (size_t i = 0; i < perm.size(); ++i) ids[perm[i]].first->pool[ids[perm[i]].second].numDof = i + 1;
  std::vector<uint32_t> bperm = hilbertOrder(dim, bpts, mn, mx);
  for (size_t i = 0; i < bperm.size(); ++i)
    bids[bperm[i]].first->pool[bids[bperm[i]].second].numDof = nUnknown - nBubble + i + 1;
}

// ---------------------------------------------------------------------------
// Pattern
// ---------------------------------------------------------------------------

void PatternBuilder::init(uint64_t n) {
  nRows = n;
  rows.assign(n, {});
  alias.assign(n, -1);
}

static inline bool isRowType(int t) { return t == kAtUnknown || t == kAtUnknownGlobal || t == kAtUnknownBubble; }
static inline bool isColType(int t) { return t == kAtUnknown || t == kAtUnknownGlobal || t == kAtUnknownBubble; }

void PatternBuilder::addElements(int64_t nElements, int nTest, int nUnk, const uint64_t *testIdx, const int *testType, const uint64_t *unkIdx, const int *unkType) {
  for (int64_t e = 0; e < nElements; ++e) {
    const uint64_t *ti = testIdx + e * nTest;
    const int *tt = testType + e * nTest;
    const uint64_t *ui = unkIdx + e * nUnk;
    const int *ut = unkType + e * nUnk;
    int64_t bubble = -1;
    for (int i = 0; i < nTest; ++i) {
      if (tt[i] == kAtLinked || tt[i] == kAtLinkedBubble) throw std::runtime_error("linked DOFs are not supported");
      if (!isRowType(tt[i])) continue;
      const uint64_t I = ti[i];
      if (tt[i] == kAtUnknownBubble) {
        if (bubble >= 0) {
          alias[I] = bubble;
          continue;
        }
        bubble = (int64_t)I;
      }
      auto &row = rows[I];
      for (int j = 0; j < nUnk; ++j) {
        if (ut[j] == kAtLinked || ut[j] == kAtLinkedBubble) throw std::runtime_error("linked DOFs are not supported");
        if (!isColType(ut[j])) continue;
        if (symmetric && ui[j] < I) continue;
        row.push_back(ui[j]);
      }
    }
  }
}

void PatternBuilder::finalize(std::vector<uint64_t> &ai, std::vector<uint64_t> &aj) const {
  std::vector<std::vector<uint64_t>> sorted(nRows);
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t i = 0; i < (int64_t)nRows; ++i) {
    if (alias[(size_t)i] >= 0) continue;
    std::vector<uint64_t> r = rows[(size_t)i];
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    sorted[(size_t)i] = std::move(r);
  }
  ai.assign(nRows + 1, 0);
  for (uint64_t i = 0; i < nRows; ++i) {
    const int64_t src = alias[i] >= 0 ? alias[i] : (int64_t)i;
    ai[i + 1] = ai[i] + sorted[(size_t)src].size();
  }
  aj.resize(ai[nRows]);
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t i = 0; i < (int64_t)nRows; ++i) {
    const int64_t src = alias[(size_t)i] >= 0 ? alias[(size_t)i] : i;
    std::copy(sorted[(size_t)src].begin(), sorted[(size_t)src].end(), aj.begin() + (int64_t)ai[(size_t)i]);
  }
}

}  // namespace femg
