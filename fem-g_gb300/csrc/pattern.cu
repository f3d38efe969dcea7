// GPU symbolic assembly of the CSR pattern of one element bucket.
//
// Replaces MatrixFactory::addPattern (src/system/MatrixFactory.cpp:459-539)
// and finalizePattern (:188-213) for a bucket whose test and unknown DOFs
// are the same field: row I (a test DOF of assemble type Unknown, Unknown
// bubble or Unknown global) holds the sorted, unique unknown DOFs of every
// element that has I; Fixed DOFs take no column; within one element the
// bubble rows after the first alias the first one (their pattern is its).
// Linked DOFs are rows and columns of their masters; a linked bubble's
// master is a bubble row of another element, whose bubble rows then share
// one pattern with the linked element's.
//
// No global sort: per element the row counts and the bubble aliases, per row
// its list of (element, local row) entries, then a warp per row gathers the
// candidate columns of its elements into shared memory, sorts them with a
// bitonic network and keeps the first of every run, once to count and once
// to write. The result does not depend on the order of the entries, so it
// is the reference's pattern bit for bit.
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace femg {

constexpr uint32_t kPatNone = 0xFFFFFFFFu;

__device__ __forceinline__ bool patRow(uint8_t t) { return t == FG_AT_UNKNOWN || t == FG_AT_UNKNOWN_BUBBLE || t == FG_AT_UNKNOWN_GLOBAL; }

// Row counts and bubble aliases, thread per element. preAliased: the
// aliases came from the host (linked bubbles: the bubble rows of a master
// element and of the element linked to it share one list), and an element's
// first bubble entry counts on the list's row.
__global__ void k_pat_count(const uint32_t *__restrict__ edof, const uint8_t *__restrict__ etype, int64_t E, int n,
                            uint32_t *__restrict__ cnt, uint32_t *__restrict__ alias, bool preAliased) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  uint32_t first = kPatNone;
  for (int i = 0; i < n; ++i) {
    const uint8_t t = etype[e * n + i];
    if (!patRow(t)) continue;
    uint32_t I = edof[e * n + i];
    if (t == FG_AT_UNKNOWN_BUBBLE) {
      if (first != kPatNone) {
        if (!preAliased) alias[I] = first;
        continue;
      }
      first = I;
      if (preAliased && alias[I] != kPatNone) I = alias[I];
    }
    atomicAdd(&cnt[I], 1u);
  }
}

// (element, local row) entries of every row, in any order
__global__ void k_pat_fill(const uint32_t *__restrict__ edof, const uint8_t *__restrict__ etype, int64_t E, int n,
                           const uint64_t *__restrict__ rowStart, uint32_t *__restrict__ fill, uint32_t *__restrict__ rowElem,
                           const uint32_t *__restrict__ alias, bool preAliased) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  bool seenBubble = false;
  for (int i = 0; i < n; ++i) {
    const uint8_t t = etype[e * n + i];
    if (!patRow(t)) continue;
    uint32_t I = edof[e * n + i];
    if (t == FG_AT_UNKNOWN_BUBBLE) {
      if (seenBubble) continue;
      seenBubble = true;
      if (preAliased && alias[I] != kPatNone) I = alias[I];
    }
    rowElem[rowStart[I] + atomicAdd(&fill[I], 1u)] = (uint32_t)(e << 6) | (uint32_t)i;
  }
}

// Warp per row: candidate columns of the row's elements, bitonic sort in
// shared memory, unique. WRITE == false: rowLen[I] = number of columns;
// WRITE == true: the columns into aj[ai[I]...].
template <bool WRITE>
__global__ void k_pat_rows(const uint32_t *__restrict__ edof, const uint8_t *__restrict__ etype, int n,
                           const uint64_t *__restrict__ rowStart, const uint32_t *__restrict__ rowElem,
                           const uint32_t *__restrict__ alias, uint64_t nRows, int cap, int upper, uint32_t *__restrict__ rowLen,
                           const uint64_t *__restrict__ ai, uint64_t *__restrict__ aj) {
  extern __shared__ uint32_t patBuf[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t *buf = patBuf + (size_t)warp * cap;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t row = (uint64_t)blockIdx.x * (blockDim.x >> 5) + warp; row < nRows; row += warps) {
    if (alias[row] != kPatNone) continue;  // an aliased bubble row: filled from its first bubble
    const uint64_t s0 = rowStart[row];
    const int cnt = (int)(rowStart[row + 1] - s0);
    const int m = cnt * n;
    int size = 1;
    while (size < m) size <<= 1;
    for (int k = lane; k < size; k += 32) {
      uint32_t v = kPatNone;
      if (k < m) {
        const uint32_t pk = rowElem[s0 + k / n];
        const int64_t e = pk >> 6;
        const int j = k % n;
        // upper storage keeps the columns at or right of the entry's own row:
        // the row itself, or for bubbles the row of the element's first bubble
        if (patRow(etype[e * n + j]) && (!upper || edof[e * n + j] >= edof[e * n + (pk & 63)])) v = edof[e * n + j];
      }
      buf[k] = v;
    }
    __syncwarp();
    for (int blk = 2; blk <= size; blk <<= 1)
      for (int str = blk >> 1; str > 0; str >>= 1) {
        for (int t = lane; t < (size >> 1); t += 32) {
          const int i = 2 * str * (t / str) + (t % str), j = i + str;
          const bool up = (i & blk) == 0;
          const uint32_t a = buf[i], b = buf[j];
          if ((a > b) == up) {
            buf[i] = b;
            buf[j] = a;
          }
        }
        __syncwarp();
      }
    // unique values in ascending order (kPatNone sorts last)
    uint32_t count = 0;
    for (int base = 0; base < size; base += 32) {
      const int k = base + lane;
      const uint32_t v = k < size ? buf[k] : kPatNone;
      const bool keep = v != kPatNone && (k == 0 || buf[k - 1] != v);
      const unsigned mask = __ballot_sync(0xffffffffu, keep);
      if (WRITE && keep) aj[ai[row] + count + __popc(mask & ((1u << lane) - 1u))] = v;
      count += __popc(mask);
    }
    if (!WRITE && lane == 0) rowLen[row] = count;
    __syncwarp();
  }
}

__global__ void k_pat_alias_len(const uint32_t *__restrict__ alias, uint64_t nRows, uint32_t *__restrict__ rowLen) {
  const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nRows && alias[r] != kPatNone) rowLen[r] = rowLen[alias[r]];
}

__global__ void k_pat_alias_copy(const uint32_t *__restrict__ alias, uint64_t nRows, const uint64_t *__restrict__ ai,
                                 uint64_t *__restrict__ aj) {
  const uint64_t r = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= nRows || alias[r] == kPatNone) return;
  const uint64_t src = ai[alias[r]], len = ai[r + 1] - ai[r];
  for (uint64_t k = lane; k < len; k += 32) aj[ai[r] + k] = aj[src + k];
}

}  // namespace femg

using namespace femg;

namespace {

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

int devAlloc(DevBuf &b, size_t bytes) {
  if (cudaMalloc(&b.p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
    cudaGetLastError();
    setLastError("fg_pattern_build: device allocation of " + std::to_string(bytes) + " bytes failed");
    return FG_ERR_OOM;
  }
  return FG_OK;
}

}  // namespace

extern "C" int fg_pattern_build(const uint64_t *elem_dof_idx, const int32_t *elem_dof_type, int64_t n_elements, int32_t n_dofs,
                                uint64_t n_rows, uint64_t *ai, uint64_t **aj, int32_t upper, const uint64_t *linked_row,
                                uint64_t n_linked) {
  if (!ai || !aj || n_elements < 0 || n_dofs <= 0 || n_dofs > 64 || (n_elements > 0 && (!elem_dof_idx || !elem_dof_type))) {
    setLastError("fg_pattern_build: invalid arguments");
    return FG_ERR_ARG;
  }
  *aj = nullptr;
  if (n_rows >= (uint64_t(1) << 32) - 1 || n_elements >= (int64_t(1) << 26)) {
    setLastError("fg_pattern_build: more than 2^32 - 2 rows or 2^26 elements");
    return FG_ERR_UNSUPPORTED;
  }
  int dev = 0;
  if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) {
    cudaGetLastError();
    setLastError("fg_pattern_build: no CUDA device");
    return FG_ERR_NO_DEVICE;
  }
  const int n = n_dofs;
  const int64_t E = n_elements;
  const size_t en = (size_t)E * n;
  std::vector<uint32_t> ed(en);
  std::vector<uint8_t> et(en);
  int bad = 0;
  int64_t linkedBubbles = 0;
  for (size_t k = 0; k < en; ++k) {
    int t = elem_dof_type[k];
    uint64_t v = elem_dof_idx[k];
    if (t == FG_AT_LINKED || t == FG_AT_LINKED_BUBBLE) {
      // a linked DOF is a row and a column of its master (MatrixFactory.cpp:468-470, :481-483);
      // a linked bubble is a bubble row of its master's (:505)
      if (!linked_row || v >= n_linked) {
        ++bad;
        continue;
      }
      v = linked_row[v];
      if (t == FG_AT_LINKED_BUBBLE) ++linkedBubbles;
      t = t == FG_AT_LINKED ? FG_AT_UNKNOWN : FG_AT_UNKNOWN_BUBBLE;
    }
    et[k] = (uint8_t)t;
    const bool row = t == FG_AT_UNKNOWN || t == FG_AT_UNKNOWN_BUBBLE || t == FG_AT_UNKNOWN_GLOBAL;
    if (row && v >= n_rows) ++bad;
    ed[k] = row ? (uint32_t)v : 0u;
  }
  if (bad) {
    setLastError("fg_pattern_build: a DOF index is not below n_rows (or a linked index not below n_linked)");
    return FG_ERR_INDEX;
  }
  DevBuf dEd, dEt, dCnt, dAlias, dStart, dFill, dElem, dLen, dAi, dAj;
  int st;
  if ((st = devAlloc(dEd, en * 4)) || (st = devAlloc(dEt, en)) || (st = devAlloc(dCnt, n_rows * 4)) ||
      (st = devAlloc(dAlias, n_rows * 4)) || (st = devAlloc(dStart, (n_rows + 1) * 8)) || (st = devAlloc(dFill, n_rows * 4)) ||
      (st = devAlloc(dLen, n_rows * 4)) || (st = devAlloc(dAi, (n_rows + 1) * 8)))
    return st;
  uint32_t *cnt = (uint32_t *)dCnt.p, *alias = (uint32_t *)dAlias.p, *fill = (uint32_t *)dFill.p, *len = (uint32_t *)dLen.p;
  uint64_t *rowStart = (uint64_t *)dStart.p, *dai = (uint64_t *)dAi.p;
  FG_CUDA(cudaMemcpy(dEd.p, ed.data(), en * 4, cudaMemcpyHostToDevice));
  FG_CUDA(cudaMemcpy(dEt.p, et.data(), en, cudaMemcpyHostToDevice));
  FG_CUDA(cudaMemset(cnt, 0, n_rows * 4));
  FG_CUDA(cudaMemset(fill, 0, n_rows * 4));
  // With linked bubbles, the rows that share one list: the reference's
  // element after element pointer assignment (MatrixFactory.cpp:505-535)
  // puts every bubble row of a master element and of the element linked to
  // it on the list of whichever bubble row was taken first; connecting the
  // bubble rows of each element gives the same groups in any element order.
  // Each group's list is kept on its smallest row.
  const bool preAliased = linkedBubbles > 0;
  if (preAliased) {
    std::vector<uint32_t> root(n_rows);
    for (uint64_t r = 0; r < n_rows; ++r) root[r] = (uint32_t)r;
    auto find = [&](uint32_t r) {
      while (root[r] != r) r = root[r] = root[root[r]];
      return r;
    };
    for (int64_t e = 0; e < E; ++e) {
      uint32_t first = kPatNone;
      for (int i = 0; i < n; ++i) {
        const size_t k = (size_t)e * n + i;
        if (et[k] != FG_AT_UNKNOWN_BUBBLE) continue;
        if (first == kPatNone) {
          first = ed[k];
          continue;
        }
        const uint32_t a = find(first), b = find(ed[k]);
        if (a != b) root[std::max(a, b)] = std::min(a, b);
      }
    }
    std::vector<uint32_t> al(n_rows, kPatNone);
    for (uint64_t r = 0; r < n_rows; ++r)
      if (find((uint32_t)r) != r) al[r] = find((uint32_t)r);
    FG_CUDA(cudaMemcpy(alias, al.data(), n_rows * 4, cudaMemcpyHostToDevice));
  } else {
    FG_CUDA(cudaMemset(alias, 0xFF, n_rows * 4));
  }
  const unsigned eb = (unsigned)std::max<int64_t>(1, (E + 255) / 256);
  if (E > 0) {
    k_pat_count<<<eb, 256>>>((const uint32_t *)dEd.p, (const uint8_t *)dEt.p, E, n, cnt, alias, preAliased);
    countLaunch();
  }
  // row starts of the entry lists (host scan)
  std::vector<uint32_t> h32(n_rows);
  std::vector<uint64_t> h64(n_rows + 1, 0);
  FG_CUDA(cudaMemcpy(h32.data(), cnt, n_rows * 4, cudaMemcpyDeviceToHost));
  uint32_t maxCnt = 0;
  for (uint64_t r = 0; r < n_rows; ++r) {
    h64[r + 1] = h64[r] + h32[r];
    maxCnt = std::max(maxCnt, h32[r]);
  }
  FG_CUDA(cudaMemcpy(rowStart, h64.data(), (n_rows + 1) * 8, cudaMemcpyHostToDevice));
  if ((st = devAlloc(dElem, h64[n_rows] * 4))) return st;
  if (E > 0) {
    k_pat_fill<<<eb, 256>>>((const uint32_t *)dEd.p, (const uint8_t *)dEt.p, E, n, rowStart, fill, (uint32_t *)dElem.p, alias,
                            preAliased);
    countLaunch();
  }
  // shared memory per warp: the largest candidate list, rounded to a power of two
  int cap = 1;
  while ((uint64_t)cap < (uint64_t)maxCnt * n) cap <<= 1;
  int wpb = 8;
  while (wpb > 1 && (size_t)cap * 4 * wpb > 96 * 1024) wpb >>= 1;
  const size_t smem = (size_t)cap * 4 * wpb;
  if (smem > 200 * 1024) {
    setLastError("fg_pattern_build: a row gathers more candidate columns than shared memory holds");
    return FG_ERR_UNSUPPORTED;
  }
  FG_CUDA(cudaFuncSetAttribute(k_pat_rows<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  FG_CUDA(cudaFuncSetAttribute(k_pat_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned rb = (unsigned)std::min<uint64_t>(std::max<uint64_t>(1, (n_rows + wpb - 1) / wpb), (uint64_t)smCount() * 64);
  if (n_rows > 0) {
    k_pat_rows<false><<<rb, 32 * wpb, smem>>>((const uint32_t *)dEd.p, (const uint8_t *)dEt.p, n, rowStart,
                                               (const uint32_t *)dElem.p, alias, n_rows, cap, upper ? 1 : 0, len, nullptr, nullptr);
    k_pat_alias_len<<<(unsigned)((n_rows + 255) / 256), 256>>>(alias, n_rows, len);
    countLaunch(2);
    FG_CUDA(cudaGetLastError());
  }
  FG_CUDA(cudaMemcpy(h32.data(), len, n_rows * 4, cudaMemcpyDeviceToHost));
  ai[0] = 0;
  for (uint64_t r = 0; r < n_rows; ++r) ai[r + 1] = ai[r] + h32[r];
  const uint64_t nnz = ai[n_rows];
  FG_CUDA(cudaMemcpy(dai, ai, (n_rows + 1) * 8, cudaMemcpyHostToDevice));
  if ((st = devAlloc(dAj, nnz * 8))) return st;
  if (n_rows > 0) {
    k_pat_rows<true><<<rb, 32 * wpb, smem>>>((const uint32_t *)dEd.p, (const uint8_t *)dEt.p, n, rowStart,
                                              (const uint32_t *)dElem.p, alias, n_rows, cap, upper ? 1 : 0, len, dai, (uint64_t *)dAj.p);
    k_pat_alias_copy<<<(unsigned)((n_rows + 7) / 8), 256>>>(alias, n_rows, dai, (uint64_t *)dAj.p);
    countLaunch(2);
    FG_CUDA(cudaGetLastError());
  }
  void *out = nullptr;
  if (cudaMallocHost(&out, std::max<uint64_t>(nnz, 1) * 8) != cudaSuccess) {
    cudaGetLastError();
    setLastError("fg_pattern_build: host allocation failed");
    return FG_ERR_OOM;
  }
  if (cudaMemcpy(out, dAj.p, nnz * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    cudaFreeHost(out);
    setLastError("fg_pattern_build: copy of the columns failed");
    return FG_ERR_CUDA;
  }
  *aj = (uint64_t *)out;
  return FG_OK;
}
