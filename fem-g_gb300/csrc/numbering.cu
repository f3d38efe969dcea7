// GPU DOF numbering: DofsManager::reorderWithHilbert(true)
// (src/dofs/DofsManager.cpp:118-331) with the Hilbert sort of
// src/reorder/Hilbert.cpp:174-288.
//
// Keys: float coordinates scaled into the box exactly as the host does it,
// an unfused float multiply then add (__fmul_rn, __fadd_rn) truncated to an
// integer per axis, walked through the Hilbert state tables (2D: 32 bits
// per axis, 3D: 21). The order is the stable order of the keys; sorting the
// composite (key, input index), which is unique, with a bitonic network
// gives it exactly, whatever sort is used. Strides of 2048 and more run as
// global compare-exchange passes, the smaller ones in shared memory.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../host/dofs.h"
#include "common.cuh"

namespace femg {

constexpr int kBitonicTile = 2048;

struct HilbertDev {
  uint8_t code[24][8];
  uint8_t next[24][8];
};

__global__ void k_hilbert_keys(int dim, uint64_t n, uint64_t padded, const float *__restrict__ pts, float3 scale, float3 scaleMin,
                               const HilbertDev tab, uint64_t *__restrict__ keys, uint32_t *__restrict__ idx) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= padded) return;
  if (i >= n) {  // padding sorts after every point
    keys[i] = ~0ull;
    idx[i] = 0xFFFFFFFFu;
    return;
  }
  const float sc[3] = {scale.x, scale.y, scale.z}, sm[3] = {scaleMin.x, scaleMin.y, scaleMin.z};
  uint32_t u[3] = {0, 0, 0};
  for (int j = 0; j < dim; ++j) u[j] = __float2uint_rz(__fadd_rn(__fmul_rn(pts[i * dim + j], sc[j]), sm[j]));
  const int begBit = (64 / dim) - 1;
  uint64_t h = 0;
  unsigned ed = 0;
  for (int m = begBit; m >= 0; --m) {
    unsigned l = 0;
    for (int c = dim - 1; c >= 0; --c) l ^= ((u[c] >> m) & 1u) << c;
    h <<= dim;
    h ^= tab.code[ed][l];
    ed = tab.next[ed][l];
  }
  keys[i] = h;
  idx[i] = (uint32_t)i;
}

__device__ __forceinline__ bool pairLess(uint64_t ka, uint32_t ia, uint64_t kb, uint32_t ib) {
  return ka < kb || (ka == kb && ia < ib);
}

// one compare-exchange pass of stride j in bitonic blocks of size k
__global__ void k_bitonic_global(uint64_t *__restrict__ keys, uint32_t *__restrict__ idx, uint64_t padded, uint64_t k, uint64_t j) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= padded / 2) return;
  const uint64_t lo = 2 * j * (t / j) + (t % j), hi = lo + j;
  const bool up = (lo & k) == 0;
  const uint64_t ka = keys[lo], kb = keys[hi];
  const uint32_t ia = idx[lo], ib = idx[hi];
  if (pairLess(kb, ib, ka, ia) == up) {
    keys[lo] = kb;
    keys[hi] = ka;
    idx[lo] = ib;
    idx[hi] = ia;
  }
}

// strides jStart, jStart/2, ..., 1 of blocks of size k inside one tile (k <= tile: the whole
// sort of the tile up to k)
__global__ void __launch_bounds__(kBitonicTile / 2) k_bitonic_tile(uint64_t *__restrict__ keys, uint32_t *__restrict__ idx, uint64_t k,
                                                                  uint64_t jStart, int full) {
  __shared__ uint64_t sk[kBitonicTile];
  __shared__ uint32_t si[kBitonicTile];
  const uint64_t base = (uint64_t)blockIdx.x * kBitonicTile;
  for (int t = threadIdx.x; t < kBitonicTile; t += blockDim.x) {
    sk[t] = keys[base + t];
    si[t] = idx[base + t];
  }
  __syncthreads();
  const uint64_t kFirst = full ? 2 : k;
  for (uint64_t kk = kFirst; kk <= k; kk <<= 1) {
    for (uint64_t j = full ? kk / 2 : jStart; j > 0; j >>= 1) {
      const int t = threadIdx.x;
      const uint64_t lo = 2 * j * (t / j) + (t % j), hi = lo + j;
      const bool up = ((base + lo) & kk) == 0;
      const uint64_t ka = sk[lo], kb = sk[hi];
      const uint32_t ia = si[lo], ib = si[hi];
      if (pairLess(kb, ib, ka, ia) == up) {
        sk[lo] = kb;
        sk[hi] = ka;
        si[lo] = ib;
        si[hi] = ia;
      }
      __syncthreads();
    }
  }
  for (int t = threadIdx.x; t < kBitonicTile; t += blockDim.x) {
    keys[base + t] = sk[t];
    idx[base + t] = si[t];
  }
}

// Stable Hilbert order of n points (float [n][dim]) in the box [mn, mx].
static int hilbertOrderGpu(int dim, uint64_t n, const float *pts, const float *mn, const float *mx, uint32_t *perm) {
  if (n == 0) return FG_OK;
  uint64_t padded = kBitonicTile;
  while (padded < n) padded <<= 1;
  // scale as the host sort computes it (float)
  const unsigned nbrBits = 64 / dim;
  const unsigned twoPow = 1u << (nbrBits - 1);
  float sc[3] = {0, 0, 0}, sm[3] = {0, 0, 0};
  for (int i = 0; i < dim; ++i) {
    sc[i] = (float)twoPow / (mx[i] - mn[i]);
    sm[i] = -mn[i] * sc[i];
  }
  HilbertDev tab;
  hilbertTableData(dim, &tab.code[0][0], &tab.next[0][0]);
  float *dPts = nullptr;
  uint64_t *keys = nullptr;
  uint32_t *idx = nullptr;
  auto release = [&]() {
    cudaFree(dPts);
    cudaFree(keys);
    cudaFree(idx);
  };
  if (cudaMalloc(&dPts, n * dim * sizeof(float)) != cudaSuccess || cudaMalloc(&keys, padded * 8) != cudaSuccess ||
      cudaMalloc(&idx, padded * 4) != cudaSuccess) {
    cudaGetLastError();
    release();
    setLastError("hilbert order: device allocation failed");
    return FG_ERR_OOM;
  }
  int st = FG_OK;
  do {
    if (cudaMemcpy(dPts, pts, n * dim * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) break;
    k_hilbert_keys<<<(unsigned)((padded + 255) / 256), 256>>>(dim, n, padded, dPts, make_float3(sc[0], sc[1], sc[2]),
                                                              make_float3(sm[0], sm[1], sm[2]), tab, keys, idx);
    const unsigned tiles = (unsigned)(padded / kBitonicTile);
    k_bitonic_tile<<<tiles, kBitonicTile / 2>>>(keys, idx, kBitonicTile, 0, 1);  // every tile sorted in alternating directions
    int launches = 2;
    for (uint64_t k = 2 * kBitonicTile; k <= padded; k <<= 1) {
      for (uint64_t j = k / 2; j >= kBitonicTile; j >>= 1) {
        k_bitonic_global<<<(unsigned)((padded / 2 + 255) / 256), 256>>>(keys, idx, padded, k, j);
        ++launches;
      }
      k_bitonic_tile<<<tiles, kBitonicTile / 2>>>(keys, idx, k, kBitonicTile / 2, 0);
      ++launches;
    }
    countLaunch(launches);
    if (cudaGetLastError() != cudaSuccess) break;
    if (cudaMemcpy(perm, idx, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) break;
    st = FG_OK;
    release();
    return st;
  } while (false);
  const cudaError_t e = cudaGetLastError();
  release();
  setLastError(std::string("hilbert order: ") + cudaGetErrorString(e));
  return FG_ERR_CUDA;
}

}  // namespace femg

using namespace femg;

extern "C" int fg_hilbert_order(int32_t dim, uint64_t n, const float *pts, const float *mn, const float *mx, uint32_t *perm) {
  if ((dim != 2 && dim != 3) || (n > 0 && (!pts || !mn || !mx || !perm)) || n >= (uint64_t(1) << 32) - 1) {
    setLastError("fg_hilbert_order: invalid arguments");
    return FG_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) {
    cudaGetLastError();
    setLastError("fg_hilbert_order: no CUDA device");
    return FG_ERR_NO_DEVICE;
  }
  return hilbertOrderGpu(dim, n, pts, mn, mx, perm);
}

extern "C" int fg_hilbert_numbering(int32_t dim, const double *bbox, uint64_t n_dofs, const float *xyz, const int32_t *assemble_type,
                                    uint64_t *num_dof) {
  if ((dim != 2 && dim != 3) || !bbox || (n_dofs > 0 && (!xyz || !assemble_type || !num_dof))) {
    setLastError("fg_hilbert_numbering: invalid arguments");
    return FG_ERR_ARG;
  }
  std::vector<float> pts, bpts;
  std::vector<uint64_t> ids, bids;
  for (uint64_t i = 0; i < n_dofs; ++i) {
    const int t = assemble_type[i];
    if (t != FG_AT_UNKNOWN && t != FG_AT_UNKNOWN_BUBBLE) continue;
    auto &P = t == FG_AT_UNKNOWN_BUBBLE ? bpts : pts;
    (t == FG_AT_UNKNOWN_BUBBLE ? bids : ids).push_back(i);
    for (int c = 0; c < dim; ++c) P.push_back(xyz[3 * i + c]);
  }
  const uint64_t nUnknown = ids.size() + bids.size(), nBubble = bids.size();
  if (nUnknown == 0) return FG_OK;
  // the box widened by a relative 1e-6, as the reference does (DofsManager.cpp)
  float mn[3], mx[3];
  for (int c = 0; c < dim; ++c) {
    mn[c] = (float)(bbox[c] - 0.000001 * std::fabs(bbox[c]));
    mx[c] = (float)(bbox[3 + c] + 0.000001 * std::fabs(bbox[3 + c]));
  }
  std::vector<uint32_t> perm(ids.size()), bperm(bids.size());
  int st = fg_hilbert_order(dim, ids.size(), pts.data(), mn, mx, perm.data());
  if (st) return st;
  if ((st = fg_hilbert_order(dim, bids.size(), bpts.data(), mn, mx, bperm.data()))) return st;
  for (size_t i = 0; i < perm.size(); ++i) num_dof[ids[perm[i]]] = i + 1;
  for (size_t i = 0; i < bperm.size(); ++i) num_dof[bids[bperm[i]]] = nUnknown - nBubble + i + 1;
  return FG_OK;
}
