// K4 + K5: deterministic row-owner reduction of element matrices and vectors
// into the CSR values and the right-hand side.
//
// Replaces MatrixFactory::addValues (src/system/MatrixFactory.cpp:233-448:
// lower_bound per entry + OpenMP atomics) and VectorFactory::addValues /
// addValuesDC (src/system/VectorFactory.cpp:122-210). Each CSR row is owned
// by a sub-warp of L lanes (L * 3 >= element DOFs, so 32/L rows share a warp);
// the sub-warp walks the row's (element, local test index) list in element
// order, and every lane adds its columns of that element row into a shared
// accumulator at the slots precomputed by fg_plan_create. Entries are
// separated by __syncwarp, so each CSR value is summed in the same order on
// every run. Rows are visited sorted by their number of contributing
// elements, so the sub-warps of a warp run loops of equal length.
// Dirichlet lifting reads the transposed element entry, as addValuesDC does
// (values[j*n + i] * valuesDC[J], src/system/VectorFactory.cpp:184).
#include "common.cuh"

namespace femg {

// The rows of one plan handled by block `blk` of `nblk` (grid-stride over row
// groups of rowsPerBlock rows).
template <typename SlotT, bool KCPLX, typename KT, typename AT, int L, int J, bool ACC>
__device__ __forceinline__ void gatherRows(const PlanDev &p, const KT *__restrict__ ke, const double2 *__restrict__ be,
                                           const double2 *__restrict__ uD, double2 *__restrict__ values,
                                           double2 *__restrict__ rhs, int rowsPerBlock, KeLayout lay, int64_t blk, int64_t nblk,
                                           int64_t v0, int64_t v1) {
  constexpr int R = 32 / L;  // rows per warp; J: columns per lane (L * J >= n)
  constexpr int SS = KCPLX ? 2 : 1;
  // offset of entry (test ii, unknown jj) inside one component of an element
  // matrix in the layout lay (compound blocks: ii = i*3 + a, jj = j*3 + b)
  auto keOff = [&](int ii, int jj) -> int { return keOffset(lay, p.nc, ii, jj); };
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / L, lt = lane % L;
  AT *A = reinterpret_cast<AT *>(smraw) + (size_t)(warp * R + sub) * p.maxRowLen * SS;
  const SlotT *slot = (const SlotT *)p.slot;
  const SlotT kFixed = (SlotT)(sizeof(SlotT) == 1 ? 0xFF : kSlotFixed);
  const SlotT kIgnore = (SlotT)(sizeof(SlotT) == 1 ? 0xFE : kSlotIgnore);
  const int n = p.n, nc = p.nc;  // element rows (test DOFs), columns (unknown DOFs)
  const size_t nn2 = (size_t)lay.ld;  // entries per component
  // visit records [v0, v1) of this launch
  const int64_t nRows = v1;
  const int64_t stride = nblk * rowsPerBlock;
  const int64_t first = v0 + blk * rowsPerBlock + warp * R + sub;
  uint4 vNext = first < nRows ? p.visit[first] : make_uint4(0, 0, 0, 0);
  for (int64_t base = v0 + blk * rowsPerBlock + warp * R; base < nRows; base += stride) {
    const int64_t idx = base + sub;
    const bool live = idx < nRows;
    const uint4 v = vNext;  // this row's record, fetched one iteration ahead
    vNext = (idx + stride < nRows) ? p.visit[idx + stride] : make_uint4(0, 0, 0, 0);
    const int64_t row = v.x;
    const uint64_t start = v.y;
    const int len = live ? (int)(v.w & 0xFFFFu) : 0;
    const uint64_t r0 = v.z;
    const int cnt = live ? (int)(v.w >> 16) : 0;
    // the row's (element, local index) list, L entries at a time in the lanes
    uint32_t myPacked = (lt < cnt) ? p.visitElem[r0 + lt] : 0u;
    for (int s = lt; s < len * SS; s += L) A[s] = (AT)0;
    int maxCnt = cnt;
#pragma unroll
    for (int off = L; off < 32; off <<= 1) maxCnt = max(maxCnt, __shfl_xor_sync(0xffffffffu, maxCnt, off));
    __syncwarp();
    double2 dc = make_double2(0.0, 0.0), bsum = make_double2(0.0, 0.0);
    // software pipeline: entry k+1's slots and values are in flight while
    // entry k is added
    SlotT sv[J], svN[J];
    KT vr[J], vi[J], vrN[J], viN[J];
    uint32_t flat = 0, flatN = 0;
    auto fetch = [&](int k, uint32_t packed, SlotT *s_, KT *r_, KT *i_, uint32_t &f_) {
      const bool act = k < cnt;
      const uint32_t e32 = packed >> 6;
      const int i = packed & 63;
      f_ = e32 * (uint32_t)n + (uint32_t)i;  // element row index (< 2^32 by plan checks)
      const SlotT *S = slot + (size_t)f_ * p.slotLd;
      const KT *K = ke + (size_t)e32 * SS * nn2;
#pragma unroll
      for (int jj = 0; jj < J; ++jj) {
        const int j = lt + L * jj;
        const bool ok = act && j < nc;
        const int o = keOff(i, j);
        s_[jj] = ok ? S[j] : kIgnore;
        r_[jj] = ok ? K[o] : (KT)0;
        i_[jj] = (ok && KCPLX) ? K[nn2 + o] : (KT)0;
      }
    };
    if (maxCnt > 0) fetch(0, __shfl_sync(0xffffffffu, myPacked, sub * L, 32), sv, vr, vi, flat);
    for (int k = 0; k < maxCnt; ++k) {
      const uint32_t packedK = __shfl_sync(0xffffffffu, myPacked, sub * L + (k % L), 32);
      if (k + 1 < maxCnt) {
        if ((k + 1) % L == 0) myPacked = (k + 1 + lt < cnt) ? p.visitElem[r0 + k + 1 + lt] : 0u;
        fetch(k + 1, __shfl_sync(0xffffffffu, myPacked, sub * L + ((k + 1) % L), 32), svN, vrN, viN, flatN);
      }
      const bool act = k < cnt;
      const int64_t e = packedK >> 6;
      const int i = packedK & 63;
      // linked DOFs (complex element matrices only): the row scales by the
      // conjugate of its coefficient, each column by its own
      const bool linked = KCPLX && p.lscale != nullptr;
      double2 cI = make_double2(1.0, 0.0);
      if (linked && act) {
        cI = p.lscale[e * n + i];
        cI.y = -cI.y;
      }
      if (be && act && lt == 0) bsum = cadd(bsum, linked ? cmul(cI, be[flat]) : be[flat]);
#pragma unroll
      for (int jj = 0; jj < J; ++jj) {
        const SlotT s = sv[jj];
        if (s == kIgnore) continue;
        if (s != kFixed) {
          AT ar = (AT)vr[jj], ai = KCPLX ? (AT)vi[jj] : (AT)0;
          if (linked) {
            const double2 c = cmul(cI, p.lscale[e * n + lt + L * jj]);
            const AT tr = ar * (AT)c.x - ai * (AT)c.y;
            ai = ar * (AT)c.y + ai * (AT)c.x;
            ar = tr;
          }
          // the lanes of one element row hit distinct slots; entries are
          // ordered by the __syncwarp below, so these adds are ordered too
          atomicAdd(&A[(int)s * SS], ar);
          if (KCPLX) atomicAdd(&A[(int)s * SS + 1], ai);
        } else {
          // (a two-field plan with fixed columns has as many columns as rows)
          const KT *Kt = ke + (size_t)e * SS * nn2;
          const int j = lt + L * jj;
          const int o = keOff(j, i);
          double2 v = make_double2((double)Kt[o], KCPLX ? (double)Kt[nn2 + o] : 0.0);
          if (linked) v = cmul(cI, v);
          dc = cadd(dc, cmul(v, uD[p.edofU[e * nc + j]]));
        }
      }
      __syncwarp();
#pragma unroll
      for (int jj = 0; jj < J; ++jj) {
        sv[jj] = svN[jj];
        vr[jj] = vrN[jj];
        vi[jj] = viN[jj];
      }
      flat = flatN;
    }
    // ACC: add into the values (several buckets sharing rows) instead of overwriting them
    for (int s = lt; s < len; s += L) {
      double2 v = make_double2(widen(A[s * SS]), KCPLX ? widen(A[s * SS + 1]) : 0.0);
      if (ACC) v = cadd(values[start + s], v);
      values[start + s] = v;
    }
    if (rhs) {
      if (uD) {  // Dirichlet lifting present: reduce the lanes' lifted terms
#pragma unroll
        for (int off = L / 2; off > 0; off >>= 1) {
          dc.x += __shfl_down_sync(0xffffffffu, dc.x, off, L);
          dc.y += __shfl_down_sync(0xffffffffu, dc.y, off, L);
        }
        if (live && lt == 0) rhs[row] = ACC ? cadd(rhs[row], cadd(bsum, dc)) : cadd(bsum, dc);
      } else if (live && lt == 0) {
        rhs[row] = ACC ? cadd(rhs[row], bsum) : bsum;
      }
    }
    __syncwarp();
  }
}

// Real FP32 element matrices in full row-major layout with n a multiple of 4
// and one-byte slots (the scalar tetrahedral orders 1 and 3): a sub-warp of
// L = n / 4 lanes per row, lane lt owning columns 4 lt .. 4 lt + 3, so that
// an element row comes in with one 16-byte load per lane and its slots with
// one 4-byte load (against 2 n / L scalar loads per lane in k_gather). Same
// visiting order, same per-entry order (entries separated by __syncwarp),
// same results. The next row's visit record is loaded while the current row
// runs, and a row's list entries L at a time, one per lane, so that the loads
// of an element row depend on a shuffle instead of a list load.
// The rows of visit records [v0, v1) handled by block blk of nblk.
template <bool ACC>
__device__ __forceinline__ void gatherRowsV4(const PlanDev &p, const float *__restrict__ ke, const double2 *__restrict__ be,
                                             const double2 *__restrict__ uD, double2 *__restrict__ values,
                                             double2 *__restrict__ rhs, int L, int64_t blk, int64_t nblk, int64_t v0, int64_t v1) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int R = 32 / L;  // rows per warp
  const int sub = lane / L, lt = lane - sub * L;
  const bool laneLive = sub < R;
  float *A = reinterpret_cast<float *>(smraw) + (size_t)(warp * R + (laneLive ? sub : 0)) * p.maxRowLen;
  const int n = p.n, nn2 = n * n;
  const uint8_t *slot = (const uint8_t *)p.slot;
  const int64_t stride = nblk * wpb * R;
  const int64_t first = v0 + (blk * wpb + warp) * R + sub;
  uint4 vNext = (laneLive && first < v1) ? p.visit[first] : make_uint4(0, 0, 0, 0);
  for (int64_t base = v0 + (blk * wpb + warp) * R; base < v1; base += stride) {
    const int64_t idx = base + sub;
    const bool live = laneLive && idx < v1;
    const uint4 v = vNext;  // this row's record, fetched one row ahead
    vNext = (laneLive && idx + stride < v1) ? p.visit[idx + stride] : make_uint4(0, 0, 0, 0);
    const int len = live ? (int)(v.w & 0xFFFFu) : 0;
    const int cnt = live ? (int)(v.w >> 16) : 0;
    // the row's (element, local row) list, L entries at a time in the lanes
    uint32_t myPacked = (lt < cnt) ? p.visitElem[v.z + lt] : 0u;
    for (int s = lt; s < len; s += L) A[s] = 0.0f;
    int maxCnt = cnt;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) maxCnt = max(maxCnt, __shfl_xor_sync(0xffffffffu, maxCnt, off));
    __syncwarp();
    double2 dc = make_double2(0.0, 0.0), bsum = make_double2(0.0, 0.0);
    float4 kv, kvN;
    uint32_t sv, svN, flat = 0, flatN = 0;
    const int srcBase = laneLive ? sub * L : 0;
    auto fetch = [&](int k, uint32_t packed, float4 &kv_, uint32_t &sv_, uint32_t &f_) {
      if (k < cnt) {
        const uint32_t e = packed >> 6, i = packed & 63;
        f_ = e * (uint32_t)n + i;
        kv_ = *reinterpret_cast<const float4 *>(ke + (size_t)e * nn2 + (size_t)i * n + 4 * lt);
        sv_ = *reinterpret_cast<const uint32_t *>(slot + (size_t)f_ * p.slotLd + 4 * lt);
      } else {
        kv_ = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        sv_ = 0xFEFEFEFEu;  // ignore
        f_ = 0;
      }
    };
    if (maxCnt > 0) fetch(0, __shfl_sync(0xffffffffu, myPacked, srcBase), kv, sv, flat);
    for (int k = 0; k < maxCnt; ++k) {
      if (k + 1 < maxCnt) {
        if ((k + 1) % L == 0) myPacked = (k + 1 + lt < cnt) ? p.visitElem[v.z + k + 1 + lt] : 0u;
        fetch(k + 1, __shfl_sync(0xffffffffu, myPacked, srcBase + (k + 1) % L), kvN, svN, flatN);
      }
      const float vals[4] = {kv.x, kv.y, kv.z, kv.w};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const uint32_t s = (sv >> (8 * c)) & 0xFFu;
        if (s < 0xFEu) {
          // an element row's columns sit in distinct slots unless the plan
          // says otherwise; successive element rows are ordered by __syncwarp
          if (p.plainSlots) A[s] += vals[c];
          else atomicAdd(&A[s], vals[c]);
        } else if (s == 0xFFu) {
          // Dirichlet lifting with the transposed entry (addValuesDC, VectorFactory.cpp:184)
          const uint32_t e = flat / (uint32_t)n, i = flat - e * (uint32_t)n;
          const int j = 4 * lt + c;
          const double kt = (double)ke[(size_t)e * nn2 + (size_t)j * n + i];
          const double2 u = uD[p.edofU[(size_t)e * n + j]];
          dc.x += kt * u.x;
          dc.y += kt * u.y;
        }
      }
      if (be && lt == 0 && k < cnt) bsum = cadd(bsum, be[flat]);
      __syncwarp();
      kv = kvN;
      sv = svN;
      flat = flatN;
    }
    for (int s = lt; s < len; s += L) {
      double2 val = make_double2(widen(A[s]), 0.0);
      if (ACC) val = cadd(values[v.y + s], val);
      values[v.y + s] = val;
    }
    if (rhs) {
      double2 dtot = dc;
      if (uD)  // the sub-warp's lifted terms, summed on its first lane
        for (int t = 1; t < L; ++t) {
          const int src = sub * L + t < 32 ? sub * L + t : lane;
          dtot.x += __shfl_sync(0xffffffffu, dc.x, src);
          dtot.y += __shfl_sync(0xffffffffu, dc.y, src);
        }
      if (live && lt == 0) {
        const double2 tot = cadd(bsum, dtot);
        rhs[v.x] = ACC ? cadd(rhs[v.x], tot) : tot;
      }
    }
    __syncwarp();
  }
}

template <bool ACC>
__global__ void __launch_bounds__(256)
    k_gather_v4(const PlanDev p, const float *__restrict__ ke, const double2 *__restrict__ be, const double2 *__restrict__ uD,
                double2 *__restrict__ values, double2 *__restrict__ rhs, int L, int64_t v0, int64_t v1) {
  gatherRowsV4<ACC>(p, ke, be, uD, values, rhs, L, blockIdx.x, gridDim.x, v0, v1);
}

// Many plans of one class in one launch (k_gather_batch with the vector loads)
__global__ void __launch_bounds__(256) k_gather_batch_v4(const GatherJob *__restrict__ jobs, int nJobs, int L) {
  int lo = 0, hi = nJobs - 1;
  while (lo < hi) {  // last job whose blockStart <= blockIdx.x
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].blockStart <= (int64_t)blockIdx.x) lo = mid;
    else hi = mid - 1;
  }
  const GatherJob &Jb = jobs[lo];
  gatherRowsV4<false>(Jb.p, (const float *)Jb.ke, Jb.be, Jb.uD, Jb.values, Jb.rhs, L, (int64_t)blockIdx.x - Jb.blockStart,
                      Jb.nBlocks, 0, (int64_t)Jb.p.nRows);
}

template <typename SlotT, bool KCPLX, typename KT, typename AT, int L, int J, bool ACC>
__global__ void __launch_bounds__(256)
    k_gather(const PlanDev p, const KT *__restrict__ ke, const double2 *__restrict__ be, const double2 *__restrict__ uD,
             double2 *__restrict__ values, double2 *__restrict__ rhs, int rowsPerBlock, KeLayout lay, int64_t v0, int64_t v1) {
  gatherRows<SlotT, KCPLX, KT, AT, L, J, ACC>(p, ke, be, uD, values, rhs, rowsPerBlock, lay, blockIdx.x, gridDim.x, v0, v1);
}

// Many plans in one launch: job q owns blocks [blockStart, blockStart + nBlocks)
template <typename SlotT, bool KCPLX, typename KT, typename AT, int L, int J>
__global__ void __launch_bounds__(256) k_gather_batch(const GatherJob *__restrict__ jobs, int nJobs, int rowsPerBlock) {
  int lo = 0, hi = nJobs - 1;
  while (lo < hi) {  // last job whose blockStart <= blockIdx.x
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].blockStart <= (int64_t)blockIdx.x) lo = mid;
    else hi = mid - 1;
  }
  const GatherJob &Jb = jobs[lo];
  gatherRows<SlotT, KCPLX, KT, AT, L, J, false>(Jb.p, (const KT *)Jb.ke, Jb.be, Jb.uD, Jb.values, Jb.rhs, rowsPerBlock, Jb.lay,
                                         (int64_t)blockIdx.x - Jb.blockStart, Jb.nBlocks, 0, (int64_t)Jb.p.nRows);
}

// k_gather_v4 where it applies: real FP32 element matrices in full layout,
// n a multiple of 4 (at most 32 columns), one-byte slots, no linked DOFs
static bool gatherV4Applies(const PlanDev &p, int keComplex, int keIsFloat, KeLayout lay) {
  return keIsFloat && !keComplex && lay.kind == kKeFull && p.n % 4 == 0 && p.n <= 32 && p.slotBytes == 1 && !p.lscale &&
         !p.coupled;
}

static int launchV4(const PlanDev &p, const float *ke, const double2 *be, const double2 *uD, double2 *values, double2 *rhs,
                    int64_t v0, int64_t v1, bool acc, cudaStream_t s) {
  const int L = p.n / 4, R = 32 / L;
  int wpb = 8;
  const size_t rowBytes = (size_t)std::max(p.maxRowLen, 1) * 4;
  while (wpb > 1 && rowBytes * R * wpb > 200 * 1024) wpb >>= 1;
  const size_t smem = rowBytes * R * wpb;
  if (smem > 200 * 1024) {
    setLastError("gather: CSR row too long for shared memory");
    return FG_ERR_UNSUPPORTED;
  }
  int64_t blocks = (v1 - v0 + (int64_t)wpb * R - 1) / ((int64_t)wpb * R);
  blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)smCount() * 16));
  if (acc) {
    static SmemAllowance allowed;
    FG_CUDA(allowSmem(k_gather_v4<true>, smem, allowed));
    k_gather_v4<true><<<(unsigned)blocks, 32 * wpb, smem, s>>>(p, ke, be, uD, values, rhs, L, v0, v1);
  } else {
    static SmemAllowance allowed;
    FG_CUDA(allowSmem(k_gather_v4<false>, smem, allowed));
    k_gather_v4<false><<<(unsigned)blocks, 32 * wpb, smem, s>>>(p, ke, be, uD, values, rhs, L, v0, v1);
  }
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

template <typename SlotT, bool KCPLX, typename KT>
static int launchTyped(const PlanDev &p, const void *ke, const double2 *be, const double2 *uD, double2 *values, double2 *rhs,
                       KeLayout lay, int64_t v0, int64_t v1, bool acc, cudaStream_t s) {
  using AT = KT;  // FP32 element matrices accumulate in FP32, FP64 ones in FP64
  const GatherShape shape = gatherShape(p.nc, p.maxRowLen, KCPLX ? 1 : 0, sizeof(KT) == 4 ? 1 : 0, 0, 0);
  const int L = shape.L, J = shape.J;
  const int R = 32 / L;
  const size_t rowBytes = (size_t)std::max(p.maxRowLen, 1) * (KCPLX ? 2 : 1) * sizeof(AT);
  int wpb = 8;
  while (wpb > 1 && rowBytes * R * wpb > 200 * 1024) wpb >>= 1;
  if (rowBytes * R * wpb > 200 * 1024) {
    setLastError("gather: CSR row too long for shared memory");
    return FG_ERR_UNSUPPORTED;
  }
  const size_t smem = rowBytes * R * wpb;
  const int rowsPerBlock = wpb * R;
  const int sms = smCount();
  int64_t blocks = (v1 - v0 + rowsPerBlock - 1) / rowsPerBlock;
  blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)sms * 16));
  bool launched = false;
#define FG_GATHER_K(LL, JJ, AA)                                                                                   \
  {                                                                                                               \
    auto kern = k_gather<SlotT, KCPLX, KT, AT, LL, JJ, AA>;                                                       \
    static SmemAllowance allowed;                                                                                \
    FG_CUDA(allowSmem(kern, smem, allowed));                                                                      \
    kern<<<(unsigned)blocks, 32 * wpb, smem, s>>>(p, (const KT *)ke, be, uD, values, rhs, rowsPerBlock, lay, v0, v1); \
  }
#define FG_GATHER_L(LL, JJ)                                                                                       \
  if (L == LL && J == JJ) {                                                                                       \
    launched = true;                                                                                              \
    if (acc) FG_GATHER_K(LL, JJ, true) else FG_GATHER_K(LL, JJ, false)                                            \
  }
  FG_GATHER_L(2, 3)
  FG_GATHER_L(4, 3)
  FG_GATHER_L(8, 3)
  FG_GATHER_L(8, 5)
  FG_GATHER_L(16, 3)
  FG_GATHER_L(32, 3)
#undef FG_GATHER_L
#undef FG_GATHER_K
  if (!launched) {
    setLastError("gather: no kernel for this (lanes, columns) shape");
    return FG_ERR_UNSUPPORTED;
  }
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

// The rows of visit records [v0, v1) (all rows: 0, nRows).
static int launchGatherRange(const PlanDev &p, const double *ke, int keComplex, int keIsFloat, KeLayout lay, const double *be,
                             const double *dirichletDev, double *values, double *rhs, int64_t v0, int64_t v1, bool acc,
                             cudaStream_t s) {
  if (v1 <= v0) return FG_OK;
  if (p.lscale && !keComplex) {
    setLastError("gather: linked DOFs need complex element matrices");
    return FG_ERR_UNSUPPORTED;
  }
  const double2 *be2 = (const double2 *)be;
  const double2 *uD = (const double2 *)dirichletDev;
  double2 *v2 = (double2 *)values;
  double2 *r2 = (double2 *)rhs;
  if (gatherV4Applies(p, keComplex, keIsFloat, lay)) {
    ProfScope prof("k_gather_v4", s);
    countLaunch();
    return launchV4(p, (const float *)ke, be2, uD, v2, r2, v0, v1, acc, s);
  }
  ProfScope prof("k_gather", s);
  countLaunch();
  if (p.slotBytes == 1) {
    if (keIsFloat)
      return keComplex ? launchTyped<uint8_t, true, float>(p, ke, be2, uD, v2, r2, lay, v0, v1, acc, s) : launchTyped<uint8_t, false, float>(p, ke, be2, uD, v2, r2, lay, v0, v1, acc, s);
    return keComplex ? launchTyped<uint8_t, true, double>(p, ke, be2, uD, v2, r2, lay, v0, v1, acc, s) : launchTyped<uint8_t, false, double>(p, ke, be2, uD, v2, r2, lay, v0, v1, acc, s);
  }
  if (keIsFloat)
    return keComplex ? launchTyped<uint16_t, true, float>(p, ke, be2, uD, v2, r2, lay, v0, v1, acc, s) : launchTyped<uint16_t, false, float>(p, ke, be2, uD, v2, r2, lay, v0, v1, acc, s);
  return keComplex ? launchTyped<uint16_t, true, double>(p, ke, be2, uD, v2, r2, lay, v0, v1, acc, s) : launchTyped<uint16_t, false, double>(p, ke, be2, uD, v2, r2, lay, v0, v1, acc, s);
}

int launchGather(fg_plan *plan, const double *ke, int keComplex, int keIsFloat, KeLayout lay, const double *be,
                 const double *dirichletDev, double *values, double *rhs, cudaStream_t s) {
  return launchGatherRange(plan->d, ke, keComplex, keIsFloat, lay, be, dirichletDev, values, rhs, 0, (int64_t)plan->d.nRows,
                           plan->accumulate != 0, s);
}

// Host values: the reduction runs range by range; after each range an event
// lets the copy stream bring that range's CSR slice to the host while the
// next range reduces (the copy, not the reduction, bounds a host-output call).
int gatherToOutputs(fg_plan *plan, const double *ke, int keComplex, int keIsFloat, KeLayout lay, const double *be,
                    const double *dirichletDev, Outputs &o, double *csr_values, cudaStream_t s) {
  const size_t nc = plan->outChunkRow.size() > 1 ? plan->outChunkRow.size() - 1 : 0;
  if (!o.hostValues || nc < 2)
    return launchGather(plan, ke, keComplex, keIsFloat, lay, be, dirichletDev, o.values, o.rhs, s);
  if (!plan->copyStream) {
    FG_CUDA(cudaStreamCreateWithFlags(&plan->copyStream, cudaStreamNonBlocking));
    plan->copyEvents.assign(nc, nullptr);
    for (auto &ev : plan->copyEvents) FG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  PlanDev pr = plan->d;  // the range-major visiting order
  pr.visit = plan->visitRanged;
  pr.visitElem = plan->visitElemRanged;
  for (size_t c = 0; c < nc; ++c) {
    const uint64_t r0 = plan->outChunkRow[c], r1 = plan->outChunkRow[c + 1];
    int st = launchGatherRange(pr, ke, keComplex, keIsFloat, lay, be, dirichletDev, o.values, o.rhs, (int64_t)r0, (int64_t)r1, false, s);
    if (st) return st;
    FG_CUDA(cudaEventRecord(plan->copyEvents[c], s));
    FG_CUDA(cudaStreamWaitEvent(plan->copyStream, plan->copyEvents[c], 0));
    const uint64_t a0 = plan->hAi[r0], a1 = plan->hAi[r1];
    if (a1 > a0)
      FG_CUDA(cudaMemcpyAsync(csr_values + 2 * a0, o.values + 2 * a0, (a1 - a0) * 16, cudaMemcpyDeviceToHost, plan->copyStream));
  }
  o.valuesCopied = true;
  return FG_OK;
}

// Shared memory and rows per block of one gather configuration
// Lanes per row and columns per lane: (2, 3), (4, 3), (8, 3), (8, 5),
// (16, 3) or (32, 3). By default the narrowest that covers n (8 x 5 for
// 25..40 columns measured 7% faster than 16 x 3 on order-4 tets); for a given
// L, J = 3 when 3L covers n, else 5 (L = 8 only).
GatherShape gatherShapeV4(int n, int maxRowLen, int wpb) {
  GatherShape g;
  g.v4 = true;
  g.L = n / 4;
  g.J = 4;
  const int R = 32 / g.L;
  const size_t rowBytes = (size_t)std::max(maxRowLen, 1) * 4;
  if (wpb <= 0) {
    wpb = 8;
    while (wpb > 1 && rowBytes * R * wpb > 200 * 1024) wpb >>= 1;
  }
  g.wpb = wpb;
  g.rowsPerBlock = wpb * R;
  g.smem = rowBytes * R * wpb;
  g.ok = n % 4 == 0 && n <= 32 && g.smem <= 200 * 1024;
  return g;
}

GatherShape gatherShape(int n, int maxRowLen, int kcplx, int keIsFloat, int L, int wpb) {
  GatherShape g;
  if (L <= 0) {
    L = 32;
    if (n <= 6) L = 2;
    else if (n <= 12) L = 4;
    else if (n <= 40) L = 8;
    else if (n <= 48) L = 16;
  }
  g.J = 3 * L >= n ? 3 : 5;
  const int R = 32 / L;
  const size_t rowBytes = (size_t)std::max(maxRowLen, 1) * (kcplx ? 2 : 1) * (keIsFloat ? 4 : 8);
  if (wpb <= 0) {
    wpb = 8;
    while (wpb > 1 && rowBytes * R * wpb > 200 * 1024) wpb >>= 1;
  }
  g.L = L;
  g.wpb = wpb;
  g.rowsPerBlock = wpb * R;
  g.smem = rowBytes * R * wpb;
  g.ok = g.smem <= 200 * 1024 && g.J * L >= n && (g.J == 3 || L == 8);
  return g;
}

template <typename SlotT, bool KCPLX, typename KT>
static int launchBatchTyped(const GatherJob *jobs, int nJobs, int64_t blocks, const GatherShape &g, cudaStream_t s) {
  using AT = KT;
#define FG_GATHER_B(LL, JJ)                                                                               \
  if (g.L == LL && g.J == JJ) {                                                                           \
    auto kern = k_gather_batch<SlotT, KCPLX, KT, AT, LL, JJ>;                                             \
    static SmemAllowance allowed;                                                                        \
    FG_CUDA(allowSmem(kern, g.smem, allowed));                                                           \
    kern<<<(unsigned)blocks, 32 * g.wpb, g.smem, s>>>(jobs, nJobs, g.rowsPerBlock);                       \
    FG_CUDA(cudaGetLastError());                                                                          \
    return FG_OK;                                                                                         \
  }
  FG_GATHER_B(2, 3)
  FG_GATHER_B(4, 3)
  FG_GATHER_B(8, 3)
  FG_GATHER_B(8, 5)
  FG_GATHER_B(16, 3)
  FG_GATHER_B(32, 3)
#undef FG_GATHER_B
  setLastError("batched gather: unsupported (lanes, columns) shape");
  return FG_ERR_ARG;
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

int launchGatherBatch(const GatherJob *jobsDev, int nJobs, int64_t blocks, int slotBytes, int kcplx, int keIsFloat,
                      const GatherShape &g, cudaStream_t s) {
  if (blocks <= 0) return FG_OK;
  countLaunch();
  if (g.v4) {
    if (slotBytes != 1 || kcplx || !keIsFloat) {
      setLastError("batched gather: vector shape for real FP32 element matrices with one-byte slots only");
      return FG_ERR_ARG;
    }
    static SmemAllowance allowed;
    FG_CUDA(allowSmem(k_gather_batch_v4, g.smem, allowed));
    ProfScope prof("k_gather_batch_v4", s);
    k_gather_batch_v4<<<(unsigned)blocks, 32 * g.wpb, g.smem, s>>>(jobsDev, nJobs, g.L);
    FG_CUDA(cudaGetLastError());
    return FG_OK;
  }
  ProfScope prof("k_gather_batch", s);
  if (slotBytes == 1) {
    if (keIsFloat)
      return kcplx ? launchBatchTyped<uint8_t, true, float>(jobsDev, nJobs, blocks, g, s) : launchBatchTyped<uint8_t, false, float>(jobsDev, nJobs, blocks, g, s);
    return kcplx ? launchBatchTyped<uint8_t, true, double>(jobsDev, nJobs, blocks, g, s) : launchBatchTyped<uint8_t, false, double>(jobsDev, nJobs, blocks, g, s);
  }
  if (keIsFloat)
    return kcplx ? launchBatchTyped<uint16_t, true, float>(jobsDev, nJobs, blocks, g, s) : launchBatchTyped<uint16_t, false, float>(jobsDev, nJobs, blocks, g, s);
  return kcplx ? launchBatchTyped<uint16_t, true, double>(jobsDev, nJobs, blocks, g, s) : launchBatchTyped<uint16_t, false, double>(jobsDev, nJobs, blocks, g, s);
}

}  // namespace femg
