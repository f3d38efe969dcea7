// Fused mixed-precision assembly: the tensor-core element contraction and the
// CSR reduction in one kernel, so that no element matrix goes through HBM.
//
// The split mixed path writes every FP32 element matrix (4 n^2 bytes per
// element) from the contraction and reads it back in the reduction. Here the
// CSR rows are cut into blocks of consecutive rows (consecutive in the Hilbert
// numbering, so a block is a compact piece of the mesh). One CTA takes one
// block at a time:
//   1. its element list (every element with a DOF row in the block, at most
//      128: one MMA tile) gathers the elements' factor rows [hi | lo] into
//      shared memory (cp.async);
//   2. one tcgen05 MMA chain per 256 columns computes the 128 element
//      matrices against one shared reference tensor image (3xTF32, FP32
//      accumulation in TMEM), Ke = D_e T;
//   3. TMEM is drained into a shared stage, keeping only the element rows
//      whose DOF row lies in the block, with the element's orientation signs
//      applied (below);
//   4. each row of the block is reduced by a sub-warp, walking its
//      (element, local row) list in element order into a shared FP32 copy of
//      the block's CSR slice at the precomputed slots (the order of the split
//      path's reduction, so results are deterministic);
//   5. the slice is written to the CSR values once, coalesced.
// Elements that touch several blocks are contracted once per block: the
// tensor pipe has room, HBM has not.
//
// One reference tensor for every element: for hierarchical H1 of order <= 3
// (and Lagrange) the element orientations only flip the signs of basis
// functions (an edge function lambda_a lambda_b P_k(lambda_b - lambda_a)
// changes sign with the edge direction when k is odd; the order-3 face
// bubble is symmetric), so T^o = S_o T^0 S_o with S_o diagonal +-1 and
// Ke^o[i][j] = s_i s_j (D_e T^0)[i][j]. The host checks that relation on the
// plan's basis tables and falls back to the split path when it does not hold
// (order 4 face functions mix under face rotations).
//
// Per block the metadata is one contiguous, 16-byte aligned record loaded by
// one bulk copy (the next block's copy overlaps the current block):
//   elems[U]      uint4 {factor row, mask of local rows in the block, sign mask, first pair}
//   rowPair[R+1]  u16  offsets of each row's pair list
//   rowCsr[R+1]   u16  offset of each row in the block's CSR slice
//   pairs[P]      u16  pair (element-local row) per list entry, element order
//   flat[P]       u32  e * n + i of each pair (the element right-hand side)
//   slots[P][n]   u8   position of each column in its CSR row
// Replaces BilinearTerm::evaluate (src/term/BilinearTerm.cpp:304-343) and
// MatrixFactory::addValues (src/system/MatrixFactory.cpp:233-307) for one
// bucket, as the split path does.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include <cuda.h>

#include "common.cuh"

namespace femg {

#include "tc_ptx.cuh"

constexpr int kFThreads = 256;
constexpr int kFTile = 128;      // elements per block: the MMA's M
constexpr int kFRowF = 16;       // floats per factor row: [hi(8) | lo(8)]
constexpr int kFPairMax = 320;   // element rows per block (stage capacity)
constexpr int kFNnzMax = 4096;   // CSR entries per block (shared slice)
constexpr int kFRowsMax = 255;   // CSR rows per block
constexpr int kFTmemCols = 256;  // TMEM columns per CTA (two CTAs per SM)

struct FusedBlock {
  uint32_t meta16;  // record offset / 16
  uint32_t r0;      // first row
  uint32_t R, U, P;
  uint32_t nnz;     // entries of the slice
  uint32_t csr;     // CSR offset of the slice
  uint32_t bytes;   // record size (multiple of 16)
};

struct FusedParams {
  const FusedBlock *blocks;
  int nBlocks;
  const unsigned char *meta;
  const float *A;  // [E][16] factor rows
  const float *B;  // [Npad][16] reference image [B_hi ; B_lo], core-matrix layout
  int n, Npad, SR, metaMax;
  const double2 *be;  // [E][n] element right-hand sides, or null
  double2 *values, *rhs;
  int acc;
  int *err;
};

struct FusedState {
  int built = 0, ok = 0;
  std::string why;
  int n = 0, Npad = 0, SR = 0, metaMax = 0, nBlocks = 0, grid = 0;
  size_t smem = 0;
  FusedBlock *blocks = nullptr;
  unsigned char *meta = nullptr;
  float *A = nullptr;
  float *B = nullptr;
  int *err = nullptr;
  int *errHost = nullptr;
  cudaEvent_t errEvent = nullptr;
  bool errPending = false;
  double avgElemsPerBlock = 0.0, elemVisits = 0.0;
};

__host__ __device__ inline uint32_t align16(uint32_t x) { return (x + 15u) & ~15u; }

// byte offsets of the sections of a block record
struct MetaLayout {
  uint32_t rowPair, rowCsr, pairs, flat, slots, size;
};
__host__ __device__ inline MetaLayout metaLayout(uint32_t U, uint32_t R, uint32_t P, uint32_t n) {
  MetaLayout m;
  m.rowPair = align16(16u * U);
  m.rowCsr = align16(m.rowPair + 2u * (R + 1));
  m.pairs = align16(m.rowCsr + 2u * (R + 1));
  m.flat = align16(m.pairs + 2u * P);
  m.slots = align16(m.flat + 4u * P);
  m.size = align16(m.slots + P * n);
  return m;
}

// TMEM columns [cBegin, cEnd) of the chunk starting at column c0 (multiples
// of 16) of this warp's 32 lanes (tile rows = elements) into the stage: entry
// (i, j) of the element matrix sits in column i n + j.
__device__ inline void fusedDrain(uint32_t tmemRow, int c0, int cBegin, int cEnd, uint4 el, bool live, float *Stage, int n, int SR) {
  for (int c = cBegin; c < cEnd;) {
    float v[32];
    int w;
    if (cEnd - c >= 32) {
      tmemLoad32(tmemRow + (uint32_t)c, v);
      w = 32;
    } else {
      tmemLoad16(tmemRow + (uint32_t)c, v);
      w = 16;
    }
    if (live) {
      const int col = c0 + c;
      int i = col / n, j = col - i * n;
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        if (k < w && i < n && ((el.y >> i) & 1u)) {
          const int pidx = (int)el.w + __popc(el.y & ((1u << i) - 1u));
          const float val = (((el.z >> i) ^ (el.z >> j)) & 1u) ? -v[k] : v[k];
          Stage[pidx * SR + j] = val;
        }
        if (++j == n) {
          j = 0;
          ++i;
        }
      }
    }
    c += w;
  }
}

__global__ void __launch_bounds__(kFThreads, 2) k_fused_tf32x3(const __grid_constant__ FusedParams fp) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t *mmaBar = reinterpret_cast<uint64_t *>(smem);
  uint64_t *metaBar = reinterpret_cast<uint64_t *>(smem + 8);  // [2]
  uint64_t *bBar = reinterpret_cast<uint64_t *>(smem + 24);
  uint32_t *tmemBase = reinterpret_cast<uint32_t *>(smem + 32);
  float *Bs = reinterpret_cast<float *>(smem + 1024);  // Npad * 16 floats
  float *As = Bs + fp.Npad * kFRowF;                   // 128 * 16 floats (Npad * 64 is a multiple of 1024)
  unsigned char *Meta0 = reinterpret_cast<unsigned char *>(As + kFTile * kFRowF);
  unsigned char *Meta1 = Meta0 + fp.metaMax;
  float *Stage = reinterpret_cast<float *>(Meta1 + fp.metaMax);
  float *Acc = Stage + kFPairMax * fp.SR;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, half = warp >> 2;
  const int n = fp.n;

  if (warp == 0) {
    tmemAlloc(tmemBase, kFTmemCols);
    tmemRelinquish();
  }
  if (tid == 0) {
    mbarInit(mmaBar, 1);
    mbarInit(&metaBar[0], 1);
    mbarInit(&metaBar[1], 1);
    mbarInit(bBar, 1);
    fenceMbarInit();
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = *tmemBase;
  const uint32_t tmemRow = tmem + ((uint32_t)(quad * 32) << 16);
  const uint32_t bBytes = (uint32_t)fp.Npad * kFRowF * 4u;
  int b = blockIdx.x;
  uint32_t mmaPhase = 0, metaParity = 0, metaPending = 0;  // per buffer: completion parity, copy in flight
  bool bPending = false, failed = false;
  if (tid == 0 && b < fp.nBlocks) {
    mbarExpectTx(bBar, bBytes);
    bulkLoad(smemAddr(Bs), fp.B, bBytes, bBar);
    const FusedBlock F0 = fp.blocks[b];
    mbarExpectTx(&metaBar[0], F0.bytes);
    bulkLoad(smemAddr(Meta0), fp.meta + (size_t)F0.meta16 * 16, F0.bytes, &metaBar[0]);
  }
  if (b < fp.nBlocks) {
    bPending = true;
    metaPending = 1u;
  }
  for (int buf = 0; b < fp.nBlocks && !failed; b += gridDim.x, buf ^= 1) {
    const FusedBlock F = fp.blocks[b];
    unsigned char *M = buf ? Meta1 : Meta0;
    const bool okMeta = mbarWait(&metaBar[buf], (metaParity >> buf) & 1u);
    if (__syncthreads_or(okMeta ? 0 : 1)) {
      if (tid == 0) atomicExch(fp.err, 1);
      failed = true;
      break;
    }
    metaParity ^= 1u << buf;
    metaPending &= ~(1u << buf);
    // the next block's record into the other buffer (its last reader, the
    // block before this one, has finished: the loop ends with a barrier)
    const int nb = b + (int)gridDim.x;
    if (nb < fp.nBlocks) {
      if (tid == 0) {
        fenceProxyAsync();
        const FusedBlock F1 = fp.blocks[nb];
        mbarExpectTx(&metaBar[buf ^ 1], F1.bytes);
        bulkLoad(smemAddr(buf ? Meta0 : Meta1), fp.meta + (size_t)F1.meta16 * 16, F1.bytes, &metaBar[buf ^ 1]);
      }
      metaPending |= 1u << (buf ^ 1);
    }
    const MetaLayout L = metaLayout(F.U, F.R, F.P, (uint32_t)n);
    const uint4 *elems = reinterpret_cast<const uint4 *>(M);
    // factor rows of the block's elements: row r, 16-byte chunk kc -> core
    // matrix (r / 8, kc) with K-direction stride 2048 bytes; rows past U read zero
    for (int c = tid; c < kFTile * 4; c += kFThreads) {
      const int r = c >> 2, kc = c & 3;
      const bool live = r < (int)F.U;
      const float *src = fp.A + (size_t)(live ? elems[r].x : 0u) * kFRowF + kc * 4;
      cpAsync16(smemAddr(As) + kc * 2048 + (r >> 3) * 128 + (r & 7) * 16, src, live ? 16u : 0u);
    }
    cpAsyncCommit();
    for (uint32_t t = tid; t < F.nnz; t += kFThreads) Acc[t] = 0.0f;
    cpAsyncWaitAll();
    fenceProxyAsync();  // the generic-proxy copies before the MMAs read them
    __syncthreads();
    if (bPending) {
      const bool okB = mbarWait(bBar, 0);
      if (__syncthreads_or(okB ? 0 : 1)) {
        if (tid == 0) atomicExch(fp.err, 1);
        failed = true;
        break;
      }
      bPending = false;
    }
    const int row = quad * 32 + lane;
    const bool live = row < (int)F.U;
    const uint4 el = live ? elems[row] : make_uint4(0, 0, 0, 0);
    const uint32_t bLbo = (uint32_t)fp.Npad * 16u;
    for (int c0 = 0; c0 < fp.Npad && !failed; c0 += kFTmemCols) {
      const int ncols = min(kFTmemCols, fp.Npad - c0);
      if (tid == 0) {
        tcFenceAfter();
        const uint32_t idesc = idescTf32(kFTile, ncols);
        // A_hi B_hi + A_lo B_hi + A_hi B_lo
        for (int ks = 0; ks < 3; ++ks) {
          const uint64_t ad = smemDesc(smemAddr(As) + (ks == 1 ? 2u : 0u) * 2048u, 2048, 128);
          const uint64_t bd = smemDesc(smemAddr(Bs) + (ks == 2 ? 2u : 0u) * bLbo + (uint32_t)(c0 >> 3) * 128u, bLbo, 128);
          mmaTf32(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
        }
        mmaCommit(mmaBar);
      }
      __syncwarp();
      const bool ok = mbarWait(mmaBar, mmaPhase);
      failed = __syncthreads_or(ok ? 0 : 1) != 0;
      if (failed) {
        if (tid == 0) atomicExch(fp.err, 1);
      } else {
        mmaPhase ^= 1u;
      }
      tcFenceAfter();
      if (!failed) {
        const int split = min(((ncols / 2 + 15) / 16) * 16, ncols);
        if (half == 0) fusedDrain(tmemRow, c0, 0, split, el, live, Stage, n, fp.SR);
        else fusedDrain(tmemRow, c0, split, ncols, el, live, Stage, n, fp.SR);
      }
      tcFenceBefore();
      __syncthreads();
    }
    if (failed) break;
    // rows of the block: a sub-warp of 8 lanes per row, 4 rows per warp
    const uint16_t *rowPair = reinterpret_cast<const uint16_t *>(M + L.rowPair);
    const uint16_t *rowCsr = reinterpret_cast<const uint16_t *>(M + L.rowCsr);
    const uint16_t *pairs = reinterpret_cast<const uint16_t *>(M + L.pairs);
    const uint32_t *flat = reinterpret_cast<const uint32_t *>(M + L.flat);
    const uint8_t *slots = M + L.slots;
    const int sub = lane >> 3, lt = lane & 7;
    for (int base = warp * 4; base < (int)F.R; base += 32) {
      const int lr = base + sub;
      const bool liveRow = lr < (int)F.R;
      const int k0 = liveRow ? rowPair[lr] : 0, cnt = liveRow ? rowPair[lr + 1] - k0 : 0;
      const int off = liveRow ? rowCsr[lr] : 0;
      int maxCnt = cnt;
      maxCnt = max(maxCnt, __shfl_xor_sync(0xffffffffu, maxCnt, 8));
      maxCnt = max(maxCnt, __shfl_xor_sync(0xffffffffu, maxCnt, 16));
      double2 bsum = make_double2(0.0, 0.0);
      for (int k = 0; k < maxCnt; ++k) {
        if (k < cnt) {
          const int p = pairs[k0 + k];
          const float *sv = Stage + p * fp.SR;
          const uint8_t *sl = slots + p * n;
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int j = lt + 8 * jj;
            if (j < n) {
              const int s = sl[j];
              // the lanes of one element row hit distinct slots (but for the
              // aliased bubble rows of upper storage); rows are ordered by the
              // __syncwarp below, so each value is summed in list order
              if (s < 0xFE) atomicAdd(&Acc[off + s], sv[j]);
            }
          }
          if (fp.be && lt == 0) bsum = cadd(bsum, fp.be[flat[p]]);
        }
        __syncwarp();
      }
      if (fp.rhs && liveRow && lt == 0) {
        const size_t r = (size_t)F.r0 + lr;
        fp.rhs[r] = fp.acc ? cadd(fp.rhs[r], bsum) : bsum;
      }
    }
    __syncthreads();
    for (uint32_t t = tid; t < F.nnz; t += kFThreads) {
      double2 v = make_double2((double)Acc[t], 0.0);
      if (fp.acc) v = cadd(fp.values[F.csr + t], v);
      fp.values[F.csr + t] = v;
    }
    __syncthreads();
  }
  if (failed) {
    // the MMA chain and the copies in flight get a second bounded chance to
    // retire before the TMEM and the shared memory are released
    mbarWait(mmaBar, mmaPhase);
    for (int k = 0; k < 2; ++k)
      if (metaPending & (1u << k)) mbarWait(&metaBar[k], (metaParity >> k) & 1u);
    if (bPending) mbarWait(bBar, 0);
  }
  __syncthreads();
  tcFenceAfter();
  if (warp == 0) tmemDealloc(tmem, kFTmemCols);
}

static FusedState *fusedState(fg_plan *plan) {
  if (!plan->fused) plan->fused = new FusedState();
  return (FusedState *)plan->fused;
}

static size_t fusedSmem(int Npad, int SR, int metaMax) {
  return 1024 + (size_t)Npad * kFRowF * 4 + (size_t)kFTile * kFRowF * 4 + 2 * (size_t)metaMax + (size_t)kFPairMax * SR * 4 +
         (size_t)kFNnzMax * 4;
}

// Sign of each basis function of orientation o against orientation 0 (bit i
// set: phi_i^o = -phi_i^0), from the basis tables; false when some function
// is neither equal nor opposite (then one reference tensor does not serve).
static bool orientationSigns(const PlanDev &p, const std::vector<double> &bval, const std::vector<double> &bgrad,
                             std::vector<uint32_t> &sign) {
  const int nb = p.nb, nq = p.nq;
  sign.assign(p.nOrient, 0u);
  for (int o = 1; o < p.nOrient; ++o)
    for (int i = 0; i < nb; ++i) {
      double scale = 0.0, dp = 0.0, dm = 0.0;
      for (int q = 0; q < nq; ++q) {
        const double v0 = bval[((size_t)0 * nq + q) * nb + i], v = bval[((size_t)o * nq + q) * nb + i];
        scale = std::max(scale, std::fabs(v0));
        dp = std::max(dp, std::fabs(v - v0));
        dm = std::max(dm, std::fabs(v + v0));
        for (int c = 0; c < 3; ++c) {
          const double g0 = bgrad[(((size_t)0 * nq + q) * nb + i) * 3 + c], g = bgrad[(((size_t)o * nq + q) * nb + i) * 3 + c];
          scale = std::max(scale, std::fabs(g0));
          dp = std::max(dp, std::fabs(g - g0));
          dm = std::max(dm, std::fabs(g + g0));
        }
      }
      const double tol = 1e-13 * std::max(scale, 1e-300);
      if (dp <= tol) continue;
      if (dm <= tol) {
        sign[o] |= 1u << i;
        continue;
      }
      return false;
    }
  return true;
}

// Builds the block records; ok = 0 with a reason when the plan does not fit
// the fused kernel (the caller then runs the split path).
static int prepareFused(fg_plan *plan) {
  FusedState *f = fusedState(plan);
  if (f->built) return FG_OK;
  f->built = 1;
  const PlanDev &p = plan->d;
  auto no = [&](const char *why) {
    f->ok = 0;
    f->why = why;
    return FG_OK;
  };
  if (p.mult != 1 || p.form != FG_FORM_0) return no("one-component H1 fields only");
  if (!p.affine) return no("affine elements only");
  if (p.n > 32) return no("at most 32 DOFs per element");
  if (p.slotBytes != 1) return no("CSR rows shorter than 254 entries only");
  if (p.lscale) return no("no linked DOFs");
  if (p.E == 0 || p.nRows == 0) return no("empty plan");
  const int n = p.n, nq = p.nq, nb = p.nb;
  const int nn2 = n * n;
  const int Npad = (nn2 + 15) / 16 * 16;
  if (Npad > 2 * kFTmemCols) return no("element matrices of at most 512 entries");
  // tables back to the host (set-up only)
  std::vector<double> w(nq), bval((size_t)p.nOrient * nq * nb), bgrad((size_t)p.nOrient * nq * nb * 3);
  FG_CUDA(cudaMemcpy(w.data(), p.w, w.size() * 8, cudaMemcpyDeviceToHost));
  FG_CUDA(cudaMemcpy(bval.data(), p.bval, bval.size() * 8, cudaMemcpyDeviceToHost));
  FG_CUDA(cudaMemcpy(bgrad.data(), p.bgrad, bgrad.size() * 8, cudaMemcpyDeviceToHost));
  std::vector<uint32_t> signOf;
  if (!orientationSigns(p, bval, bgrad, signOf)) return no("orientations that do more than flip basis signs");
  const int64_t E = p.E;
  const uint64_t nRows = p.nRows;
  std::vector<uint64_t> rowPtr(nRows + 1);
  std::vector<uint32_t> rowElem;
  std::vector<uint8_t> slot((size_t)E * n * p.slotLd);
  std::vector<int32_t> orient((size_t)E, 0);
  FG_CUDA(cudaMemcpy(rowPtr.data(), p.rowPtr, rowPtr.size() * 8, cudaMemcpyDeviceToHost));
  rowElem.resize(rowPtr[nRows]);
  if (!rowElem.empty()) FG_CUDA(cudaMemcpy(rowElem.data(), p.rowElem, rowElem.size() * 4, cudaMemcpyDeviceToHost));
  FG_CUDA(cudaMemcpy(slot.data(), p.slot, slot.size(), cudaMemcpyDeviceToHost));
  if (p.orient) FG_CUDA(cudaMemcpy(orient.data(), p.orient, (size_t)E * 4, cudaMemcpyDeviceToHost));
  for (uint8_t s : slot)
    if (s == 0xFF) return no("no fixed (Dirichlet) columns");
  const std::vector<uint64_t> &ai = plan->hAi;
  // blocks of consecutive rows
  std::vector<FusedBlock> blocks;
  std::vector<unsigned char> meta;
  std::vector<int64_t> mark((size_t)E, -1);
  std::vector<int32_t> local((size_t)E, 0);
  std::vector<uint32_t> elems, need;
  int metaMax = 16;
  double visits = 0.0;
  for (uint64_t r = 0; r < nRows;) {
    const uint64_t r0 = r;
    const int64_t id = (int64_t)blocks.size();
    elems.clear();
    uint64_t P = 0, nnz = 0;
    while (r < nRows && r - r0 < (uint64_t)kFRowsMax) {
      const uint64_t cnt = rowPtr[r + 1] - rowPtr[r], len = ai[r + 1] - ai[r];
      uint32_t fresh = 0;
      for (uint64_t k = rowPtr[r]; k < rowPtr[r + 1]; ++k) {
        const uint32_t e = rowElem[k] >> 6;
        if (mark[e] != id) {
          mark[e] = id;  // provisional: undone below when the row does not fit
          local[e] = -1 - (int32_t)fresh;
          ++fresh;
        }
      }
      const bool fits = elems.size() + fresh <= (size_t)kFTile && P + cnt <= (uint64_t)kFPairMax && nnz + len <= (uint64_t)kFNnzMax;
      for (uint64_t k = rowPtr[r]; k < rowPtr[r + 1]; ++k) {
        const uint32_t e = rowElem[k] >> 6;
        if (local[e] < 0) {
          if (fits) {
            local[e] = (int32_t)elems.size();
            elems.push_back(e);
          } else {
            mark[e] = -1;
            local[e] = 0;
          }
        }
      }
      if (!fits) break;
      P += cnt;
      nnz += len;
      ++r;
    }
    if (r == r0) return no("a CSR row with more elements, contributions or entries than a block holds");
    const uint32_t R = (uint32_t)(r - r0), U = (uint32_t)elems.size();
    // elements in increasing order (the order of the gathered factor rows)
    std::vector<uint32_t> order(elems);
    std::sort(order.begin(), order.end());
    for (uint32_t u = 0; u < U; ++u) local[order[u]] = (int32_t)u;
    need.assign(U, 0u);
    for (uint64_t rr = r0; rr < r; ++rr)
      for (uint64_t k = rowPtr[rr]; k < rowPtr[rr + 1]; ++k) need[local[rowElem[k] >> 6]] |= 1u << (rowElem[k] & 63);
    std::vector<uint32_t> pairBase(U);
    uint32_t acc = 0;
    for (uint32_t u = 0; u < U; ++u) {
      pairBase[u] = acc;
      acc += (uint32_t)__builtin_popcount(need[u]);
    }
    const MetaLayout L = metaLayout(U, R, (uint32_t)P, (uint32_t)n);
    FusedBlock fb;
    fb.meta16 = (uint32_t)(meta.size() / 16);
    fb.r0 = (uint32_t)r0;
    fb.R = R;
    fb.U = U;
    fb.P = (uint32_t)P;
    fb.nnz = (uint32_t)nnz;
    fb.csr = (uint32_t)ai[r0];
    fb.bytes = L.size;
    const size_t at = meta.size();
    meta.resize(at + L.size, 0);
    unsigned char *m = meta.data() + at;
    uint4 *el = reinterpret_cast<uint4 *>(m);
    for (uint32_t u = 0; u < U; ++u) el[u] = make_uint4(order[u], need[u], signOf[orient[order[u]]], pairBase[u]);
    uint16_t *rowPair = reinterpret_cast<uint16_t *>(m + L.rowPair);
    uint16_t *rowCsr = reinterpret_cast<uint16_t *>(m + L.rowCsr);
    uint16_t *pairs = reinterpret_cast<uint16_t *>(m + L.pairs);
    uint32_t *flat = reinterpret_cast<uint32_t *>(m + L.flat);
    uint8_t *slots = m + L.slots;
    uint32_t k2 = 0;
    for (uint32_t lr = 0; lr < R; ++lr) {
      const uint64_t rr = r0 + lr;
      rowPair[lr] = (uint16_t)k2;
      rowCsr[lr] = (uint16_t)(ai[rr] - ai[r0]);
      for (uint64_t k = rowPtr[rr]; k < rowPtr[rr + 1]; ++k) {
        const uint32_t e = rowElem[k] >> 6, i = rowElem[k] & 63;
        const uint32_t u = (uint32_t)local[e];
        const uint32_t pidx = pairBase[u] + (uint32_t)__builtin_popcount(need[u] & ((1u << i) - 1u));
        pairs[k2++] = (uint16_t)pidx;
        flat[pidx] = e * (uint32_t)n + i;
        std::memcpy(slots + (size_t)pidx * n, &slot[((size_t)e * n + i) * p.slotLd], (size_t)n);
      }
    }
    rowPair[R] = (uint16_t)k2;
    rowCsr[R] = (uint16_t)nnz;
    metaMax = std::max(metaMax, (int)L.size);
    visits += U;
    blocks.push_back(fb);
  }
  if ((double)meta.size() >= 16.0 * 4294967295.0) return no("block records beyond 2^36 bytes");
  // reference tensor image [B_hi ; B_lo] of orientation 0
  std::vector<float> img;
  buildB(p, w, bval, bgrad, 0, Npad, 8, img, true);
  const int SR = n | 1;  // odd stage stride: the drain's stores hit distinct banks
  const size_t smem = fusedSmem(Npad, SR, metaMax);
  if (smem > 113 * 1024) return no("block records too large for two CTAs per SM");
  FG_CUDA(cudaMalloc(&f->blocks, blocks.size() * sizeof(FusedBlock)));
  FG_CUDA(cudaMemcpy(f->blocks, blocks.data(), blocks.size() * sizeof(FusedBlock), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMalloc(&f->meta, meta.size()));
  FG_CUDA(cudaMemcpy(f->meta, meta.data(), meta.size(), cudaMemcpyHostToDevice));
  FG_CUDA(cudaMalloc(&f->B, img.size() * 4));
  FG_CUDA(cudaMemcpy(f->B, img.data(), img.size() * 4, cudaMemcpyHostToDevice));
  FG_CUDA(cudaMalloc(&f->A, (size_t)E * kFRowF * 4));
  FG_CUDA(cudaMalloc(&f->err, sizeof(int)));
  FG_CUDA(cudaMemset(f->err, 0, sizeof(int)));
  FG_CUDA(cudaMallocHost(&f->errHost, sizeof(int)));
  *f->errHost = 0;
  FG_CUDA(cudaEventCreateWithFlags(&f->errEvent, cudaEventDisableTiming));
  f->n = n;
  f->Npad = Npad;
  f->SR = SR;
  f->metaMax = metaMax;
  f->nBlocks = (int)blocks.size();
  f->smem = smem;
  f->grid = std::max(1, std::min(f->nBlocks, 2 * smCount()));
  f->avgElemsPerBlock = visits / std::max<size_t>(blocks.size(), 1);
  f->elemVisits = visits / (double)E;
  f->ok = 1;
  return FG_OK;
}

// whether a mixed call of these terms runs fused
bool fusedApplies(fg_plan *plan, const DevTerms &dt) {
  if (!plan->mixedFused || dt.complexKe || dt.hasElastic || dt.hasJacMod || dt.nonSym || plan->d.nFixed > 0) return false;
  if (dt.tensorMassTerm >= 0) return false;
  if (prepareFused(plan) != FG_OK) {
    cudaGetLastError();
    return false;
  }
  return fusedState(plan)->ok != 0;
}

static int fusedCheckTimeout(FusedState *f, bool wait) {
  if (!f->errPending) return FG_OK;
  if (wait) {
    if (cudaEventSynchronize(f->errEvent) != cudaSuccess) return FG_ERR_CUDA;
  } else if (cudaEventQuery(f->errEvent) != cudaSuccess) {
    cudaGetLastError();
    return FG_OK;
  }
  f->errPending = false;
  if (*f->errHost) {
    *f->errHost = 0;
    cudaMemset(f->err, 0, sizeof(int));
    setLastError("fused mixed path: a bounded device wait timed out");
    return FG_ERR_TIMEOUT;
  }
  return FG_OK;
}

int fusedTimeout(fg_plan *plan, bool wait) { return plan->fused ? fusedCheckTimeout(fusedState(plan), wait) : FG_OK; }

// Factor rows, then the fused contraction and reduction into values / rhs
// (device pointers), be: element right-hand sides or null.
int launchFused(fg_plan *plan, const DevTerms &dt, const DevTerms *dterms, const double2 *be, double2 *values, double2 *rhs,
                cudaStream_t s) {
  FusedState *f = fusedState(plan);
  int st = fusedCheckTimeout(f, false);
  if (st) return st;
  const PlanDev &p = plan->d;
  if ((st = launchFactorsCompact(p, dterms, dt.tensorTerm >= 0, f->A, s))) return st;
  FusedParams fp;
  std::memset(&fp, 0, sizeof(fp));
  fp.blocks = f->blocks;
  fp.nBlocks = f->nBlocks;
  fp.meta = f->meta;
  fp.A = f->A;
  fp.B = f->B;
  fp.n = f->n;
  fp.Npad = f->Npad;
  fp.SR = f->SR;
  fp.metaMax = f->metaMax;
  fp.be = be;
  fp.values = values;
  fp.rhs = rhs;
  fp.acc = plan->accumulate;
  fp.err = f->err;
  static SmemAllowance allowed;
  FG_CUDA(allowSmem(k_fused_tf32x3, f->smem, allowed));
  {
    ProfScope prof("k_fused_tf32x3", s);
    k_fused_tf32x3<<<f->grid, kFThreads, f->smem, s>>>(fp);
    countLaunch();
    FG_CUDA(cudaGetLastError());
  }
  FG_CUDA(cudaMemcpyAsync(f->errHost, f->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaEventRecord(f->errEvent, s));
  f->errPending = true;
  return FG_OK;
}

}  // namespace femg

using namespace femg;

extern "C" int fg_plan_set_mixed_fused(fg_plan *plan, int32_t on) {
  if (!plan || (on != 0 && on != 1)) {
    setLastError("fg_plan_set_mixed_fused: invalid arguments");
    return FG_ERR_ARG;
  }
  plan->mixedFused = on;
  return FG_OK;
}

extern "C" int fg_plan_fused_info(fg_plan *plan, int32_t *applies, int32_t *blocks, double *elems_per_block,
                                  double *contractions_per_element) {
  if (!plan) return FG_ERR_ARG;
  int st = prepareFused(plan);
  if (st) return st;
  FusedState *f = fusedState(plan);
  if (applies) *applies = f->ok;
  if (blocks) *blocks = f->nBlocks;
  if (elems_per_block) *elems_per_block = f->avgElemsPerBlock;
  if (contractions_per_element) *contractions_per_element = f->elemVisits;
  if (!f->ok) setLastError("fused mixed path not applicable: " + f->why);
  return FG_OK;
}

extern "C" void fusedDestroy(fg_plan *plan) {
  FusedState *f = (FusedState *)plan->fused;
  if (!f) return;
  cudaFree(f->blocks);
  cudaFree(f->meta);
  cudaFree(f->A);
  cudaFree(f->B);
  cudaFree(f->err);
  if (f->errHost) cudaFreeHost(f->errHost);
  if (f->errEvent) cudaEventDestroy(f->errEvent);
  delete f;
  plan->fused = nullptr;
}
