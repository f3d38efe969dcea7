// Multi-frequency assembly: the system of the AFrequency module at n_freq
// angular frequencies from one integration of the element matrices.
//
// The reference assembles one frequency per assemble() call: every term with a
// time derivative is scaled by the module factor of the formulation's current
// frequency, -omega^2 for dt2 and -i omega for dt1, before the element matrix
// is summed (src/term/Assembler.cpp:263-305; AFrequencyModule,
// src/system/MatrixModule.cpp:100-171). The terms split into at most three
// groups by time derivative, K (none), C (dt) and M (dt2), whose element
// matrices do not depend on the frequency. They are integrated once (FP64
// element kernels, or the mixed-precision factor rows and one tensor-core
// contraction over all groups), and one row-owner reduction accumulates the
// group sums of each CSR row in shared memory and writes every frequency's
//   values_f = K + (-i omega_f) C + (-omega_f^2) M
// and right-hand side (sources, plus the Dirichlet lifting of each group
// scaled the same way). The reduction visits the element rows in the order
// of the single-frequency gather, so each group sum is deterministic.
#include <cstring>
#include <functional>

#include "common.cuh"

namespace femg {

constexpr int kMaxGroups = 3;
constexpr int kMaxFreq = 64;

struct MultiIn {
  const void *ke[kMaxGroups];    // element matrices of group g (KT)
  int64_t stride[kMaxGroups];    // KT entries from one element to the next
  int cplx[kMaxGroups];          // group g has an imaginary part (at +n*n)
  int realFactor[kMaxGroups];    // the factors of group g are real for every output
  int imagFactor[kMaxGroups];    // ... purely imaginary for every output
  int G, F, R;
  int anyCplx;                   // some group has an imaginary part: two accumulators per group and slot, else one
  KeLayout lay;                  // element-matrix layout (ld entries per component)
  const double2 *coef;           // [F][G] factors of the value arrays
  const double2 *rcoef;          // [R][G] factors of the liftings in the right-hand sides
  const double2 *be;             // [E][n] element right-hand sides or null
  const double2 *uD;             // Dirichlet values or null
  double2 *const *values;        // F value arrays [nnz] (device table)
  double2 *const *rhs;           // R right-hand sides [nRows] (device table), or null
};

template <typename SlotT, typename KT, int L, int J>
__global__ void __launch_bounds__(256)
    k_gather_multi(const PlanDev p, const MultiIn in, int rowsPerBlock) {
  using AT = KT;
  constexpr int R = 32 / L;  // rows per warp; J columns per lane (L * J >= n)
  const int G = in.G, F = in.F;
  auto keOff = [&](int ii, int jj) -> int { return keOffset(in.lay, p.n, ii, jj); };
  extern __shared__ __align__(16) unsigned char smraw[];
  AT *cf = reinterpret_cast<AT *>(smraw);  // [F][G][2] factors in the accumulation type
  for (int k = threadIdx.x; k < F * G; k += blockDim.x) {
    cf[2 * k] = (AT)in.coef[k].x;
    cf[2 * k + 1] = (AT)in.coef[k].y;
  }
  __syncthreads();
  const size_t cfBytes = ((size_t)F * G * 2 * sizeof(AT) + 15) / 16 * 16;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / L, lt = lane % L;
  // accumulators per slot: (re, im) per group when some group is complex,
  // else one real sum per group
  const int perSlot = in.anyCplx ? 2 * G : G;
  const int gStep = in.anyCplx ? 2 : 1;
  AT *A = reinterpret_cast<AT *>(smraw + cfBytes) + (size_t)(warp * R + sub) * p.maxRowLen * perSlot;
  const SlotT *slot = (const SlotT *)p.slot;
  const SlotT kFixed = (SlotT)(sizeof(SlotT) == 1 ? 0xFF : kSlotFixed);
  const SlotT kIgnore = (SlotT)(sizeof(SlotT) == 1 ? 0xFE : kSlotIgnore);
  const int n = p.n;
  const int nn2 = in.lay.ld;  // entries per component
  const int64_t nRows = (int64_t)p.nRows;
  const int64_t stride = (int64_t)gridDim.x * rowsPerBlock;
  for (int64_t base = (int64_t)blockIdx.x * rowsPerBlock + warp * R; base < nRows; base += stride) {
    const int64_t idx = base + sub;
    const bool live = idx < nRows;
    const uint4 v = live ? p.visit[idx] : make_uint4(0, 0, 0, 0);
    const int64_t row = v.x;
    const uint64_t start = v.y;
    const int len = live ? (int)(v.w & 0xFFFFu) : 0;
    const uint64_t r0 = v.z;
    const int cnt = live ? (int)(v.w >> 16) : 0;
    for (int s = lt; s < len * perSlot; s += L) A[s] = (AT)0;
    int maxCnt = cnt;
#pragma unroll
    for (int off = L; off < 32; off <<= 1) maxCnt = max(maxCnt, __shfl_xor_sync(0xffffffffu, maxCnt, off));
    __syncwarp();
    double2 dc[kMaxGroups];
#pragma unroll
    for (int g = 0; g < kMaxGroups; ++g) dc[g] = make_double2(0.0, 0.0);
    double2 bsum = make_double2(0.0, 0.0);
    for (int k = 0; k < maxCnt; ++k) {
      if (k < cnt) {
        const uint32_t packed = p.visitElem[r0 + k];
        const int64_t e = packed >> 6;
        const int i = packed & 63;
        const SlotT *S = slot + ((size_t)e * n + i) * p.slotLd;
        if (in.be && lt == 0) bsum = cadd(bsum, in.be[e * n + i]);
#pragma unroll
        for (int jj = 0; jj < J; ++jj) {
          const int j = lt + L * jj;
          if (j >= n) continue;
          const SlotT s = S[j];
          if (s == kIgnore) continue;
          if (s != kFixed) {
            const int o = keOff(i, j);
#pragma unroll
            for (int g = 0; g < kMaxGroups; ++g) {
              if (g >= G) break;
              const KT *K = (const KT *)in.ke[g] + e * in.stride[g];
              // distinct slots per lane within an element row; rows are
              // separated by the __syncwarp below, so the adds are ordered
              atomicAdd(&A[(int)s * perSlot + gStep * g], (AT)K[o]);
              if (in.cplx[g]) atomicAdd(&A[(int)s * perSlot + gStep * g + 1], (AT)K[nn2 + o]);
            }
          } else {
            // lifting with the transposed entry (VectorFactory::addValuesDC)
            const int o = keOff(j, i);
            const double2 u = in.uD[p.edof[e * n + j]];
#pragma unroll
            for (int g = 0; g < kMaxGroups; ++g) {
              if (g >= G) break;
              const KT *K = (const KT *)in.ke[g] + e * in.stride[g];
              const double2 kv = make_double2((double)K[o], in.cplx[g] ? (double)K[nn2 + o] : 0.0);
              dc[g] = cadd(dc[g], cmul(kv, u));
            }
          }
        }
      }
      __syncwarp();
    }
    for (int s = lt; s < len; s += L) {
      AT ar[kMaxGroups], ai[kMaxGroups];
#pragma unroll
      for (int g = 0; g < kMaxGroups; ++g) {
        ar[g] = g < G ? A[s * perSlot + gStep * g] : (AT)0;
        ai[g] = (g < G && in.cplx[g]) ? A[s * perSlot + gStep * g + 1] : (AT)0;
      }
      for (int f = 0; f < F; ++f) {
        AT re = (AT)0, im = (AT)0;
#pragma unroll
        for (int g = 0; g < kMaxGroups; ++g) {
          if (g >= G) break;
          const AT cr = cf[2 * (f * G + g)], ci = cf[2 * (f * G + g) + 1];
          // real sums and real or imaginary factors (the usual case) skip the
          // zero products: they cost FP64 issue slots on the FP64 path
          if (in.realFactor[g]) re += cr * ar[g];
          else if (in.imagFactor[g]) im += ci * ar[g];
          else {
            re += cr * ar[g];
            im += ci * ar[g];
          }
          if (in.cplx[g]) {
            re -= ci * ai[g];
            im += cr * ai[g];
          }
        }
        in.values[f][start + s] = make_double2(widen(re), widen(im));
      }
    }
    if (in.rhs) {
      if (in.uD) {
#pragma unroll
        for (int g = 0; g < kMaxGroups; ++g)
#pragma unroll
          for (int off = L / 2; off > 0; off >>= 1) {
            dc[g].x += __shfl_down_sync(0xffffffffu, dc[g].x, off, L);
            dc[g].y += __shfl_down_sync(0xffffffffu, dc[g].y, off, L);
          }
      }
      if (live && lt == 0)
        for (int r = 0; r < in.R; ++r) {
          double2 v = bsum;
#pragma unroll
          for (int g = 0; g < kMaxGroups; ++g)
            if (g < G) v = cadd(v, cmul(in.rcoef[r * G + g], dc[g]));
          in.rhs[r][row] = v;
        }
    }
    __syncwarp();
  }
}

template <typename SlotT, typename KT>
static int launchMultiTyped(const PlanDev &p, const MultiIn &in, cudaStream_t s) {
  // three columns per lane: the 8 x 5 shape of the single-frequency
  // reduction measured 43% slower here (complex accumulators per group, and
  // 16 frequencies written per row)
  const int n = p.n;
  int L = 32;
  if (n <= 6) L = 2;
  else if (n <= 12) L = 4;
  else if (n <= 24) L = 8;
  else if (n <= 48) L = 16;
  const int J = 3;
  const int R = 32 / L;
  const size_t cfBytes = ((size_t)in.F * in.G * 2 * sizeof(KT) + 15) / 16 * 16;
  const size_t rowBytes = (size_t)std::max(p.maxRowLen, 1) * (in.anyCplx ? 2 : 1) * in.G * sizeof(KT);
  int wpb = 8;
  while (wpb > 1 && cfBytes + rowBytes * R * wpb > 200 * 1024) wpb >>= 1;
  const size_t smem = cfBytes + rowBytes * R * wpb;
  if (smem > 200 * 1024) {
    setLastError("multi-frequency gather: CSR row too long for shared memory");
    return FG_ERR_UNSUPPORTED;
  }
  const int rowsPerBlock = wpb * R;
  int64_t blocks = ((int64_t)p.nRows + rowsPerBlock - 1) / rowsPerBlock;
  blocks = std::min<int64_t>(blocks, (int64_t)smCount() * 16);
  bool launched = false;
#define FG_MULTI_L(LL, JJ)                                                                         \
  if (L == LL && J == JJ) {                                                                        \
    launched = true;                                                                               \
    auto kern = k_gather_multi<SlotT, KT, LL, JJ>;                                                 \
    static SmemAllowance allowed;                                                                                \
    FG_CUDA(allowSmem(kern, smem, allowed));                                                                      \
    kern<<<(unsigned)blocks, 32 * wpb, smem, s>>>(p, in, rowsPerBlock);                            \
  }
  FG_MULTI_L(2, 3)
  FG_MULTI_L(4, 3)
  FG_MULTI_L(8, 3)
  FG_MULTI_L(8, 5)
  FG_MULTI_L(16, 3)
  FG_MULTI_L(32, 3)
#undef FG_MULTI_L
  if (!launched) {
    setLastError("multi-frequency gather: no kernel for this (lanes, columns) shape");
    return FG_ERR_UNSUPPORTED;
  }
  FG_CUDA(cudaGetLastError());
  return FG_OK;
}

static int launchGatherMulti(fg_plan *plan, const MultiIn &in, bool isFloat, cudaStream_t s) {
  const PlanDev &p = plan->d;
  if (p.nRows == 0) return FG_OK;
  ProfScope prof("k_gather_multi", s);
  countLaunch();
  if (p.slotBytes == 1)
    return isFloat ? launchMultiTyped<uint8_t, float>(p, in, s) : launchMultiTyped<uint8_t, double>(p, in, s);
  return isFloat ? launchMultiTyped<uint16_t, float>(p, in, s) : launchMultiTyped<uint16_t, double>(p, in, s);
}

struct MultiState {
  DevTerms terms[kMaxGroups];
  DevTerms *dev[kMaxGroups] = {nullptr, nullptr, nullptr};
  std::vector<void *> arrays[kMaxGroups];
  double *ke[kMaxGroups] = {nullptr, nullptr, nullptr};
  size_t keBytes[kMaxGroups] = {0, 0, 0};
  double2 *coef = nullptr;                   // [kMaxFreq][kMaxGroups] value factors, then as many lifting factors
  double2 **ptrs = nullptr;                  // device tables: value arrays, then right-hand sides
  double *values = nullptr, *rhs = nullptr;  // staging for host outputs
  size_t valuesBytes = 0, rhsBytes = 0;
};

static MultiState *multiState(fg_plan *plan) {
  if (!plan->multi) plan->multi = new MultiState();
  return (MultiState *)plan->multi;
}

}  // namespace femg

using namespace femg;

extern "C" void multiDestroy(fg_plan *plan) {
  MultiState *m = (MultiState *)plan->multi;
  if (!m) return;
  for (int g = 0; g < kMaxGroups; ++g) {
    for (void *p : m->arrays[g]) cudaFree(p);
    cudaFree(m->dev[g]);
    cudaFree(m->ke[g]);
  }
  cudaFree(m->coef);
  cudaFree(m->ptrs);
  cudaFree(m->values);
  cudaFree(m->rhs);
  delete m;
  plan->multi = nullptr;
}

namespace {

// Splits the terms by time derivative, integrates each group once (unit
// factor) and runs the fused reduction. coefOf(dts, G, coef, rcoef) fills
// the [F][G] value factors and [R][G] lifting factors. values[f] /
// rhs[r]: host or device arrays ([nnz] / [nRows]); rhs may be null.
int runGroups(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, int32_t mixed, const double *dirichlet, int F,
              double *const *values, int R, double *const *rhs, cudaStream_t s,
              const std::function<int(const int *, int, double2 *, double2 *)> &coefOf) {
  MultiState *m = multiState(plan);
  const PlanDev &p = plan->d;
  if (p.coupled) {
    setLastError("several frequencies / separate matrices: two-field plans are assembled with fg_assemble_fp64");
    return FG_ERR_UNSUPPORTED;
  }
  if (plan->accumulate) {
    setLastError("several frequencies / separate matrices: the plan accumulates; assemble one frequency at a time");
    return FG_ERR_UNSUPPORTED;
  }
  if (p.lscale) {
    setLastError("several frequencies / separate matrices: plans with linked DOFs are assembled one frequency at a time");
    return FG_ERR_UNSUPPORTED;
  }
  // groups by time derivative; the factors are applied in the reduction
  int dts[kMaxGroups], G = 0;
  fg_term_desc grp[kMaxTerms];
  for (int d = FG_DT_NONE; d <= FG_DT_2; ++d) {
    int cnt = 0;
    for (int t = 0; t < n_terms; ++t) {
      if (terms[t].dt < FG_DT_NONE || terms[t].dt > FG_DT_2) {
        setLastError("unknown time derivative");
        return FG_ERR_ARG;
      }
      if (terms[t].kind == FG_TERM_SOURCE && terms[t].dt != FG_DT_NONE) {
        setLastError("a linear term cannot carry a time derivative");
        return FG_ERR_ARG;
      }
      if (terms[t].dt == d) {
        grp[cnt] = terms[t];
        grp[cnt].dt = FG_DT_NONE;
        ++cnt;
      }
    }
    if (!cnt) continue;
    int st = uploadTerms(plan, grp, cnt, 0.0, &m->terms[G], m->arrays[G]);
    if (st) return st;
    if (!m->dev[G]) FG_CUDA(cudaMalloc(&m->dev[G], sizeof(DevTerms)));
    FG_CUDA(cudaMemcpyAsync(m->dev[G], &m->terms[G], sizeof(DevTerms), cudaMemcpyHostToDevice, s));
    dts[G++] = d;
  }
  std::vector<double2> coef((size_t)2 * kMaxFreq * kMaxGroups, make_double2(0.0, 0.0));
  int st = coefOf(dts, G, coef.data(), coef.data() + (size_t)kMaxFreq * kMaxGroups);
  if (st) return st;
  if (!m->coef) FG_CUDA(cudaMalloc(&m->coef, coef.size() * sizeof(double2)));
  FG_CUDA(cudaMemcpyAsync(m->coef, coef.data(), coef.size() * sizeof(double2), cudaMemcpyHostToDevice, s));
  const double *uD = nullptr;
  if ((st = uploadDirichlet(plan, dirichlet, &uD, s))) return st;
  // outputs: device arrays in place, host arrays through staging buffers
  std::vector<double2 *> dv(F), dr(R, nullptr);
  std::vector<char> hv(F, 0), hr(R, 0);
  size_t stageV = 0, stageR = 0;
  for (int f = 0; f < F; ++f) {
    hv[f] = !isDevicePointer(values[f]);
    stageV += hv[f];
  }
  for (int r = 0; r < R; ++r) {
    hr[r] = rhs[r] && !isDevicePointer(rhs[r]);
    stageR += hr[r];
  }
  if (stageV && (st = ensureDevice((void **)&m->values, &m->valuesBytes, stageV * p.nnz * 16))) return st;
  if (stageR && (st = ensureDevice((void **)&m->rhs, &m->rhsBytes, stageR * p.nRows * 16))) return st;
  for (int f = 0, k = 0; f < F; ++f) dv[f] = hv[f] ? (double2 *)(m->values + 2 * p.nnz * k++) : (double2 *)values[f];
  for (int r = 0, k = 0; r < R; ++r) dr[r] = hr[r] ? (double2 *)(m->rhs + 2 * p.nRows * k++) : (double2 *)rhs[r];
  const bool anyRhs = R > 0 && rhs[0];
  if (!m->ptrs) FG_CUDA(cudaMalloc(&m->ptrs, 2 * kMaxFreq * sizeof(double2 *)));
  std::vector<double2 *> table(2 * kMaxFreq, nullptr);
  std::copy(dv.begin(), dv.end(), table.begin());
  std::copy(dr.begin(), dr.end(), table.begin() + kMaxFreq);
  FG_CUDA(cudaMemcpyAsync(m->ptrs, table.data(), table.size() * sizeof(double2 *), cudaMemcpyHostToDevice, s));
  // source terms are linear terms without time derivative: group of dt 0
  const int g0 = dts[0] == FG_DT_NONE ? 0 : -1;
  double *be = nullptr;
  const bool source = g0 == 0 && m->terms[0].hasSource && anyRhs;
  if (source) {
    if ((st = ensureDevice((void **)&plan->be, &plan->beBytes, (size_t)p.E * p.n * 16))) return st;
    be = plan->be;
  }
  MultiIn in;
  std::memset(&in, 0, sizeof(in));
  in.G = G;
  in.F = F;
  for (int g = 0; g < G; ++g) {
    bool re = true, im = true;
    for (int f = 0; f < F; ++f) {
      re = re && coef[(size_t)f * G + g].y == 0.0;
      im = im && coef[(size_t)f * G + g].x == 0.0;
    }
    in.realFactor[g] = re;
    in.imagFactor[g] = im && !re;
  }
  in.R = anyRhs ? R : 0;
  in.coef = m->coef;
  in.rcoef = m->coef + (size_t)kMaxFreq * kMaxGroups;
  in.be = (const double2 *)be;
  in.uD = (const double2 *)uD;
  in.values = m->ptrs;
  in.rhs = anyRhs ? m->ptrs + kMaxFreq : nullptr;
  const size_t nn = (size_t)p.n * p.n;
  bool isFloat = false;
  if (!mixed) {
    in.lay = keFull(p.n);
    for (int g = 0; g < G; ++g) {
      const int ncomp = m->terms[g].complexKe ? 2 : 1;
      if ((st = ensureDevice((void **)&m->ke[g], &m->keBytes[g], (size_t)p.E * ncomp * nn * sizeof(double)))) return st;
      if (p.E > 0)
        if ((st = launchElementFp64(plan, m->terms[g], m->dev[g], m->ke[g], g == g0 && source ? be : nullptr, s))) return st;
      in.ke[g] = m->ke[g];
      in.stride[g] = (int64_t)(ncomp * nn);
      in.cplx[g] = ncomp == 2;
    }
  } else {
    int ncomp = 1;
    for (int g = 0; g < G; ++g) {
      if (m->terms[g].complexKe) ncomp = 2;
      for (int t = 0; t < m->terms[g].n; ++t)
        if ((m->terms[g].t[t].kind != FG_TERM_SOURCE && m->terms[g].t[t].coef.cls == kExprPoint) || m->terms[g].hasJacMod ||
            m->terms[g].tensorPoint || m->terms[g].nonSym) {
          setLastError("mixed path: bilinear coefficients must be constant per element, without Jacobian modificators");
          return FG_ERR_UNSUPPORTED;
        }
    }
    if ((st = prepareMixed(plan, ncomp, G))) return st;
    if ((st = mixedCheckTimeout(plan, false))) return st;
    if (source)
      if ((st = launchRhsFp64(plan, m->dev[0], be, s))) return st;
    if (p.E > 0) {
      const DevTerms *devs[kMaxGroups] = {m->dev[0], m->dev[1], m->dev[2]};
      uint32_t tensorMask = 0;
      for (int g = 0; g < G; ++g)
        if (m->terms[g].tensorTerm >= 0) tensorMask |= 1u << g;
      if ((st = launchMixedElement(plan, devs, G, tensorMask, s))) return st;
    }
    const float *ke = mixedKe(plan, &in.lay);
    const size_t ld = (size_t)in.lay.ld;
    for (int g = 0; g < G; ++g) {
      in.ke[g] = ke + (size_t)g * ncomp * ld;
      in.stride[g] = (int64_t)((size_t)G * ncomp * ld);
      in.cplx[g] = ncomp == 2 && m->terms[g].complexKe;
    }
    isFloat = true;
  }
  in.anyCplx = 0;
  for (int g = 0; g < G; ++g) in.anyCplx |= in.cplx[g] ? 1 : 0;
  if ((st = launchGatherMulti(plan, in, isFloat, s))) return st;
  if (mixed)
    if ((st = mixedRecordError(plan, s))) return st;
  bool anyHost = false;
  for (int f = 0; f < F; ++f)
    if (hv[f]) {
      FG_CUDA(cudaMemcpyAsync(values[f], dv[f], p.nnz * 16, cudaMemcpyDeviceToHost, s));
      anyHost = true;
    }
  for (int r = 0; r < R; ++r)
    if (hr[r]) {
      FG_CUDA(cudaMemcpyAsync(rhs[r], dr[r], p.nRows * 16, cudaMemcpyDeviceToHost, s));
      anyHost = true;
    }
  if (anyHost) {
    FG_CUDA(cudaStreamSynchronize(s));
    if (mixed) return mixedCheckTimeout(plan, true);
  }
  return FG_OK;
}

}  // namespace

extern "C" int fg_assemble_multi_freq(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, const double *omegas, int32_t n_freq,
                                      int32_t mixed, const double *dirichlet, double *csr_values, double *rhs, void *stream) {
  if (!plan) return FG_ERR_ARG;
  if (!terms || n_terms <= 0 || n_terms > kMaxTerms || !omegas || n_freq <= 0 || n_freq > kMaxFreq || !csr_values) {
    setLastError("fg_assemble_multi_freq: terms, 1..64 frequencies and csr_values are required");
    return FG_ERR_ARG;
  }
  const PlanDev &p = plan->d;
  std::vector<double *> v(n_freq), r(n_freq);
  for (int f = 0; f < n_freq; ++f) {
    v[f] = csr_values + 2 * p.nnz * (size_t)f;
    r[f] = rhs ? rhs + 2 * p.nRows * (size_t)f : nullptr;
  }
  // AFrequency factors (src/term/Assembler.cpp:283-295), on values and liftings alike
  auto coefOf = [&](const int *dts, int G, double2 *coef, double2 *rcoef) {
    for (int f = 0; f < n_freq; ++f)
      for (int g = 0; g < G; ++g) {
        const double w = omegas[f];
        const double2 c = dts[g] == FG_DT_2 ? make_double2(-w * w, 0.0) : dts[g] == FG_DT_1 ? make_double2(0.0, -w) : make_double2(1.0, 0.0);
        coef[(size_t)f * G + g] = c;
        rcoef[(size_t)f * G + g] = c;
      }
    return FG_OK;
  };
  return runGroups(plan, terms, n_terms, mixed, dirichlet, n_freq, v.data(), rhs ? n_freq : 0, r.data(), (cudaStream_t)stream, coefOf);
}

extern "C" int fg_assemble_separate(fg_plan *plan, const fg_term_desc *terms, int32_t n_terms, int32_t mixed, const double *dirichlet,
                                    double *k_values, double *c_values, double *m_values, double *rhs, void *stream) {
  if (!plan) return FG_ERR_ARG;
  if (!terms || n_terms <= 0 || n_terms > kMaxTerms) {
    setLastError("fg_assemble_separate: terms are required");
    return FG_ERR_ARG;
  }
  bool have[3] = {false, false, false};
  for (int t = 0; t < n_terms; ++t)
    if (terms[t].kind != FG_TERM_SOURCE && terms[t].dt >= FG_DT_NONE && terms[t].dt <= FG_DT_2) have[terms[t].dt] = true;
  double *out[3] = {k_values, c_values, m_values};
  for (int d = 0; d < 3; ++d) {
    if (have[d] && !out[d]) {
      setLastError("fg_assemble_separate: the formulation has a matrix whose output array is NULL");
      return FG_ERR_ARG;
    }
  }
  // value array f <- group f (the groups present, in the order K, C, M); the
  // right-hand side lifts with K alone (src/term/Assembler.cpp:306-347)
  auto coefOf = [&](const int *dts, int G, double2 *coef, double2 *rcoef) {
    for (int f = 0; f < G; ++f)
      for (int g = 0; g < G; ++g) coef[(size_t)f * G + g] = make_double2(f == g ? 1.0 : 0.0, 0.0);
    for (int g = 0; g < G; ++g) rcoef[g] = make_double2(dts[g] == FG_DT_NONE ? 1.0 : 0.0, 0.0);
    return FG_OK;
  };
  // a source without K terms still makes a group of dt 0
  bool sourceOnlyK = false;
  for (int t = 0; t < n_terms; ++t)
    if (terms[t].kind == FG_TERM_SOURCE) sourceOnlyK = !have[0];
  if (sourceOnlyK && !k_values) {
    setLastError("fg_assemble_separate: source terms need k_values (the stiffness group carries the right-hand side)");
    return FG_ERR_ARG;
  }
  std::vector<double *> vv;
  for (int d = 0; d < 3; ++d)
    if (have[d] || (d == FG_DT_NONE && sourceOnlyK)) vv.push_back(out[d]);
  double *r[1] = {rhs};
  return runGroups(plan, terms, n_terms, mixed, dirichlet, (int)vv.size(), vv.data(), rhs ? 1 : 0, r, (cudaStream_t)stream, coefOf);
}
